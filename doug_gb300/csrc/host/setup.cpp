// Host setup for the GB300 solver: control words, input formats and DOUG's
// np=1 setup (strength, aggregation, smoothed aggregation, Galerkin product,
// overlapping subdomains).  Node ids are 0-based inside this file; aggregate
// numbers stay 1-based (0 = unaggregated) because the reference's repair
// logic tests them against zero.
//
// Build with -ffp-contract=off: the coarse aggregation depends on the exact
// bits of the Galerkin product, which the reference evaluates in source order.
#include "setup.hpp"

#include <algorithm>
#include <cctype>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <chrono>
#include <cstdlib>
#include <sstream>
#include <atomic>
#include <deque>
#include <thread>

namespace dg {

// Phase timing on stderr when DG_SETUP_TIMING is set in the environment.
struct PhaseTimer {
  bool on = std::getenv("DG_SETUP_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  double total = 0;
  // seconds since the previous lap, also added to total
  double lap(const char *what) {
    auto now = std::chrono::steady_clock::now();
    const double dt = std::chrono::duration<double>(now - t).count();
    if (on) fprintf(stderr, "[setup] %-28s %8.3f s\n", what, dt);
    t = now;
    total += dt;
    return dt;
  }
};

// ---------------------------------------------------------------------------
// control words (controls.F90:159-246, DOUG_utils.F90:629-1150)
// ---------------------------------------------------------------------------
static std::string first10_noblank(const std::string &s) {
  std::string b;
  for (size_t i = 0; i < s.size() && i < 10; i++)
    if (s[i] != ' ') b.push_back(s[i]);
  return b;
}

bool parse_i10(const std::string &s, int &out) {
  std::string b = first10_noblank(s);
  if (b.empty()) { out = 0; return true; }
  char *end = nullptr;
  long v = strtol(b.c_str(), &end, 10);
  if (*end) return false;
  out = (int)v;
  return true;
}

bool parse_f10_5(const std::string &s, double &out) {
  std::string b = first10_noblank(s);
  if (b.empty()) { out = 0.0; return true; }
  size_t p = 0;
  bool neg = false;
  if (b[p] == '+' || b[p] == '-') { neg = b[p] == '-'; p++; }
  std::string mant;
  bool dot = false;
  int ndig = 0;
  while (p < b.size() && (isdigit((unsigned char)b[p]) || b[p] == '.')) {
    if (b[p] == '.') { if (dot) return false; dot = true; } else ndig++;
    mant.push_back(b[p++]);
  }
  if (ndig == 0) return false;
  int expo = 0;
  if (p < b.size()) {
    char e = b[p];
    if (e == 'e' || e == 'E' || e == 'd' || e == 'D') p++;
    if (p >= b.size()) return false;
    char *end = nullptr;
    long ev = strtol(b.c_str() + p, &end, 10);
    if (*end || end == b.c_str() + p) return false;
    expo = (int)ev;
  }
  // F10.5 without a decimal point: five implied decimals
  std::string num = mant + "e" + std::to_string(dot ? expo : expo - 5);
  double v = strtod(num.c_str(), nullptr);
  out = neg ? -v : v;
  return true;
}

bool parse_l1(const std::string &s, bool &out) {
  if (s.empty()) return false;
  char c = s[0];
  if (c == '.' && s.size() > 1) c = s[1];
  if (c == 'T' || c == 't') { out = true; return true; }
  if (c == 'F' || c == 'f') { out = false; return true; }
  return false;
}

bool ctl_apply(Controls &c, const std::string &w1, const std::string &w2, std::string &err) {
  // the first occurrence of a word wins; repeats only warn in the reference
  auto I = [&](const char *nm, int &f) -> int {
    if (w1 != nm) return 0;
    if (f == -1 && !parse_i10(w2, f)) { err = "bad integer for " + w1 + ": '" + w2 + "'"; return -1; }
    return 1;
  };
  auto R = [&](const char *nm, double &f) -> int {
    if (w1 != nm) return 0;
    if (f == -1.0 && !parse_f10_5(w2, f)) { err = "bad real for " + w1 + ": '" + w2 + "'"; return -1; }
    return 1;
  };
  auto L = [&](const char *nm, bool &f) -> int {
    if (w1 != nm) return 0;
    if (!parse_l1(w2, f)) { err = "bad logical for " + w1 + ": '" + w2 + "'"; return -1; }
    return 1;
  };
  auto S = [&](const char *nm, std::string &f) -> int {
    if (w1 != nm) return 0;
    if (f.empty()) f = w2;
    return 1;
  };
  int r = 0;
#define TRY(x) if ((r = (x)) != 0) return r > 0;
  TRY(I("solver", c.solver)) TRY(I("method", c.method)) TRY(I("fine_method", c.fine_method))
  TRY(I("num_iters", c.num_iters)) TRY(I("grid_size", c.grid_size))
  TRY(I("coarse_method", c.coarse_method)) TRY(I("num_subdomains", c.num_subdomains))
  TRY(I("levels", c.levels)) TRY(I("overlap", c.overlap)) TRY(I("smoothers", c.smoothers))
  TRY(I("input_type", c.input_type)) TRY(I("matrix_type", c.matrix_type))
  TRY(I("initial_guess", c.initial_guess)) TRY(I("number_of_blocks", c.number_of_blocks))
  TRY(I("radius1", c.radius1)) TRY(I("radius2", c.radius2)) TRY(I("minasize1", c.minasize1))
  TRY(I("minasize2", c.minasize2)) TRY(I("maxasize1", c.maxasize1)) TRY(I("maxasize2", c.maxasize2))
  TRY(I("debug", c.debug)) TRY(I("verbose", c.verbose)) TRY(I("plotting", c.plotting))
  TRY(R("strong1", c.strong1)) TRY(R("strong2", c.strong2)) TRY(R("solve_tolerance", c.solve_tolerance))
  TRY(I("solve_maxiters", c.solve_maxiters))
  TRY(L("symmstruct", c.symmstruct)) TRY(L("symmnumeric", c.symmnumeric))
  TRY(I("interpolation_type", c.interpolation_type))
  TRY(S("assembled_mtx_file", c.assembled_mtx_file)) TRY(I("assembled_mtx_format", c.assembled_mtx_format))
  TRY(S("assembled_rhs_file", c.assembled_rhs_file)) TRY(I("assembled_rhs_format", c.assembled_rhs_format))
  TRY(S("info_file", c.info_file)) TRY(S("elemmat_rhs_file", c.elemmat_rhs_file))
  TRY(S("freedom_lists_file", c.freedom_lists_file)) TRY(S("coords_file", c.coords_file))
  TRY(S("freemap_file", c.freemap_file))
  TRY(S("solution_file", c.solution_file)) TRY(I("solution_format", c.solution_format))
  TRY(I("start_vec_type", c.start_vec_type))
  TRY(I("maxcie", c.maxcie)) TRY(I("maxnd", c.maxnd)) TRY(I("cutbal", c.cutbal))
  TRY(I("center_type", c.center_type)) TRY(L("hanging_nodes", c.hanging_nodes))
#undef TRY
  if (w1 == "executable") {  // not a reference word: doug_aggr (aggr) or doug_geom (geom)
    if (w2 != "aggr" && w2 != "geom") { err = "executable must be aggr or geom: '" + w2 + "'"; return false; }
    if (c.executable == -1) c.executable = w2 == "geom" ? 1 : 0;
    return true;
  }
  return true;  // unknown words are ignored
}

static std::string getword(const std::string &line, int num) {
  // words are separated by blanks only (DOUG_utils.F90:1518-1544)
  int n = (int)line.size();
  while (n > 0 && (line[n - 1] == ' ' || line[n - 1] == '\r')) n--;
  int j = 0, k = 0;
  for (int i = 1; i <= num; i++) {
    while (j < n && line[j] == ' ') j++;
    if (j >= n) return "";
    k = j;
    while (j < n && line[j] != ' ') j++;
  }
  return line.substr(k, j - k);
}

bool ctl_parse_text(Controls &c, const std::string &text, std::string &err) {
  std::istringstream is(text);
  std::string line;
  while (std::getline(is, line)) {
    if (line.size() > 300) line.resize(300);
    while (!line.empty() && (line.back() == ' ' || line.back() == '\r')) line.pop_back();
    if (line.empty() || line[0] == '#') continue;
    std::string w1 = getword(line, 1), w2 = getword(line, 2);
    for (auto &ch : w1)
      if (ch >= 'A' && ch <= 'Z') ch = (char)(ch + 32);
    if (!ctl_apply(c, w1, w2, err)) return false;
  }
  return true;
}

void ctl_finish(Controls &c) {
  if (c.solve_maxiters == -1) c.solve_maxiters = 100;
  if (c.executable == 1) c.fine_method = 1;
}

// ---------------------------------------------------------------------------
// formats
// ---------------------------------------------------------------------------
static bool slurp(const std::string &path, std::vector<unsigned char> &buf) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long L = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf.resize((size_t)L + 1);
  size_t got = L > 0 ? fread(buf.data(), 1, (size_t)L, f) : 0;
  fclose(f);
  if ((long)got != L) return false;
  buf[(size_t)L] = 0;
  buf.resize((size_t)L);
  return true;
}
static uint32_t rd_be32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static uint32_t rd_le32(const unsigned char *p) {
  return ((uint32_t)p[3] << 24) | ((uint32_t)p[2] << 16) | ((uint32_t)p[1] << 8) | p[0];
}
static double rd_bed(const unsigned char *p) {
  uint64_t u = ((uint64_t)rd_be32(p) << 32) | rd_be32(p + 4);
  double d;
  memcpy(&d, &u, 8);
  return d;
}
static double rd_led(const unsigned char *p) {
  uint64_t u = ((uint64_t)rd_le32(p + 4) << 32) | rd_le32(p);
  double d;
  memcpy(&d, &u, 8);
  return d;
}

// One Fortran unformatted sequential record (little-endian 4-byte markers;
// negative markers are gfortran sub-records of a long record).
static bool fortran_record(const std::vector<unsigned char> &b, size_t &pos,
                           std::vector<unsigned char> &rec) {
  rec.clear();
  for (;;) {
    if (pos + 4 > b.size()) return false;
    int32_t m = (int32_t)rd_le32(&b[pos]);
    size_t len = (size_t)(m < 0 ? -(int64_t)m : m);
    if (pos + 8 + len > b.size()) return false;
    rec.insert(rec.end(), b.begin() + (long)pos + 4, b.begin() + (long)(pos + 4 + len));
    pos += 8 + len;
    if (m >= 0) return true;
  }
}

static void skip_sep(const char *&p) {
  while (*p == ',' || isspace((unsigned char)*p)) p++;
}
static bool next_double(const char *&p, double &v) {
  skip_sep(p);
  char tmp[64];
  int k = 0;
  while (*p && !isspace((unsigned char)*p) && *p != ',' && k < 63) {
    char ch = *p++;
    tmp[k++] = (ch == 'd' || ch == 'D') ? 'e' : ch;
  }
  tmp[k] = 0;
  char *end = nullptr;
  v = strtod(tmp, &end);
  return k > 0 && *end == 0;
}
static bool next_int(const char *&p, long &v) {
  skip_sep(p);
  char *end = nullptr;
  v = strtol(p, &end, 10);
  if (end == p) return false;
  p = end;
  return true;
}

bool read_assembled(const std::string &path, int format, int &n, std::vector<int> &ii,
                    std::vector<int> &jj, std::vector<double> &vv, std::string &err) {
  std::vector<unsigned char> b;
  if (!slurp(path, b)) { err = "Unable to open assembled file: " + path; return false; }
  long N = 0, NNZ = 0;
  if (format == 0 || format < 0) {
    b.push_back(0);
    const char *p = (const char *)b.data();
    if (!next_int(p, N) || !next_int(p, NNZ)) { err = "File " + path + " too short!"; return false; }
    long cnt = std::max(N, NNZ);
    ii.resize(cnt); jj.resize(cnt); vv.resize(cnt);
    for (long k = 0; k < cnt; k++) {
      long a, c;
      double v;
      if (!next_int(p, a) || !next_int(p, c) || !next_double(p, v)) {
        err = "[ReadInSparseAssembledBulk_TextBinary] File too short! " + path;
        return false;
      }
      ii[k] = (int)a; jj[k] = (int)c; vv[k] = v;
    }
  } else if (format == 1) {
    size_t pos = 0;
    std::vector<unsigned char> rec;
    if (!fortran_record(b, pos, rec) || rec.size() < 8) { err = "File " + path + " too short!"; return false; }
    N = (int32_t)rd_le32(&rec[0]); NNZ = (int32_t)rd_le32(&rec[4]);
    long cnt = std::max(N, NNZ);
    if (!fortran_record(b, pos, rec) || (long)rec.size() < 16 * cnt) { err = "File " + path + " too short!"; return false; }
    ii.resize(cnt); jj.resize(cnt); vv.resize(cnt);
    for (long k = 0; k < cnt; k++) {
      ii[k] = (int32_t)rd_le32(&rec[16 * k]);
      jj[k] = (int32_t)rd_le32(&rec[16 * k + 4]);
      vv[k] = rd_led(&rec[16 * k + 8]);
    }
  } else if (format == 2) {
    if (b.size() < 8) { err = "File " + path + " too short!"; return false; }
    N = (int32_t)rd_be32(&b[0]); NNZ = (int32_t)rd_be32(&b[4]);
    long cnt = std::max(N, NNZ);
    if ((long)b.size() < 8 + 16 * cnt) { err = "File " + path + " too short!"; return false; }
    ii.resize(cnt); jj.resize(cnt); vv.resize(cnt);
    for (long k = 0; k < cnt; k++) {
      ii[k] = (int32_t)rd_be32(&b[8 + 16 * k]);
      jj[k] = (int32_t)rd_be32(&b[8 + 16 * k + 4]);
      vv[k] = rd_bed(&b[8 + 16 * k + 8]);
    }
  } else {
    err = "[ReadInSparseAssembledHeader] Data format not recognized";
    return false;
  }
  // header swap when n > nnz (SpMtx_class.F90:421-425)
  n = (int)std::min(N, NNZ);
  if (N <= NNZ) n = (int)N;
  return true;
}

bool read_vector(const std::string &path, int format, int n, std::vector<double> &x,
                 std::string &err) {
  std::vector<unsigned char> b;
  if (!slurp(path, b)) { err = "Unable to open vector file: " + path; return false; }
  x.assign(n, 0.0);
  if (format == 0) {
    b.push_back(0);
    const char *p = (const char *)b.data();
    long m;
    if (!next_int(p, m) || m != n) {
      err = "[Vect_ReadFromFile_Text] : Number of vector elements in file is not as expected.";
      return false;
    }
    for (int k = 0; k < n; k++)
      if (!next_double(p, x[k])) { err = "[Vect_ReadFromFile_Text] : End of file reached to early."; return false; }
  } else if (format == 1 || format < 0) {
    size_t pos = 0;
    std::vector<unsigned char> rec;
    if (!fortran_record(b, pos, rec) || (long)rec.size() < 8L * n) {
      err = "[Vect_ReadFromFile_Binary] : End of file reached to early.";
      return false;
    }
    for (int k = 0; k < n; k++) x[k] = rd_led(&rec[8 * (size_t)k]);
  } else if (format == 2) {
    if (b.size() < 4 || (int)rd_be32(&b[0]) != n || b.size() < 4 + 8 * (size_t)n) {
      err = "[Vect_ReadFromFile_XDR] : Number of vector elements in file is not as expected.";
      return false;
    }
    for (int k = 0; k < n; k++) x[k] = rd_bed(&b[4 + 8 * (size_t)k]);
  } else {
    err = "[Vect_ReadFromFile] Data format not recognized";
    return false;
  }
  return true;
}

void structured_laplace(int n, int &nrows, std::vector<int> &ii, std::vector<int> &jj, std::vector<double> &vv,
                        std::vector<double> &b) {
  if (n < 1) n = 100;
  nrows = n * n;
  ii.clear(); jj.clear(); vv.clear();
  auto put = [&](int r, int c, double v) { ii.push_back(r); jj.push_back(c); vv.push_back(v); };
  for (int ri = 1; ri <= n; ri++)
    for (int ci = 1; ci <= n; ci++) {
      const int mri = (ri - 1) * n + ci;
      put(mri, mri, 4.0);
      if (ci > 1) put(mri, mri - 1, -1.0);
      if (ci < n) put(mri, mri + 1, -1.0);
      if (ri > 1) put(mri, mri - n, -1.0);
      if (ri < n) put(mri, mri + n, -1.0);
    }
  b.assign((size_t)nrows, -1.0);
}

bool read_elemental(const std::string &info, const std::string &freelists, const std::string &elemmat,
                    int number_of_blocks, ElementMesh &M, std::string &err) {
  std::vector<unsigned char> b, rec;
  size_t pos = 0;
  // info_file: one record nell, ngf, nsd, mfrelt, nnode (Mesh.F90:305-307)
  if (!slurp(info, b)) { err = "Unable to open info file: " + info; return false; }
  if (!fortran_record(b, pos, rec) || rec.size() < 20) { err = "info file too short: " + info; return false; }
  M.nell = (int32_t)rd_le32(&rec[0]);
  M.ngf = (int32_t)rd_le32(&rec[4]);
  M.nsd = (int32_t)rd_le32(&rec[8]);
  M.mfrelt = (int32_t)rd_le32(&rec[12]);
  M.nnode = (int32_t)rd_le32(&rec[16]);
  if (M.nell <= 0 || M.ngf <= 0 || M.mfrelt <= 0) { err = "info file: bad mesh sizes in " + info; return false; }
  // freedom lists: per element one record nfrelt, mhead(1:nfrelt) (Mesh.F90:452-460)
  if (!slurp(freelists, b)) { err = "Unable to open freedom lists file: " + freelists; return false; }
  pos = 0;
  M.eptr.assign(1, 0);
  M.efree.clear();
  for (int e = 0; e < M.nell; e++) {
    if (!fortran_record(b, pos, rec) || rec.size() < 4) { err = "freedom lists file too short: " + freelists; return false; }
    const int nf = (int32_t)rd_le32(&rec[0]);
    if (nf < 0 || nf > M.mfrelt || rec.size() < 4 + 4 * (size_t)nf) {
      err = "freedom lists file: bad element record in " + freelists;
      return false;
    }
    for (int i = 0; i < nf; i++) M.efree.push_back((int32_t)rd_le32(&rec[4 + 4 * (size_t)i]));
    M.eptr.push_back((int)M.efree.size());
  }
  if (number_of_blocks > 1) M.ngf = *std::max_element(M.efree.begin(), M.efree.end());  // Mesh.F90:313-319
  // element matrices and right-hand sides: per element nfrelt records (one per
  // column) and one record of the right-hand side (ElemMtxs_distribute.F90:572-575)
  if (!slurp(elemmat, b)) { err = "Unable to open element matrix file: " + elemmat; return false; }
  pos = 0;
  M.emat_off.assign(1, 0);
  M.emat.clear();
  M.erhs.clear();
  for (int e = 0; e < M.nell; e++) {
    const int nf = M.eptr[(size_t)e + 1] - M.eptr[(size_t)e];
    for (int j = 0; j < nf; j++) {
      if (!fortran_record(b, pos, rec) || rec.size() < 8 * (size_t)nf) {
        err = "element matrix file too short: " + elemmat;
        return false;
      }
      for (int k = 0; k < nf; k++) M.emat.push_back(rd_led(&rec[8 * (size_t)k]));
    }
    if (!fortran_record(b, pos, rec) || rec.size() < 8 * (size_t)nf) {
      err = "element matrix file too short: " + elemmat;
      return false;
    }
    for (int k = 0; k < nf; k++) M.erhs.push_back(rd_led(&rec[8 * (size_t)k]));
    M.emat_off.push_back((int64_t)M.emat.size());
  }
  return check_elements(M, err);
}

bool read_geometry(const std::string &coords_path, const std::string &freemap_path, int nsd, int nnode, int ngf,
                   NodeGeometry &G, std::string &err) {
  if (nsd < 1 || nsd > 3 || nnode < 1 || ngf < 1) { err = "node geometry: bad sizes in the info file"; return false; }
  std::vector<unsigned char> b, rec;
  size_t pos = 0;
  if (!slurp(coords_path, b) || !fortran_record(b, pos, rec) || rec.size() < (size_t)8 * nsd * nnode) {
    err = "cannot read node coordinates from " + coords_path;
    return false;
  }
  G.nsd = nsd;
  G.nnode = nnode;
  G.coords.resize((size_t)nsd * nnode);
  for (size_t q = 0; q < G.coords.size(); q++) G.coords[q] = rd_led(rec.data() + 8 * q);
  pos = 0;
  if (!slurp(freemap_path, b) || !fortran_record(b, pos, rec) || rec.size() < (size_t)4 * ngf) {
    err = "cannot read the freedom map from " + freemap_path;
    return false;
  }
  G.freemap.resize((size_t)ngf);
  for (int f = 0; f < ngf; f++) {
    G.freemap[(size_t)f] = (int32_t)rd_le32(rec.data() + 4 * f);
    if (G.freemap[(size_t)f] < 1 || G.freemap[(size_t)f] > nnode) {
      err = "freemap: freedom " + std::to_string(f + 1) + " maps to node " + std::to_string(G.freemap[(size_t)f]);
      return false;
    }
  }
  return true;
}

bool check_elements(const ElementMesh &M, std::string &err) {
  if (M.nell <= 0 || M.ngf <= 0 || (int)M.eptr.size() != M.nell + 1 || M.eptr[0] != 0) {
    err = "elements: bad element count or freedom list offsets";
    return false;
  }
  for (int e = 0; e < M.nell; e++)
    if (M.eptr[(size_t)e + 1] < M.eptr[(size_t)e]) { err = "elements: freedom list offsets decrease"; return false; }
  if ((int64_t)M.efree.size() != M.eptr.back() || (int64_t)M.erhs.size() != M.eptr.back() ||
      (int)M.emat_off.size() != M.nell + 1 || (int64_t)M.emat.size() != M.emat_off.back()) {
    err = "elements: array sizes do not match the freedom lists";
    return false;
  }
  for (int e = 0; e < M.nell; e++) {
    const int64_t nf = M.eptr[(size_t)e + 1] - M.eptr[(size_t)e];
    if (M.emat_off[(size_t)e + 1] - M.emat_off[(size_t)e] != nf * nf) {
      err = "elements: element matrix size does not match its freedom count";
      return false;
    }
  }
  for (int g : M.efree)
    if (g < 1 || g > M.ngf) { err = "[Mesh_readFileFreelists] - freedom index out of range"; return false; }
  return true;
}

void assemble_elements(const ElementMesh &M, int &n, std::vector<int> &ii, std::vector<int> &jj,
                       std::vector<double> &vv, std::vector<double> &b, std::vector<int> &lg_fmap) {
  // local freedoms: used freedoms in increasing global order (Mesh.F90:1131-1191, one partition)
  std::vector<int> gl((size_t)M.ngf + 1, 0);
  for (int g : M.efree) gl[(size_t)g] = 1;
  lg_fmap.clear();
  for (int g = 1; g <= M.ngf; g++)
    if (gl[(size_t)g]) { lg_fmap.push_back(g); gl[(size_t)g] = (int)lg_fmap.size(); }
  n = (int)lg_fmap.size();
  // Every row is assembled on its own (rows split among host threads): its
  // element occurrences are visited in element order, and for each column
  // the non-zero contributions are summed in that order (element order, then
  // row i, column j within the element), the entries sorted by column.  This
  // is the serial element loop's arithmetic, row by row.
  std::vector<int64_t> occ_ptr((size_t)n + 1, 0);
  for (int64_t q = 0; q < (int64_t)M.efree.size(); q++) occ_ptr[(size_t)gl[(size_t)M.efree[(size_t)q]]]++;
  for (int r = 0; r < n; r++) occ_ptr[(size_t)r + 1] += occ_ptr[(size_t)r];
  std::vector<int> occ_e(M.efree.size()), occ_i(M.efree.size());
  {
    std::vector<int64_t> fill(occ_ptr.begin(), occ_ptr.end() - 1);
    for (int e = 0; e < M.nell; e++)
      for (int i = M.eptr[(size_t)e]; i < M.eptr[(size_t)e + 1]; i++) {
        const int li = gl[(size_t)M.efree[(size_t)i]] - 1;
        occ_e[(size_t)fill[(size_t)li]] = e;
        occ_i[(size_t)fill[(size_t)li]++] = i - M.eptr[(size_t)e];
      }
  }
  const int nth = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  std::vector<std::vector<int>> tcol((size_t)nth);
  std::vector<std::vector<double>> tval((size_t)nth);
  std::vector<int64_t> rcount((size_t)n, 0);
  b.assign((size_t)n, 0.0);
  auto work = [&](int t) {
    const int r0 = (int)((int64_t)n * t / nth), r1 = (int)((int64_t)n * (t + 1) / nth);
    std::vector<std::pair<int, double>> ent;
    for (int r = r0; r < r1; r++) {
      ent.clear();
      double br = 0.0;
      for (int64_t q = occ_ptr[(size_t)r]; q < occ_ptr[(size_t)r + 1]; q++) {
        const int e = occ_e[(size_t)q], i = occ_i[(size_t)q];
        const int e0 = M.eptr[(size_t)e], nf = M.eptr[(size_t)e + 1] - e0;
        const double *Ae = &M.emat[(size_t)M.emat_off[(size_t)e]];
        for (int j = 0; j < nf; j++) {
          const double a = Ae[(size_t)j * nf + i];
          if (a != 0.0) ent.push_back({gl[(size_t)M.efree[(size_t)(e0 + j)]] - 1, a});
        }
        br += M.erhs[(size_t)(e0 + i)];
      }
      b[(size_t)r] = br;
      std::stable_sort(ent.begin(), ent.end(),
                       [](const std::pair<int, double> &x, const std::pair<int, double> &y) { return x.first < y.first; });
      int64_t cnt = 0;
      for (size_t q = 0; q < ent.size();) {
        double sv = 0.0;
        size_t q1 = q;
        for (; q1 < ent.size() && ent[q1].first == ent[q].first; q1++) sv += ent[q1].second;
        tcol[(size_t)t].push_back(ent[q].first);
        tval[(size_t)t].push_back(sv);
        cnt++;
        q = q1;
      }
      rcount[(size_t)r] = cnt;
    }
  };
  {
    std::vector<std::thread> pool;
    for (int t = 1; t < nth; t++) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
  }
  std::vector<int64_t> rp((size_t)n + 1, 0);
  for (int r = 0; r < n; r++) rp[(size_t)r + 1] = rp[(size_t)r] + rcount[(size_t)r];
  std::vector<int> col;
  std::vector<double> val;
  col.reserve((size_t)rp[(size_t)n]);
  val.reserve((size_t)rp[(size_t)n]);
  for (int t = 0; t < nth; t++) {
    col.insert(col.end(), tcol[(size_t)t].begin(), tcol[(size_t)t].end());
    val.insert(val.end(), tval[(size_t)t].begin(), tval[(size_t)t].end());
    std::vector<int>().swap(tcol[(size_t)t]);
    std::vector<double>().swap(tval[(size_t)t]);
  }
  // COO in row order with the reference's flipped indices (ElemMtxs_assemble.F90:262-266)
  ii.resize(col.size());
  jj.resize(col.size());
  vv = val;
  for (int r = 0; r < n; r++)
    for (int64_t q = rp[(size_t)r]; q < rp[(size_t)r + 1]; q++) {
      ii[(size_t)q] = col[(size_t)q] + 1;
      jj[(size_t)q] = r + 1;
    }
}

bool write_solution(const std::string &path, int format, const double *x, int n, std::string &err) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) { err = "cannot open " + path; return false; }
  if (format == 0) {
    fprintf(f, "%6d\n", n);
    for (int k = 0; k < n; k++) fprintf(f, "%21.14E\n", x[k]);
  } else if (format == 1) {
    uint32_t m = (uint32_t)(8 * n);
    fwrite(&m, 4, 1, f);
    fwrite(x, 8, (size_t)n, f);
    fwrite(&m, 4, 1, f);
  } else if (format == 2) {
    unsigned char hb[4] = {(unsigned char)(n >> 24), (unsigned char)(n >> 16),
                           (unsigned char)(n >> 8), (unsigned char)n};
    fwrite(hb, 1, 4, f);
    for (int k = 0; k < n; k++) {
      uint64_t u;
      memcpy(&u, &x[k], 8);
      unsigned char o[8];
      for (int q = 0; q < 8; q++) o[q] = (unsigned char)(u >> (56 - 8 * q));
      fwrite(o, 1, 8, f);
    }
  } else {
    fclose(f);
    err = "Solution format is not valid";
    return false;
  }
  fclose(f);
  return true;
}

// ---------------------------------------------------------------------------
// sparse helpers with DOUG's ordering semantics
// ---------------------------------------------------------------------------
// stable bucketing by row (SpMtx_arrange ROWS, sort=.false.)
static Csr rows_of(const Coo &m) {
  Csr c;
  c.nrows = m.nrows; c.ncols = m.ncols;
  c.ptr.assign((size_t)m.nrows + 1, 0);
  for (size_t k = 0; k < m.size(); k++) c.ptr[(size_t)m.i[k] + 1]++;
  for (int r = 0; r < m.nrows; r++) c.ptr[(size_t)r + 1] += c.ptr[(size_t)r];
  c.col.resize(m.size()); c.val.resize(m.size());
  std::vector<int64_t> fill(c.ptr.begin(), c.ptr.end() - 1);
  for (size_t k = 0; k < m.size(); k++) {
    int64_t d = fill[(size_t)m.i[k]]++;
    c.col[(size_t)d] = m.j[k]; c.val[(size_t)d] = m.v[k];
  }
  return c;
}
// stable bucketing by column: a "row view" of the transpose
static Csr cols_of(const Coo &m) {
  Coo t;
  t.nrows = m.ncols; t.ncols = m.nrows;
  t.i = m.j; t.j = m.i; t.v = m.v;
  return rows_of(t);
}
static Coo coo_of(const Csr &c) {
  Coo m;
  m.nrows = c.nrows; m.ncols = c.ncols;
  m.i.resize(c.col.size()); m.j = c.col; m.v = c.val;
  for (int r = 0; r < c.nrows; r++)
    for (int64_t k = c.ptr[(size_t)r]; k < c.ptr[(size_t)r + 1]; k++) m.i[(size_t)k] = r;
  return m;
}

// Rows [0, n) in contiguous blocks on up to 16 host threads (one block
// below 4096 rows): fn(lo, hi) must only write rows lo..hi-1, so the result
// is the same for any thread count.
template <class F>
static void parallel_rows(int n, F fn) {
  const int nt = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  if (n < 4096 || nt < 2) {
    fn(0, n);
    return;
  }
  const int chunk = (n + nt - 1) / nt;
  std::vector<std::thread> th;
  for (int t = 1; t < nt; t++) {
    const int lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo < hi) th.emplace_back([&fn, lo, hi] { fn(lo, hi); });
  }
  fn(0, std::min(n, chunk));
  for (auto &x : th) x.join();
}

// SpMtx_AB (SpMtx_op_AB.f90:39-200): A given as a row view, B as a row view
// (of B, or of B^T).  Output row i lists its columns in first-touch order;
// each value is summed in the order A's row entries, then B's row entries,
// are visited; explicit zeros are kept.  Rows are independent: counted and
// filled in parallel blocks.
static Csr spgemm_first_touch(const Csr &A, const Csr &B) {
  Csr C;
  C.nrows = A.nrows; C.ncols = B.ncols;
  C.ptr.assign((size_t)A.nrows + 1, 0);
  parallel_rows(A.nrows, [&](int lo, int hi) {
    std::vector<int> mark((size_t)B.ncols, -1);
    for (int i = lo; i < hi; i++) {
      int64_t cnt = 0;
      for (int64_t k = A.ptr[(size_t)i]; k < A.ptr[(size_t)i + 1]; k++) {
        int kk = A.col[(size_t)k];
        for (int64_t j = B.ptr[(size_t)kk]; j < B.ptr[(size_t)kk + 1]; j++) {
          int jj = B.col[(size_t)j];
          if (mark[(size_t)jj] != i) { mark[(size_t)jj] = i; cnt++; }
        }
      }
      C.ptr[(size_t)i + 1] = cnt;
    }
  });
  for (int i = 0; i < A.nrows; i++) C.ptr[(size_t)i + 1] += C.ptr[(size_t)i];
  C.col.resize((size_t)C.ptr.back());
  C.val.resize((size_t)C.ptr.back());
  parallel_rows(A.nrows, [&](int lo, int hi) {
    std::vector<int> mark((size_t)B.ncols, -1);
    std::vector<int64_t> pos((size_t)B.ncols, 0);
    for (int i = lo; i < hi; i++) {
      int64_t base = C.ptr[(size_t)i], nind = 0;
      for (int64_t k = A.ptr[(size_t)i]; k < A.ptr[(size_t)i + 1]; k++) {
        int kk = A.col[(size_t)k];
        double av = A.val[(size_t)k];
        for (int64_t j = B.ptr[(size_t)kk]; j < B.ptr[(size_t)kk + 1]; j++) {
          int jj = B.col[(size_t)j];
          double prod = av * B.val[(size_t)j];
          if (mark[(size_t)jj] != i) {
            mark[(size_t)jj] = i;
            pos[(size_t)jj] = base + nind;
            C.col[(size_t)(base + nind)] = jj;
            C.val[(size_t)(base + nind)] = prod;
            nind++;
          } else {
            C.val[(size_t)pos[(size_t)jj]] = C.val[(size_t)pos[(size_t)jj]] + prod;
          }
        }
      }
    }
  });
  return C;
}

// ---------------------------------------------------------------------------
// strength of connection and aggregation
// ---------------------------------------------------------------------------
struct ScaledMatrix {
  Csr M;                     // DOUG row order
  std::vector<double> diag;  // unscaled diagonal (last diagonal entry of each row)
  bool symmetric = false;    // symmstruct && symmnumeric
  std::vector<char> strong;  // per entry
  std::vector<int64_t> sptr; // sorted strong adjacency
  std::vector<int> scol;
};

// SpMtx_scale (SpMtx_arrangement.F90:298-346) applied entrywise.
static void scale_rows(ScaledMatrix &S) {
  Csr &M = S.M;
  S.diag.assign((size_t)std::max(M.nrows, M.ncols), 0.0);
  // diag(indi)=val for every diagonal entry, in entry order
  for (int r = 0; r < M.nrows; r++)
    for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++)
      if (M.col[(size_t)k] == r) S.diag[(size_t)r] = M.val[(size_t)k];
  std::vector<double> s(S.diag.size());
  if (S.symmetric) {
    for (size_t q = 0; q < s.size(); q++) s[q] = std::sqrt(std::fabs(S.diag[q]));
    for (int r = 0; r < M.nrows; r++)
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++) {
        double v = M.val[(size_t)k] / s[(size_t)r];
        M.val[(size_t)k] = v / s[(size_t)M.col[(size_t)k]];
      }
  } else {
    for (size_t q = 0; q < s.size(); q++) s[q] = std::fabs(S.diag[q]);
    for (int r = 0; r < M.nrows; r++)
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++)
        M.val[(size_t)k] = M.val[(size_t)k] / s[(size_t)r];
  }
}

// SpMtx_unscale (SpMtx_arrangement.F90:350-388).
static void unscale_rows(ScaledMatrix &S) {
  Csr &M = S.M;
  std::vector<double> s(S.diag.size());
  if (S.symmetric) {
    for (size_t q = 0; q < s.size(); q++) s[q] = std::sqrt(std::fabs(S.diag[q]));
    for (int r = 0; r < M.nrows; r++)
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++) {
        double v = M.val[(size_t)k] * s[(size_t)r];
        M.val[(size_t)k] = v * s[(size_t)M.col[(size_t)k]];
      }
  } else {
    for (size_t q = 0; q < s.size(); q++) s[q] = std::fabs(S.diag[q]);
    for (int r = 0; r < M.nrows; r++)
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++)
        M.val[(size_t)k] = M.val[(size_t)k] * s[(size_t)r];
  }
}

// SpMtx_find_strong (SpMtx_aggregation.F90:829-900) + sorted strong
// adjacency SpMtx_build_refs_symm(sortdown) (SpMtx_arrangement.F90:461-568).
static void find_strong(ScaledMatrix &S, double alpha) {
  const Csr &M = S.M;
  const int n = M.nrows;
  S.strong.assign(M.col.size(), 0);
  S.sptr.assign((size_t)n + 1, 0);
  parallel_rows(n, [&](int lo, int hi) {
    for (int r = lo; r < hi; r++) {
      double mx = (double)(-1.0e15f);
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++)
        if (M.col[(size_t)k] != r) mx = std::max(mx, std::fabs(M.val[(size_t)k]));
      mx = mx * alpha;
      int64_t cnt = 0;
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++) {
        if (M.col[(size_t)k] != r) S.strong[(size_t)k] = std::fabs(M.val[(size_t)k]) > mx;
        else S.strong[(size_t)k] = S.diag[(size_t)r] > mx;  // unscaled diagonal
        if (S.strong[(size_t)k] && M.col[(size_t)k] != r && M.col[(size_t)k] < n) cnt++;
      }
      S.sptr[(size_t)r + 1] = cnt;
    }
  });
  for (int r = 0; r < n; r++) S.sptr[(size_t)r + 1] += S.sptr[(size_t)r];
  // strong off-diagonal neighbours of each row, by |value| descending; equal
  // magnitudes keep their entry order (stable)
  S.scol.assign((size_t)S.sptr.back(), 0);
  parallel_rows(n, [&](int lo, int hi) {
    std::vector<int64_t> tmp;
    for (int r = lo; r < hi; r++) {
      tmp.clear();
      for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++)
        if (S.strong[(size_t)k] && M.col[(size_t)k] != r && M.col[(size_t)k] < n) tmp.push_back(k);
      std::stable_sort(tmp.begin(), tmp.end(), [&](int64_t a, int64_t b) {
        return std::fabs(M.val[(size_t)a]) > std::fabs(M.val[(size_t)b]);
      });
      int64_t q = S.sptr[(size_t)r];
      for (int64_t k : tmp) S.scol[(size_t)q++] = M.col[(size_t)k];
    }
  });
}

// Persistent state of the reference's aggregation (SAVE variables):
// allmind (Aggregate_mod.F90:348) and beta (SpMtx_aggregation.F90:81).
struct AggState {
  int allmind = INT_MAX;
  double beta = 1.0e-5;
};

static constexpr int kAggregated = INT_MAX;       // D_AGGREGATED
static constexpr int kPending = INT_MAX / 2;      // D_PENDING

class Colourer {  // lets_colour / can_add_roundlayer (Aggregate_mod.F90:287-497)
 public:
  Colourer(const ScaledMatrix &S, int r, int maxasize, std::vector<int> &stat,
           std::vector<int> &dist, std::vector<int> &nodes, AggState &st)
      : S_(S), r_(r), maxa_(maxasize), stat_(stat), dist_(dist), nodes_(nodes), st_(st) {}

  // returns ok (0..3); nodes_[0..nneigs) are the found nodes
  int colour(int seed, int &nneigs) {
    nneigs = 0;
    stat_[(size_t)seed] = 1;
    dist_[(size_t)seed] = 0;
    inl_.assign(1, seed);
    return layer(0, nneigs);
  }

 private:
  int layer(int lay, int &nneigs) {
    bool fits = true;
    std::vector<int> newl;
    if (lay <= 2 * r_) {
      for (size_t q = 0; q < inl_.size(); q++) {
        int ln = inl_[q];
        for (int64_t k = S_.sptr[(size_t)ln]; k < S_.sptr[(size_t)ln + 1]; k++) {
          int cn = S_.scol[(size_t)k];
          if (stat_[(size_t)cn] <= 0) {
            if (stat_[(size_t)cn] == 0) {
              newl.push_back(cn);
              dist_[(size_t)cn] = dist_[(size_t)ln] + 1;
            }
            stat_[(size_t)cn] -= 1;  // weight for the rounding step
          }
        }
      }
    }
    if (lay <= r_) {  // rounding
      int nround = 0;
      std::vector<int> rounders;
      int mind = INT_MAX, maxd = 0;
      for (int cn : newl) {
        int d = -stat_[(size_t)cn];
        mind = std::min(mind, d);
        maxd = std::max(maxd, d);
      }
      if (mind < st_.allmind) st_.allmind = mind;
      if (mind < maxd || mind > st_.allmind) {
        for (size_t q = 0; q < newl.size(); q++) {
          if (stat_[(size_t)newl[q]] == -maxd) {
            nround++;
            if (nneigs + (int)inl_.size() + 1 > maxa_) { fits = false; break; }
            inl_.push_back(newl[q]);
            rounders.push_back(newl[q]);
            newl[q] = -1;
          }
        }
      }
      if (!fits) rounders.clear();
      newl.erase(std::remove(newl.begin(), newl.end(), -1), newl.end());
      for (int rn : rounders)
        for (int64_t k = S_.sptr[(size_t)rn]; k < S_.sptr[(size_t)rn + 1]; k++) {
          int cn = S_.scol[(size_t)k];
          if (stat_[(size_t)cn] == 0) {
            newl.push_back(cn);
            dist_[(size_t)cn] = dist_[(size_t)rn] + 1;
          }
        }
      (void)nround;
    }
    if (lay <= r_ && nneigs + (int)inl_.size() > maxa_) fits = false;
    if (fits) {
      for (int v : inl_) {
        stat_[(size_t)v] = lay + 1;
        put(nneigs++, v);
      }
      if (lay <= 2 * r_) {
        for (int v : newl) stat_[(size_t)v] = kPending - 1;
        inl_ = newl;
        return layer(lay + 1, nneigs);
      }
      return 3;
    }
    for (int v : inl_) dist_[(size_t)v] = 0;
    for (int v : newl) dist_[(size_t)v] = 0;
    for (int q = 0; q < nneigs; q++) dist_[(size_t)nodes_[(size_t)q]] = 0;
    for (int v : inl_) put(nneigs++, v);
    if (nneigs > 0) return lay > r_ ? 2 : 1;
    return 0;
  }

  void put(int pos, int v) {
    if ((size_t)pos >= nodes_.size()) nodes_.resize(2 * nodes_.size() + 64, 0);
    nodes_[(size_t)pos] = v;
  }

  const ScaledMatrix &S_;
  int r_, maxa_;
  std::vector<int> &stat_, &dist_, &nodes_;
  AggState &st_;
  std::vector<int> inl_;
};

static void form_aggr(Aggregates &ag, int nagr, int n, const std::vector<int> &num) {
  ag.nagr = nagr;
  ag.num = num;
  ag.starts.assign((size_t)nagr + 1, 0);
  for (int i = 0; i < n; i++)
    if (num[(size_t)i] > 0) ag.starts[(size_t)num[(size_t)i]]++;
  for (int a = 0; a < nagr; a++) ag.starts[(size_t)a + 1] += ag.starts[(size_t)a];
  ag.nodes.assign((size_t)ag.starts[(size_t)nagr], 0);
  std::vector<int> fill(ag.starts.begin(), ag.starts.end() - 1);
  for (int i = 0; i < n; i++)
    if (num[(size_t)i] > 0) ag.nodes[(size_t)fill[(size_t)num[(size_t)i] - 1]++] = i + 1;
}

// SpMtx_aggregate (SpMtx_aggregation.F90:49-641), one process.
static bool aggregate(ScaledMatrix &S, int neighood, int minasize, int maxasize, double alpha,
                      bool coarse, AggState &st, Aggregates &inner, Aggregates &full,
                      std::string &err) {
  const Csr &M = S.M;
  int n = M.nrows;
  std::vector<int> aggrnum((size_t)n, 0);
  int nagrs = 0, nisolated = 0;
  bool toosmall = false;
  int sn = (int)std::sqrt((float)n);
  int maxasizelargest;
  if (alpha >= 0 || sn * sn != n) {
    // the reference's nodes(n) can receive a node twice (a neighbour of two
    // rounder nodes is queued by each), so the list may outgrow n on small
    // graphs; it is sized with room for that
    std::vector<int> stat((size_t)n, 0), dist((size_t)n, 0), nodes((size_t)4 * n + 64, 0);
    // nextgoodstart (1-based, length n): good seeds at the head, the outer
    // layer of the newest aggregate at the tail, exactly as the reference.
    // The reference compacts the head list before every seed choice (drops
    // the seeds aggregated meanwhile) and then takes the first seed that
    // repeats an earlier one, else the first.  Validity belongs to a node,
    // not to a list position, so the same choice comes from an append-only
    // list L: a cursor over its first valid entry and a queue of the
    // positions where a node occurs for the second time (positions only
    // grow).  The explicit array is rebuilt only for an iteration whose tail
    // writes could reach the head, where the reference's overlapping use of
    // the one array has to be replayed.
    std::vector<int> ngs((size_t)n + 1, 0);
    std::vector<int> L;
    std::vector<int> occ((size_t)n, 0);
    std::deque<size_t> rep;
    size_t cur = 0;
    int64_t nvalid = 0;  // entries of L whose node is not aggregated
    auto append = [&](int v) {
      L.push_back(v);
      if (++occ[(size_t)v] == 2) rep.push_back(L.size() - 1);
      nvalid++;
    };
    auto rebuild = [&](int cnt) {  // L = ngs[1..cnt]
      for (int v : L) occ[(size_t)v] = 0;
      L.clear();
      rep.clear();
      cur = 0;
      nvalid = 0;
      for (int q = 1; q <= cnt; q++) append(ngs[(size_t)q]);
      for (int v : L)  // entries of aggregated nodes are not valid
        if (stat[(size_t)v] >= kPending) nvalid--;
    };
    maxasizelargest = coarse ? 3 * maxasize : maxasize + 4 * (2 * neighood);
    if (!coarse) st.beta = alpha / 4.0;
    Colourer col(S, neighood, maxasize, stat, dist, nodes, st);
    int first = 0;
    for (;;) {
      const int64_t valid_start = nvalid;  // the reference's compacted ngood
      int start;
      if (nvalid == 0) {
        while (first < n && stat[(size_t)first] >= kPending) first++;
        if (first >= n) break;
        start = first;
      } else {
        while (stat[(size_t)L[cur]] >= kPending) cur++;
        while (!rep.empty() && stat[(size_t)L[rep.front()]] >= kPending) rep.pop_front();
        start = rep.empty() ? L[cur] : L[rep.front()];
      }
      int nneigs = 0;
      int ok = col.colour(start, nneigs);
      if (ok <= 0) { err = "aggregation found nothing"; return false; }
      nagrs++;
      int next_layer;
      if (ok == 3) {
        std::vector<int> layerlen((size_t)2 * neighood + 3, 0);
        int maxlayer = 0;
        if (!toosmall && nneigs < minasize) toosmall = true;
        for (int q = nneigs - 1; q >= 0; q--) {
          int k = stat[(size_t)nodes[(size_t)q]];
          if (k > maxlayer) maxlayer = k;
          if (k <= neighood + 1) break;
          if (k > 2 * neighood + 2) { err = "aggregation layer out of range"; return false; }
          layerlen[(size_t)k]++;
        }
        next_layer = neighood + 2;
        int best = layerlen[(size_t)neighood + 2];
        for (int q = neighood + 3; q <= maxlayer; q++)
          if (best < layerlen[(size_t)q]) { best = layerlen[(size_t)q]; next_layer = q; }
      } else if (ok == 2) {
        next_layer = neighood + 2;
        if (!toosmall && nneigs < minasize) toosmall = true;
      } else {
        next_layer = 0;
      }
      // the outer layer's size first: it decides whether the tail writes of
      // the reference can reach its head list
      int nouter_all = 0;
      if (next_layer > neighood + 1)
        for (int q = 0; q < nneigs; q++) {
          int node = nodes[(size_t)q];
          if (!(stat[(size_t)node] <= neighood + 1 && q + 1 <= maxasize) && stat[(size_t)node] == next_layer)
            nouter_all++;
        }
      const bool replay = valid_start + 2 * (int64_t)nouter_all >= (int64_t)n;
      int ngood = 0;
      if (replay) {  // the reference's compacted head list in the array
        for (size_t q = cur; q < L.size(); q++)
          if (stat[(size_t)L[q]] < kPending) ngs[(size_t)++ngood] = L[q];
      }
      int mindistance = INT_MAX, nouters = 0;
      std::vector<int> outer;
      for (int q = 0; q < nneigs; q++) {
        int node = nodes[(size_t)q];
        if (stat[(size_t)node] <= neighood + 1 && q + 1 <= maxasize) {
          stat[(size_t)node] = kAggregated;
          aggrnum[(size_t)node] = nagrs;
          nvalid -= occ[(size_t)node];
        } else if (next_layer > neighood + 1) {
          if (stat[(size_t)node] == next_layer) {
            mindistance = std::min(mindistance, dist[(size_t)node]);
            nouters++;
            if (replay) ngs[(size_t)(n - nouters + 1)] = node;
            else outer.push_back(node);
          }
        }
      }
      if (replay) {
        for (int q = 1; q <= nouters; q++)
          if (dist[(size_t)ngs[(size_t)(n - q + 1)]] == mindistance) {
            ngood++;
            ngs[(size_t)ngood] = ngs[(size_t)(n - q + 1)];
          }
        rebuild(ngood);
      } else {
        for (int v : outer)
          if (dist[(size_t)v] == mindistance) append(v);
      }
      for (int q = 0; q < nneigs; q++) {
        int node = nodes[(size_t)q];
        if (stat[(size_t)node] != kAggregated) { dist[(size_t)node] = 0; stat[(size_t)node] = 0; }
      }
    }
  } else {
    // Cartesian aggregates (:332-346); the reference divides by the radius,
    // so a radius below 1 (the coarse default nint(3 n^(1/4) / (2 r1 + 1) - 1)
    // on a tiny coarse matrix) stops it with an integer division fault: here
    // it is an input error
    if (neighood < 1) {
      err = "Cartesian aggregation needs an aggregation radius >= 1 (radius " + std::to_string(neighood) +
            "); set radius1 / radius2";
      return false;
    }
    int nsa = (sn + neighood - 1) / neighood, k = 0;
    for (int i = 1; i <= sn; i++)
      for (int j = 1; j <= sn; j++)
        aggrnum[(size_t)k++] = ((i + neighood - 1) / neighood - 1) * nsa + (j + neighood - 1) / neighood;
    nagrs = *std::max_element(aggrnum.begin(), aggrnum.end());
    maxasizelargest = maxasize + 4 * (2 * neighood);
  }
  std::vector<int> fullnum;
  int full_nagrs;
  if (!toosmall) {
    fullnum = aggrnum;
    full_nagrs = std::max(0, n > 0 ? *std::max_element(fullnum.begin(), fullnum.end()) : 0);
    form_aggr(inner, nagrs, n, aggrnum);
  } else {
    // repair of too small aggregates (:369-591)
    std::vector<std::vector<int>> members((size_t)nagrs + 1);
    for (int i = 0; i < n; i++) members[(size_t)aggrnum[(size_t)i]].push_back(i);
    int nagrs_new = nagrs;
    for (int a = 1; a <= nagrs; a++) {
      int asz = (int)members[(size_t)a].size();
      if (asz >= minasize) continue;
      std::vector<int> cols;
      std::vector<double> wsum;
      for (int node : members[(size_t)a]) {
        for (int64_t k = M.ptr[(size_t)node]; k < M.ptr[(size_t)node + 1]; k++) {
          int cn = M.col[(size_t)k];
          if (cn >= n) continue;
          int colr = aggrnum[(size_t)cn];
          if (colr > 0 && colr != a) {
            size_t q = 0;
            for (; q < cols.size(); q++)
              if (cols[q] == colr) { wsum[q] = wsum[q] + std::fabs(M.val[(size_t)k]); break; }
            if (q == cols.size()) {
              if ((int)cols.size() >= 4 * maxasize) { err = "mnstructneigs too small"; return false; }
              cols.push_back(colr);
              wsum.push_back(std::fabs(M.val[(size_t)k]));
            }
          }
        }
      }
      double best = 0.0;
      int eater = 0;
      for (size_t q = 0; q < cols.size(); q++)
        if (best < wsum[q] && (int)members[(size_t)cols[q]].size() + asz <= maxasize) {
          best = wsum[q];
          eater = cols[q];
        }
      if (best >= alpha || (coarse && best >= st.beta)) {
        if (eater == 0) { err = "aggregate repair without an eater"; return false; }
        for (int node : members[(size_t)a]) {
          members[(size_t)eater].push_back(node);
          aggrnum[(size_t)node] = eater;
        }
        members[(size_t)a].clear();
        nagrs_new--;
      } else {
        // give the nodes away one by one, scanning from the last member
        std::vector<int> &mem = members[(size_t)a];
        int nleft = asz;
        bool reduced = true;
        while (nleft > 0 && reduced) {
          reduced = false;
          for (int q = (int)mem.size() - 1; q >= 0; q--) {
            int node = mem[(size_t)q];
            if (node < 0) continue;
            for (int64_t k = M.ptr[(size_t)node]; k < M.ptr[(size_t)node + 1]; k++) {
              int cn = M.col[(size_t)k];
              if (cn >= n) continue;
              int colr = aggrnum[(size_t)cn];
              if (colr != a) {
                if (colr < 1) { err = "repair found an unaggregated neighbour"; return false; }
                if ((int)members[(size_t)colr].size() < maxasizelargest &&
                    std::fabs(M.val[(size_t)k]) >= st.beta) {
                  members[(size_t)colr].push_back(node);
                  aggrnum[(size_t)node] = colr;
                  mem[(size_t)q] = -1;
                  nleft--;
                  reduced = true;
                  break;
                }
              }
            }
          }
        }
        if (nleft > 0 && nleft < asz) {
          std::vector<int> keep;
          for (int v : mem) if (v >= 0) keep.push_back(v);
          mem = keep;
        } else if (nleft == 0) {
          mem.clear();
          nagrs_new--;
        }
        // nleft == asz: the aggregate stays as it was
      }
    }
    int naggregated = 0;
    for (int a = 1; a <= nagrs; a++) naggregated += (int)members[(size_t)a].size();
    full_nagrs = nagrs_new;
    int cnt = *std::max_element(aggrnum.begin(), aggrnum.end());
    if (cnt > nagrs_new) {  // renumber in first-touch order (:539-559)
      std::vector<int> map((size_t)cnt + 1, 0);
      int colc = 0;
      for (int i = 0; i < n; i++) {
        int a = aggrnum[(size_t)i];
        if (a > 0) {
          if (map[(size_t)a] == 0) map[(size_t)a] = ++colc;
          aggrnum[(size_t)i] = map[(size_t)a];
        }
      }
    }
    fullnum.assign((size_t)n, 0);
    if (n == naggregated) {
      fullnum = aggrnum;
      full_nagrs = *std::max_element(fullnum.begin(), fullnum.end());
    } else {
      for (int i = 0; i < n; i++) {
        if (aggrnum[(size_t)i] > 0) fullnum[(size_t)i] = aggrnum[(size_t)i];
        else fullnum[(size_t)i] = ++full_nagrs;
      }
    }
    form_aggr(inner, nagrs_new, n, aggrnum);
    nisolated = n - naggregated;
  }
  (void)nisolated;
  form_aggr(full, full_nagrs, n, fullnum);
  return true;
}

// ---------------------------------------------------------------------------
// smoothed aggregation (CoarseMtx.F90:50-516)
// ---------------------------------------------------------------------------
static Coo smoother(const Csr &A, const std::vector<char> &strong, double omega, bool assign_diag) {
  int N = std::max(A.nrows, A.ncols);
  std::vector<double> d((size_t)N, 0.0);
  for (int r = 0; r < A.nrows; r++)
    for (int64_t k = A.ptr[(size_t)r]; k < A.ptr[(size_t)r + 1]; k++) {
      if (A.col[(size_t)k] == r) d[(size_t)r] = assign_diag ? A.val[(size_t)k] : d[(size_t)r] + A.val[(size_t)k];
      else if (!strong[(size_t)k]) d[(size_t)r] = d[(size_t)r] + A.val[(size_t)k];
    }
  Coo S;
  S.nrows = A.nrows; S.ncols = A.nrows;
  S.i.reserve(A.col.size()); S.j.reserve(A.col.size()); S.v.reserve(A.col.size());
  for (int r = 0; r < A.nrows; r++)
    for (int64_t k = A.ptr[(size_t)r]; k < A.ptr[(size_t)r + 1]; k++) {
      int c = A.col[(size_t)k];
      double v;
      if (c == r) v = 1.0 - omega;
      else if (strong[(size_t)k]) v = -(omega / d[(size_t)r] * A.val[(size_t)k]);
      else v = 0.0;  // weak connections stay as explicit zeros
      S.i.push_back(r); S.j.push_back(c); S.v.push_back(v);
    }
  return S;
}

// CoarseMtxBuild (CoarseMtx.F90:476-516): T = A R^T (R arranged by columns),
// AC = R T with R's rows re-bucketed from that column order.  Fills out.R
// (rows = coarse freedoms, columns ascending), out.P (= R^T, coarse freedoms
// ascending per fine node) and R's final COO order in out.R_i/R_j/R_v.
static Csr galerkin(const Csr &A, const Coo &Rcoo, int n, SetupResult &out, PhaseTimer *tm = nullptr) {
  Csr Rcols = cols_of(Rcoo);                 // column view: for each fine node, coarse freedoms ascending
  if (tm) tm->lap("R by columns");
  Csr Tm = spgemm_first_touch(A, Rcols);     // n x ncoarse
  if (tm) tm->lap("T = A R^T");
  Coo RcolOrder;                             // R's COO after arrangement by columns
  RcolOrder.nrows = Rcoo.nrows; RcolOrder.ncols = Rcoo.ncols;
  RcolOrder.i.reserve(Rcoo.size()); RcolOrder.j.reserve(Rcoo.size()); RcolOrder.v.reserve(Rcoo.size());
  for (int col = 0; col < Rcols.nrows; col++)
    for (int64_t k = Rcols.ptr[(size_t)col]; k < Rcols.ptr[(size_t)col + 1]; k++) {
      RcolOrder.i.push_back(Rcols.col[(size_t)k]);
      RcolOrder.j.push_back(col);
      RcolOrder.v.push_back(Rcols.val[(size_t)k]);
    }
  out.R = rows_of(RcolOrder);
  out.P = Rcols;
  out.P.nrows = n; out.P.ncols = Rcoo.nrows;
  if (tm) tm->lap("R by rows");
  Csr AC = spgemm_first_touch(out.R, Tm);
  out.R_i.clear(); out.R_j.clear(); out.R_v.clear();
  out.R_i.reserve(RcolOrder.size()); out.R_j.reserve(RcolOrder.size()); out.R_v.reserve(RcolOrder.size());
  for (size_t k = 0; k < RcolOrder.size(); k++) {
    out.R_i.push_back(RcolOrder.i[k] + 1); out.R_j.push_back(RcolOrder.j[k] + 1);
    out.R_v.push_back(RcolOrder.v[k]);
  }
  return AC;
}

// Add_layers (Decomposition.f90:56-99) for every node list in turn: each
// subdomain is its list grown by `overlap` breadth-first layers over the
// pattern of A; appended to out.sd_ptr / out.sd_nodes (1-based ids)
static void grow_subdomains(const Csr &A, const std::vector<std::vector<int>> &lists, int overlap, SetupResult &out) {
  const int n = A.nrows;
  out.sd_ptr.assign(1, 0);
  out.sd_nodes.clear();
  std::vector<int> onfront((size_t)n, 0), nodes;
  for (const auto &base : lists) {
    nodes = base;
    for (int v : nodes) onfront[(size_t)v] = -1;
    size_t lo = 0, hi = nodes.size();
    for (int layer = 1; layer <= overlap; layer++) {
      for (size_t q = lo; q < hi; q++) {
        int v = nodes[q];
        for (int64_t k = A.ptr[(size_t)v]; k < A.ptr[(size_t)v + 1]; k++) {
          int w = A.col[(size_t)k];
          if (onfront[(size_t)w] == 0) { onfront[(size_t)w] = layer; nodes.push_back(w); }
        }
      }
      lo = hi;
      hi = nodes.size();
    }
    for (int v : nodes) { onfront[(size_t)v] = 0; out.sd_nodes.push_back(v + 1); }
    out.sd_ptr.push_back((int64_t)out.sd_nodes.size());
  }
}

// 1-based triplets (0-based accepted, SpMtx_class.F90:441-444) to 0-based COO
static bool triplets(int n, const std::vector<int> &ii, const std::vector<int> &jj, const std::vector<double> &vv,
                     Coo &A0, std::string &err) {
  size_t nnz = vv.size();
  int shift = (nnz > 0 && ii[0] == 0) ? 1 : 0;
  A0 = Coo();
  A0.nrows = n; A0.ncols = n;
  A0.i.resize(nnz); A0.j.resize(nnz); A0.v = vv;
  for (size_t k = 0; k < nnz; k++) {
    int a = ii[k] + shift - 1, b = jj[k] + shift - 1;
    if (a < 0 || a >= n || b < 0 || b >= n) {
      err = "matrix entry " + std::to_string(k + 1) + " out of range";
      return false;
    }
    A0.i[k] = a; A0.j[k] = b;
  }
  return true;
}

bool build_setup_geom(const Controls &c_in, int n, const std::vector<int> &ii, const std::vector<int> &jj,
                      const std::vector<double> &vv, const std::vector<int> *part, int nparts,
                      const std::vector<int> *efree, const std::vector<int> *lg_fmap, const NodeGeometry *G,
                      SetupResult &out, std::string &err) {
  Controls c = c_in;
  out = SetupResult();
  out.n = n;
  PhaseTimer tm;
  if (c.method == 2 || c.method == 3) {
    err = "method " + std::to_string(c.method) +
          " restricts a residual the one-process reference never sets (pcg.F90:146-149)";
    return false;
  }
  if (c.levels > 2) { err = "doug_geom builds no coarse level for levels " + std::to_string(c.levels); return false; }
  if (c.levels == 2 && (c.input_type != 1 || !efree || !lg_fmap || !G)) {
    err = "the geometric coarse grid needs elemental input with node coordinates (coords_file, freemap_file)";
    return false;
  }
  Coo A0;
  if (!triplets(n, ii, jj, vv, A0, err)) return false;
  const Csr A = rows_of(A0);  // FinePreconditioner_Init arranges A by rows (Preconditioner_base.F90:109)
  out.fine.num.assign((size_t)n, 0);
  out.fine_full.num.assign((size_t)n, 0);
  out.overlap = c.overlap < 0 ? std::max(c.smoothers, 0) : c.overlap;  // geom.F90:96-100, before the coarse init
  out.levels = c.levels;
  std::vector<std::vector<int>> lists;
  if (part) {
    lists.resize((size_t)nparts);
    for (int i = 0; i < n; i++) lists[(size_t)(*part)[(size_t)i] - 1].push_back(i);
  } else {
    lists.resize(1);
    for (int i = 0; i < n; i++) lists[0].push_back(i);
  }
  grow_subdomains(A, lists, out.overlap, out);
  tm.lap("subdomains + overlap");
  out.smoothers = c.smoothers;
  if (c.levels == 2) {
    out.smoothers = 0;  // CoarsePreconditioner_geometric.F90:53
    Coo Rcoo;
    std::vector<double> cxyz;
    if (!geometric_restriction(c, *efree, *G, *lg_fmap, Rcoo, cxyz, err)) return false;
    tm.lap("geometric coarse grid");
    Csr AC = galerkin(A, Rcoo, n, out);
    out.AC_i.reserve(AC.col.size()); out.AC_j.reserve(AC.col.size()); out.AC_v.reserve(AC.col.size());
    for (int r = 0; r < AC.nrows; r++)
      for (int64_t k = AC.ptr[(size_t)r]; k < AC.ptr[(size_t)r + 1]; k++) {
        out.AC_i.push_back(r + 1); out.AC_j.push_back(AC.col[(size_t)k] + 1); out.AC_v.push_back(AC.val[(size_t)k]);
      }
    out.coarse_xyz = cxyz;
    const std::vector<int> keep = independent_coarse(AC);
    const int nk = keep.empty() ? 0 : *std::max_element(keep.begin(), keep.end());
    if (nk < AC.nrows) {  // the solve uses the independent coarse freedoms only
      Coo Rs, ACs;
      Rs.nrows = nk; Rs.ncols = n;
      for (size_t k = 0; k < Rcoo.size(); k++)
        if (keep[(size_t)Rcoo.i[k]]) { Rs.i.push_back(keep[(size_t)Rcoo.i[k]] - 1); Rs.j.push_back(Rcoo.j[k]); Rs.v.push_back(Rcoo.v[k]); }
      ACs.nrows = ACs.ncols = nk;
      for (int r = 0; r < AC.nrows; r++)
        for (int64_t k = AC.ptr[(size_t)r]; k < AC.ptr[(size_t)r + 1]; k++)
          if (keep[(size_t)r] && keep[(size_t)AC.col[(size_t)k]]) {
            ACs.i.push_back(keep[(size_t)r] - 1); ACs.j.push_back(keep[(size_t)AC.col[(size_t)k]] - 1);
            ACs.v.push_back(AC.val[(size_t)k]);
          }
      Csr Rcols = cols_of(Rs);
      out.P = Rcols;
      out.P.nrows = n; out.P.ncols = nk;
      Coo Rc;  // by columns, then rows
      Rc.nrows = nk; Rc.ncols = n;
      for (int col = 0; col < Rcols.nrows; col++)
        for (int64_t k = Rcols.ptr[(size_t)col]; k < Rcols.ptr[(size_t)col + 1]; k++) {
          Rc.i.push_back(Rcols.col[(size_t)k]); Rc.j.push_back(col); Rc.v.push_back(Rcols.val[(size_t)k]);
        }
      out.R = rows_of(Rc);
      AC = rows_of(ACs);
    }
    out.AC = AC;
    tm.lap("restriction + Galerkin");
  }
  out.A = A;
  return true;
}

bool build_setup(const Controls &c_in, int n, const std::vector<int> &ii, const std::vector<int> &jj,
                 const std::vector<double> &vv, const std::vector<int> *part, int nparts,
                 SetupResult &out, std::string &err, const RobustHook *robust, bool on_device) {
  Controls c = c_in;
  out = SetupResult();
  out.n = n;
  PhaseTimer tm;
  if (c.fine_method < 0 || c.fine_method > 2) {
    err = "Wrong fine method " + std::to_string(c.fine_method);
    return false;
  }
  if (c.method == 2 || c.method == 3) {
    // the one-process reference restricts a residual vector it allocates but
    // never sets for these multiplicative variants (pcg.F90:146-149, 264-266)
    err = "method " + std::to_string(c.method) +
          " restricts a residual the one-process reference never sets (pcg.F90:146-149)";
    return false;
  }
  if (c.coarse_method > 2) {  // aggr.F90:155-165 (3: build_setup_rbm, with node coordinates)
    err = c.coarse_method == 3 ? std::string("coarse_method 3 needs node coordinates (elemental input with "
                                             "coords_file / freemap_file or dg_set_node_geometry)")
                               : "Wrong coarse method " + std::to_string(c.coarse_method);
    return false;
  }
  if (c.coarse_method == 2 && !robust) {
    err = "coarse_method 2 (robust coarse space) needs the device B-solve";
    return false;
  }
  Coo A0;
  if (!triplets(n, ii, jj, vv, A0, err)) return false;
  // Partitionings_aggr_InitFine (Partitioning_aggr.F90:33-117)
  out.strong1 = (c.strong1 != 0.0) ? c.strong1 : 0.67;
  out.r1 = c.radius1 > 0 ? c.radius1 : 2;
  out.min1 = c.minasize1 > 0 ? c.minasize1 : (int)(0.5 * (double)((2 * out.r1 + 1) * (2 * out.r1 + 1)));
  out.max1 = c.maxasize1 > 0 ? c.maxasize1 : (2 * out.r1 + 1) * (2 * out.r1 + 1);
  AggState st;
  ScaledMatrix SA;
  SA.M = rows_of(A0);
  tm.lap("arrange by rows");
  SA.symmetric = c.symmstruct && c.symmnumeric;
  scale_rows(SA);
  tm.lap("scale");
  find_strong(SA, out.strong1);
  tm.lap("fine strength");
  if (!aggregate(SA, out.r1, out.min1, out.max1, out.strong1, false, st, out.fine, out.fine_full, err))
    return false;
  unscale_rows(SA);
  tm.lap("fine aggregation");
  out.t_aggregation = tm.total;
  const Csr &A = SA.M;
  // IntRestBuild (CoarseMtx.F90:50-474); smoothers are capped at radius1
  if (c.smoothers > c.radius1) c.smoothers = c.radius1;
  int sm = c.smoothers;
  if (sm < 0) { err = "smoothers must be >= 0 for the smoothed-aggregation coarse space"; return false; }
  Csr AC;
  if (on_device && c.device_setup == 1 && c.coarse_method <= 1 && sm <= 1) {
    // smoother, re-bucketing and the three first-touch products on the GPU
    if (!device_restriction_galerkin(A, SA.strong, out.fine, sm, c.omega, out, AC, out.t_coarse, err)) return false;
    out.coarse_on_device = true;
    tm.lap("restriction + Galerkin (GPU)");
  } else {
  Coo T;  // tentative prolongator as restriction rows
  T.nrows = out.fine.nagr; T.ncols = n;
  T.i.reserve((size_t)n); T.j.reserve((size_t)n); T.v.reserve((size_t)n);
  for (int a = 0; a < out.fine.nagr; a++)
    for (int q = out.fine.starts[(size_t)a]; q < out.fine.starts[(size_t)a + 1]; q++) {
      T.i.push_back(a); T.j.push_back(out.fine.nodes[(size_t)q] - 1); T.v.push_back(1.0);
    }
  Csr Trows = rows_of(T);
  Csr R;  // reference's Restrict, arranged by rows after SpMtx_AB
  Coo Rcoo;
  if (sm == 0) {
    Rcoo = T;
  } else {
    Coo S = smoother(A, SA.strong, c.omega, false);
    tm.lap("smoother");
    if (sm == 1) {
      R = spgemm_first_touch(Trows, cols_of(S));
      tm.lap("R = T S^T");
    } else {
      Coo S2 = smoother(A, SA.strong, c.omega, true);
      Csr SS = spgemm_first_touch(rows_of(S2), rows_of(S));
      auto mul = [&](const Csr &X, const Csr &Y) { return spgemm_first_touch(X, Y); };
      Csr S2r = rows_of(S2);
      if (sm == 3) R = mul(Trows, mul(SS, S2r));
      else if (sm == 4) R = mul(Trows, mul(SS, SS));
      else if (sm == 5) R = mul(Trows, mul(mul(SS, SS), S2r));
      else if (sm == 6) R = mul(Trows, mul(mul(SS, SS), SS));
      else if (sm == 7) R = mul(Trows, mul(mul(mul(SS, SS), SS), S2r));
      else if (sm == 8) { Csr S4 = mul(SS, SS); R = mul(Trows, mul(S4, S4)); }
      else R = mul(Trows, cols_of(coo_of(SS)));  // 2 (and >8, performed as 2)
    }
    Rcoo = coo_of(R);
  }
  if (c.coarse_method == 2) {
    // CoarsePreconditioner_robust_Init (CoarsePreconditioner_robust.F90:34-63): the
    // supports are R's rows in R's entry order (CoarseProjectionMtxsBuild,
    // RobustCoarseMtx.f90:85-103); the new R holds q_i on S_i, rows one after
    // the other (RobustRestrictMtxBuild, :175-202)
    const int na = Rcoo.nrows;
    std::vector<int64_t> sp((size_t)na + 1, 0);
    for (size_t k = 0; k < Rcoo.size(); k++) sp[(size_t)Rcoo.i[k] + 1]++;
    for (int a = 0; a < na; a++) sp[(size_t)a + 1] += sp[(size_t)a];
    std::vector<int> sn(Rcoo.size());
    std::vector<int64_t> fp(sp.begin(), sp.end() - 1);
    for (size_t k = 0; k < Rcoo.size(); k++) sn[(size_t)fp[(size_t)Rcoo.i[k]]++] = Rcoo.j[k];
    std::vector<double> q;
    if (!(*robust)(A, sp, sn, q, err)) return false;
    Coo Rh;
    Rh.nrows = na; Rh.ncols = Rcoo.ncols;
    Rh.i.resize(sn.size()); Rh.j = sn; Rh.v = q;
    for (int a = 0; a < na; a++)
      for (int64_t k = sp[(size_t)a]; k < sp[(size_t)a + 1]; k++) Rh.i[(size_t)k] = a;
    Rcoo = Rh;
    tm.lap("robust coarse space");
  }
  tm.lap("restriction");
  AC = galerkin(A, Rcoo, n, out, &tm);
  out.t_coarse = tm.lap("Galerkin");
  }
  // Partitionings_aggr_InitCoarse (Partitioning_aggr.F90:120-193)
  out.strong2 = c.strong2 > 0 ? c.strong2 : out.strong1 / 2.0;
  ScaledMatrix SC;
  SC.M = AC;
  SC.symmetric = false;
  scale_rows(SC);
  find_strong(SC, out.strong2);
  if (c.radius2 > 0) out.r2 = c.radius2;
  else {
    int nn = (int)std::sqrt(1.0 * (double)n);
    out.r2 = (int)std::lround(3.0 * std::sqrt((double)nn) / (double)(2 * out.r1 + 1) - 1.0);
  }
  if (c.minasize2 > 0) out.min2 = c.minasize2;
  else if (c.radius2 > 0) out.min2 = 2 * c.radius2 + 1;
  else out.min2 = (int)(0.5 * (double)((2 * out.r2 + 1) * (2 * out.r2 + 1)));
  out.max2 = c.maxasize2 > 0 ? c.maxasize2 : (2 * out.r2 + 1) * (2 * out.r2 + 1);
  if (!aggregate(SC, out.r2, out.min2, out.max2, out.strong2, true, st, out.coarse,
                 out.coarse_full, err))
    return false;
  unscale_rows(SC);
  tm.lap("coarse aggregation");
  out.AC = SC.M;
  out.AC_i.reserve(out.AC.col.size()); out.AC_j.reserve(out.AC.col.size()); out.AC_v.reserve(out.AC.col.size());
  for (int r = 0; r < out.AC.nrows; r++)
    for (int64_t k = out.AC.ptr[(size_t)r]; k < out.AC.ptr[(size_t)r + 1]; k++) {
      out.AC_i.push_back(r + 1); out.AC_j.push_back(out.AC.col[(size_t)k] + 1);
      out.AC_v.push_back(out.AC.val[(size_t)k]);
    }
  // subdomains (Preconditioner_base.F90:96-123, Decomposition.f90:56-99)
  out.overlap = c.overlap < 0 ? std::max(c.smoothers, 0) : c.overlap;
  out.smoothers = c.smoothers;
  out.levels = c.levels;
  int np = part ? nparts : out.coarse_full.nagr;
  std::vector<std::vector<int>> lists((size_t)np);
  if (part) {  // Get_nodes (Decomposition.f90:35-53) for every part in one sweep
    for (int i = 0; i < n; i++) lists[(size_t)(*part)[(size_t)i] - 1].push_back(i);
  } else {  // Get_aggregate_nodes (Aggregate_mod.F90:162-190)
    std::vector<int> loc((size_t)n, 0);
    const Aggregates &ca = out.coarse_full, &fa = out.fine_full;
    for (int p = 1; p <= np; p++) {
      std::vector<int> &nodes = lists[(size_t)p - 1];
      for (int q = ca.starts[(size_t)p - 1]; q < ca.starts[(size_t)p]; q++) {
        int f = ca.nodes[(size_t)q];
        for (int t = fa.starts[(size_t)f - 1]; t < fa.starts[(size_t)f]; t++) {
          int node = fa.nodes[(size_t)t] - 1;
          if (!loc[(size_t)node]) { loc[(size_t)node] = 1; nodes.push_back(node); }
        }
      }
      for (int v : nodes) loc[(size_t)v] = 0;
    }
  }
  // the reference restarts each overlap layer one entry early; that entry's
  // neighbours are already marked, so the visited order is unchanged
  grow_subdomains(A, lists, out.overlap, out);
  tm.lap("subdomains + overlap");
  out.A = A;
  return true;
}

// The three aggregation passes of smoothed aggregation on a weighted graph
// (vertex v's neighbours col[ptr[v]..ptr[v+1]) with weights val, strong
// flags): (1) a vertex whose strong neighbours are all free starts an
// aggregate with them; (2) a free vertex joins the phase-1 aggregate of its
// strongest aggregated strong neighbour (first on ties); (3) every vertex
// still free starts an aggregate with its free strong neighbours.  Vertices
// in order; agg[v] = 0-based aggregate; returns the number of aggregates.
static int three_phase_aggregate(int nv, const std::vector<int64_t> &ptr, const std::vector<int> &col,
                                 const std::vector<double> &val, const std::vector<char> &strong,
                                 std::vector<int> &agg) {
  agg.assign((size_t)nv, -1);
  int na = 0;
  for (int I = 0; I < nv; I++) {
    if (agg[(size_t)I] >= 0) continue;
    bool free_all = true;
    for (int64_t q = ptr[(size_t)I]; q < ptr[(size_t)I + 1] && free_all; q++)
      if (strong[(size_t)q] && col[(size_t)q] != I && agg[(size_t)col[(size_t)q]] >= 0) free_all = false;
    if (!free_all) continue;
    agg[(size_t)I] = na;
    for (int64_t q = ptr[(size_t)I]; q < ptr[(size_t)I + 1]; q++)
      if (strong[(size_t)q]) agg[(size_t)col[(size_t)q]] = na;
    na++;
  }
  const std::vector<int> agg1 = agg;
  for (int I = 0; I < nv; I++) {
    if (agg1[(size_t)I] >= 0) continue;
    int best = -1;
    double bv = 0.0;
    for (int64_t q = ptr[(size_t)I]; q < ptr[(size_t)I + 1]; q++)
      if (strong[(size_t)q] && agg1[(size_t)col[(size_t)q]] >= 0 && (best < 0 || val[(size_t)q] > bv)) {
        best = agg1[(size_t)col[(size_t)q]];
        bv = val[(size_t)q];
      }
    if (best >= 0) agg[(size_t)I] = best;
  }
  for (int I = 0; I < nv; I++) {
    if (agg[(size_t)I] >= 0) continue;
    agg[(size_t)I] = na;
    for (int64_t q = ptr[(size_t)I]; q < ptr[(size_t)I + 1]; q++)
      if (strong[(size_t)q] && agg[(size_t)col[(size_t)q]] < 0) agg[(size_t)col[(size_t)q]] = na;
    na++;
  }
  return na;
}

// ---------------------------------------------------------------------------
// Smoothed aggregation over nodal blocks with a rigid-body near-nullspace
// (coarse_method 3; no counterpart in the reference, whose aggregation is
// scalar: SpMtx_aggregation.F90:49-641).  The method is the smoothed
// aggregation of Vanek, Mandel and Brezina (Computing 56 (1996) 179-196) for
// systems: aggregates of mesh nodes from the block strength ||A_IJ||_F >
// theta sqrt(||A_II||_F ||A_JJ||_F); per aggregate the rigid-body modes
// (nsd translations, 1 or 3 rotations about the aggregate's centroid)
// orthonormalised by twice-repeated modified Gram-Schmidt (columns that
// vanish are dropped) form the tentative prolongator; radius1 rounds of
// aggregation (the later ones over the previous round's aggregates) set
// the aggregate size; Jacobi smoothing
// P = (I - omega D^-1 A) P_tent with omega = 4 / (3 rho(D^-1 A)), rho by 20
// power steps; R = P^T and AC = R A P.  Every loop runs in a fixed order, so
// the oracle's restatement gives the same bits.
// ---------------------------------------------------------------------------
bool build_setup_rbm(const Controls &c_in, int n, const std::vector<int> &ii, const std::vector<int> &jj,
                     const std::vector<double> &vv, const std::vector<int> *part, int nparts,
                     const std::vector<int> &unode, int nsd, const std::vector<double> &xyz, SetupResult &out,
                     std::string &err) {
  Controls c = c_in;
  out = SetupResult();
  out.n = n;
  PhaseTimer tm;
  if (c.method == 2 || c.method == 3) {
    err = "method " + std::to_string(c.method) +
          " restricts a residual the one-process reference never sets (pcg.F90:146-149)";
    return false;
  }
  if (c.fine_method < 0 || c.fine_method > 2) {
    err = "Wrong fine method " + std::to_string(c.fine_method);
    return false;
  }
  if (!part) {
    err = "coarse_method 3 builds no coarse aggregates for subdomains: give a partition (dg_set_partition)";
    return false;
  }
  if (nsd != 2 && nsd != 3) { err = "coarse_method 3 needs 2-D or 3-D node coordinates"; return false; }
  if ((int)unode.size() != n) { err = "coarse_method 3: the node of every unknown is needed"; return false; }
  Coo A0;
  if (!triplets(n, ii, jj, vv, A0, err)) return false;
  const Csr A = rows_of(A0);
  tm.lap("arrange by rows");
  out.strong1 = (c.strong1 != 0.0) ? c.strong1 : 0.67;
  const double theta = out.strong1;
  // nodes in order of first appearance; a node's unknowns ascending are its
  // components 1..nsd
  std::vector<int> nid(xyz.size() / (size_t)nsd + 1, -1), node_of((size_t)n), comp((size_t)n);
  std::vector<int> node_glob, ncomp;
  for (int u = 0; u < n; u++) {
    const int g = unode[(size_t)u];
    if (g < 0 || (size_t)g >= nid.size() - 1) { err = "coarse_method 3: node of unknown out of range"; return false; }
    if (nid[(size_t)g] < 0) { nid[(size_t)g] = (int)node_glob.size(); node_glob.push_back(g); ncomp.push_back(0); }
    const int k = nid[(size_t)g];
    node_of[(size_t)u] = k;
    comp[(size_t)u] = ncomp[(size_t)k]++;
  }
  const int nn = (int)node_glob.size();
  for (int k = 0; k < nn; k++)
    if (ncomp[(size_t)k] != nsd) {
      err = "coarse_method 3 needs all " + std::to_string(nsd) + " freedoms of every node (node " +
            std::to_string(node_glob[(size_t)k] + 1) + " has " + std::to_string(ncomp[(size_t)k]) + ")";
      return false;
    }
  std::vector<std::vector<int>> node_unk((size_t)nn);
  for (int u = 0; u < n; u++) node_unk[(size_t)node_of[(size_t)u]].push_back(u);
  // block norms ||A_IJ||_F^2, neighbours in first-touch order
  std::vector<int64_t> nptr((size_t)nn + 1, 0);
  std::vector<int> ncol;
  std::vector<double> nval;
  {
    std::vector<int> pos((size_t)nn, -1);
    for (int I = 0; I < nn; I++) {
      const int64_t base = (int64_t)ncol.size();
      for (int u : node_unk[(size_t)I])
        for (int64_t k = A.ptr[(size_t)u]; k < A.ptr[(size_t)u + 1]; k++) {
          const int J = node_of[(size_t)A.col[(size_t)k]];
          const double a = A.val[(size_t)k];
          if (pos[(size_t)J] < 0) { pos[(size_t)J] = (int)ncol.size(); ncol.push_back(J); nval.push_back(a * a); }
          else nval[(size_t)pos[(size_t)J]] = nval[(size_t)pos[(size_t)J]] + a * a;
        }
      for (int64_t q = base; q < (int64_t)ncol.size(); q++) pos[(size_t)ncol[(size_t)q]] = -1;
      nptr[(size_t)I + 1] = (int64_t)ncol.size();
    }
  }
  std::vector<double> dnorm((size_t)nn, 0.0);
  for (size_t q = 0; q < nval.size(); q++) nval[q] = std::sqrt(nval[q]);
  for (int I = 0; I < nn; I++)
    for (int64_t q = nptr[(size_t)I]; q < nptr[(size_t)I + 1]; q++)
      if (ncol[(size_t)q] == I) dnorm[(size_t)I] = nval[(size_t)q];
  std::vector<char> strong(ncol.size(), 0);
  for (int I = 0; I < nn; I++)
    for (int64_t q = nptr[(size_t)I]; q < nptr[(size_t)I + 1]; q++) {
      const int J = ncol[(size_t)q];
      strong[(size_t)q] = J != I && nval[(size_t)q] > theta * std::sqrt(dnorm[(size_t)I] * dnorm[(size_t)J]);
    }
  tm.lap("block strength");
  // aggregation rounds: round 1 aggregates the nodes over the strong block
  // graph; every further round (radius1 rounds in all, at least 1)
  // aggregates the previous round's aggregates over the graph of their
  // strong connections (weight: the sum of the block norms between them)
  std::vector<int> agg;
  int na = three_phase_aggregate(nn, nptr, ncol, nval, strong, agg);
  const int rounds = c.radius1 > 0 ? c.radius1 : 1;
  for (int round = 2; round <= rounds && na > 1; round++) {
    std::vector<int64_t> gptr((size_t)na + 1, 0);
    std::vector<int> gcol;
    std::vector<double> gval;
    std::vector<std::vector<int>> members((size_t)na);
    for (int I = 0; I < nn; I++) members[(size_t)agg[(size_t)I]].push_back(I);
    std::vector<int> pos((size_t)na, -1);
    for (int a = 0; a < na; a++) {
      const int64_t base = (int64_t)gcol.size();
      for (int I : members[(size_t)a])
        for (int64_t q = nptr[(size_t)I]; q < nptr[(size_t)I + 1]; q++) {
          if (!strong[(size_t)q]) continue;
          const int b = agg[(size_t)ncol[(size_t)q]];
          if (b == a) continue;
          if (pos[(size_t)b] < 0) { pos[(size_t)b] = (int)gcol.size(); gcol.push_back(b); gval.push_back(nval[(size_t)q]); }
          else gval[(size_t)pos[(size_t)b]] = gval[(size_t)pos[(size_t)b]] + nval[(size_t)q];
        }
      for (int64_t q = base; q < (int64_t)gcol.size(); q++) pos[(size_t)gcol[(size_t)q]] = -1;
      gptr[(size_t)a + 1] = (int64_t)gcol.size();
    }
    std::vector<char> gstrong(gcol.size(), 1);
    std::vector<int> agg2;
    const int na2 = three_phase_aggregate(na, gptr, gcol, gval, gstrong, agg2);
    for (int I = 0; I < nn; I++) agg[(size_t)I] = agg2[(size_t)agg[(size_t)I]];
    na = na2;
  }
  tm.lap("node aggregation");
  // tentative prolongator: rigid-body modes per aggregate, orthonormalised
  std::vector<std::vector<int>> agg_nodes((size_t)na);
  for (int I = 0; I < nn; I++) agg_nodes[(size_t)agg[(size_t)I]].push_back(I);
  const int nmodes = nsd == 3 ? 6 : 3;
  std::vector<int> cfirst((size_t)na + 1, 0);   // coarse freedoms of aggregate a: [cfirst[a], cfirst[a+1])
  std::vector<std::vector<double>> Q((size_t)na);
  for (int a = 0; a < na; a++) {
    const std::vector<int> &nodes = agg_nodes[(size_t)a];
    const int m = (int)nodes.size(), rows = m * nsd;
    double cen[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < nsd; d++) {
      for (int I : nodes) cen[d] = cen[d] + xyz[(size_t)node_glob[(size_t)I] * nsd + d];
      cen[d] = cen[d] / (double)m;
    }
    std::vector<double> B((size_t)rows * nmodes, 0.0);  // column-major rows x nmodes
    for (int t = 0; t < m; t++) {
      const int g = node_glob[(size_t)nodes[(size_t)t]];
      const double x = xyz[(size_t)g * nsd] - cen[0], y = xyz[(size_t)g * nsd + 1] - cen[1];
      const double z = nsd == 3 ? xyz[(size_t)g * nsd + 2] - cen[2] : 0.0;
      for (int d = 0; d < nsd; d++) B[(size_t)d * rows + (size_t)t * nsd + d] = 1.0;
      double *r = &B[(size_t)nsd * rows + (size_t)t * nsd];
      if (nsd == 2) {
        r[0] = -y; r[1] = x;
      } else {
        r[1] = -z; r[2] = y;                       // about x: (0, -z, y)
        r[(size_t)rows] = z; r[(size_t)rows + 2] = -x;   // about y: (z, 0, -x)
        r[2 * (size_t)rows] = -y; r[2 * (size_t)rows + 1] = x;  // about z: (-y, x, 0)
      }
    }
    std::vector<double> &q = Q[(size_t)a];
    int kept = 0;
    for (int col = 0; col < nmodes; col++) {
      std::vector<double> v(B.begin() + (size_t)col * rows, B.begin() + (size_t)(col + 1) * rows);
      double n0 = 0.0;
      for (int i = 0; i < rows; i++) n0 = n0 + v[(size_t)i] * v[(size_t)i];
      n0 = std::sqrt(n0);
      for (int pass = 0; pass < 2; pass++)
        for (int p2 = 0; p2 < kept; p2++) {
          const double *qp = &q[(size_t)p2 * rows];
          double h = 0.0;
          for (int i = 0; i < rows; i++) h = h + qp[i] * v[(size_t)i];
          for (int i = 0; i < rows; i++) v[(size_t)i] = v[(size_t)i] - h * qp[i];
        }
      double nv = 0.0;
      for (int i = 0; i < rows; i++) nv = nv + v[(size_t)i] * v[(size_t)i];
      nv = std::sqrt(nv);
      if (!(nv > 1e-8 * n0)) continue;
      for (int i = 0; i < rows; i++) q.push_back(v[(size_t)i] / nv);
      kept++;
    }
    cfirst[(size_t)a + 1] = cfirst[(size_t)a] + kept;
  }
  const int nc = cfirst[(size_t)na];
  // P_tent by rows: unknown u of node t (position t in its aggregate), component d
  std::vector<int> pos_in_agg((size_t)nn, 0);
  for (int a = 0; a < na; a++)
    for (size_t t = 0; t < agg_nodes[(size_t)a].size(); t++) pos_in_agg[(size_t)agg_nodes[(size_t)a][t]] = (int)t;
  Coo Pt;
  Pt.nrows = n; Pt.ncols = nc;
  for (int u = 0; u < n; u++) {
    const int I = node_of[(size_t)u], a = agg[(size_t)I];
    const int rows = (int)agg_nodes[(size_t)a].size() * nsd;
    const int r = pos_in_agg[(size_t)I] * nsd + comp[(size_t)u];
    for (int col = cfirst[(size_t)a]; col < cfirst[(size_t)a + 1]; col++) {
      Pt.i.push_back(u); Pt.j.push_back(col);
      Pt.v.push_back(Q[(size_t)a][(size_t)(col - cfirst[(size_t)a]) * rows + r]);
    }
  }
  const Csr Ptr = rows_of(Pt);
  tm.lap("tentative prolongator");
  // omega = 4 / (3 rho(D^-1 A)), rho from 20 power steps
  std::vector<double> dg((size_t)n, 0.0);
  for (int u = 0; u < n; u++)
    for (int64_t k = A.ptr[(size_t)u]; k < A.ptr[(size_t)u + 1]; k++)
      if (A.col[(size_t)k] == u) dg[(size_t)u] = A.val[(size_t)k];
  for (int u = 0; u < n; u++)
    if (!(dg[(size_t)u] > 0.0)) { err = "coarse_method 3: non-positive diagonal at unknown " + std::to_string(u + 1); return false; }
  std::vector<double> xv((size_t)n), yv((size_t)n);
  for (int u = 0; u < n; u++) xv[(size_t)u] = 1.0 + (double)(u % 7) / 7.0;
  double rho = 0.0;
  for (int it = 0; it < 20; it++) {
    parallel_rows(n, [&](int lo, int hi) {
      for (int u = lo; u < hi; u++) {
        double sacc = 0.0;
        for (int64_t k = A.ptr[(size_t)u]; k < A.ptr[(size_t)u + 1]; k++)
          sacc = sacc + A.val[(size_t)k] * xv[(size_t)A.col[(size_t)k]];
        yv[(size_t)u] = sacc / dg[(size_t)u];
      }
    });
    double ny = 0.0, nx = 0.0;
    for (int u = 0; u < n; u++) { ny = ny + yv[(size_t)u] * yv[(size_t)u]; nx = nx + xv[(size_t)u] * xv[(size_t)u]; }
    ny = std::sqrt(ny);
    rho = ny / std::sqrt(nx);
    for (int u = 0; u < n; u++) xv[(size_t)u] = yv[(size_t)u] / ny;
  }
  const double omega = 4.0 / (3.0 * rho);
  tm.lap("spectral radius");
  // P = P_tent - omega D^-1 (A P_tent), the pattern of A P_tent
  Csr AP = spgemm_first_touch(A, Ptr);
  Coo Rcoo;  // R = P^T as coarse x fine, unknown after unknown
  Rcoo.nrows = nc; Rcoo.ncols = n;
  {
    std::vector<double> ptv((size_t)nc, 0.0);
    for (int u = 0; u < n; u++) {
      for (int64_t k = Ptr.ptr[(size_t)u]; k < Ptr.ptr[(size_t)u + 1]; k++) ptv[(size_t)Ptr.col[(size_t)k]] = Ptr.val[(size_t)k];
      const double w = omega / dg[(size_t)u];
      for (int64_t k = AP.ptr[(size_t)u]; k < AP.ptr[(size_t)u + 1]; k++) {
        const int col = AP.col[(size_t)k];
        Rcoo.i.push_back(col); Rcoo.j.push_back(u); Rcoo.v.push_back(ptv[(size_t)col] - w * AP.val[(size_t)k]);
      }
      for (int64_t k = Ptr.ptr[(size_t)u]; k < Ptr.ptr[(size_t)u + 1]; k++) ptv[(size_t)Ptr.col[(size_t)k]] = 0.0;
    }
  }
  tm.lap("smoothed prolongator");
  Csr AC = galerkin(A, Rcoo, n, out, &tm);
  tm.lap("Galerkin");
  out.AC = AC;
  out.AC_i.reserve(AC.col.size()); out.AC_j.reserve(AC.col.size()); out.AC_v.reserve(AC.col.size());
  for (int r = 0; r < AC.nrows; r++)
    for (int64_t k = AC.ptr[(size_t)r]; k < AC.ptr[(size_t)r + 1]; k++) {
      out.AC_i.push_back(r + 1); out.AC_j.push_back(AC.col[(size_t)k] + 1); out.AC_v.push_back(AC.val[(size_t)k]);
    }
  // unknowns' aggregates (1-based) for export; no coarse aggregates
  std::vector<int> num((size_t)n);
  for (int u = 0; u < n; u++) num[(size_t)u] = agg[(size_t)node_of[(size_t)u]] + 1;
  form_aggr(out.fine, na, n, num);
  out.fine_full = out.fine;
  out.coarse.num.clear();
  out.overlap = c.overlap < 0 ? std::max(c.smoothers, 0) : c.overlap;
  out.smoothers = c.smoothers;
  out.levels = c.levels;
  std::vector<std::vector<int>> lists((size_t)nparts);
  for (int i = 0; i < n; i++) lists[(size_t)(*part)[(size_t)i] - 1].push_back(i);
  grow_subdomains(A, lists, out.overlap, out);
  tm.lap("subdomains + overlap");
  out.A = A;
  return true;
}

namespace {

void append_aggregates(Aggregates &dst, const Aggregates &src, int member_off) {
  if (dst.starts.empty()) dst.starts.push_back(0);
  for (int v : src.num) dst.num.push_back(v ? v + dst.nagr : 0);
  const int base = dst.starts.back();
  for (size_t a = 1; a < src.starts.size(); a++) dst.starts.push_back(base + src.starts[a]);
  for (int v : src.nodes) dst.nodes.push_back(v + member_off);
  dst.nagr += src.nagr;
}

// dst = diag(dst, src): src's rows after dst's rows, its columns after dst's columns
void append_block(Csr &dst, const Csr &src) {
  if (dst.ptr.empty()) dst.ptr.push_back(0);
  const int64_t base = dst.ptr.back();
  for (int r = 0; r < src.nrows; r++) dst.ptr.push_back(base + src.ptr[(size_t)r + 1]);
  for (int c : src.col) dst.col.push_back(c + dst.ncols);
  dst.val.insert(dst.val.end(), src.val.begin(), src.val.end());
  dst.nrows += src.nrows;
  dst.ncols += src.ncols;
}

}  // namespace

bool build_setup_systems(const Controls &c, const std::vector<int64_t> &sys_row,
                         const std::vector<int64_t> &sys_tri, const std::vector<int> &ii,
                         const std::vector<int> &jj, const std::vector<double> &vv, SetupResult &out,
                         std::string &err) {
  const int K = (int)sys_row.size() - 1;
  std::vector<SetupResult> S((size_t)K);
  std::vector<std::string> errs((size_t)K);
  std::vector<char> ok((size_t)K, 0);
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int k; (k = next.fetch_add(1)) < K;) {
      const int64_t t0 = sys_tri[(size_t)k], t1 = sys_tri[(size_t)k + 1];
      const int r0 = (int)sys_row[(size_t)k];
      std::vector<int> li((size_t)(t1 - t0)), lj((size_t)(t1 - t0));
      std::vector<double> lv(vv.begin() + t0, vv.begin() + t1);
      for (int64_t q = t0; q < t1; q++) {
        li[(size_t)(q - t0)] = ii[(size_t)q] - r0;
        lj[(size_t)(q - t0)] = jj[(size_t)q] - r0;
      }
      ok[(size_t)k] = build_setup(c, (int)(sys_row[(size_t)k + 1] - r0), li, lj, lv, nullptr, 0, S[(size_t)k],
                                  errs[(size_t)k]);
    }
  };
  const int nth = std::max(1, std::min(K, (int)std::thread::hardware_concurrency()));
  std::vector<std::thread> pool;
  for (int t = 1; t < nth; t++) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  for (int k = 0; k < K; k++)
    if (!ok[(size_t)k]) {
      err = "system " + std::to_string(k + 1) + ": " + errs[(size_t)k];
      return false;
    }
  out = SetupResult();
  out.n = (int)sys_row[(size_t)K];
  const SetupResult &S0 = S[0];
  out.overlap = S0.overlap; out.smoothers = S0.smoothers; out.levels = S0.levels;
  out.strong1 = S0.strong1; out.strong2 = S0.strong2;
  out.r1 = S0.r1; out.r2 = S0.r2; out.min1 = S0.min1; out.max1 = S0.max1; out.min2 = S0.min2; out.max2 = S0.max2;
  out.sd_ptr.assign(1, 0);
  for (int k = 0; k < K; k++) {
    const SetupResult &Sk = S[(size_t)k];
    const int row_off = (int)sys_row[(size_t)k];
    const int agg_off = out.fine.nagr, cagg_off = out.AC.nrows;
    append_aggregates(out.fine, Sk.fine, row_off);
    append_aggregates(out.fine_full, Sk.fine_full, row_off);
    append_aggregates(out.coarse, Sk.coarse, agg_off);
    append_aggregates(out.coarse_full, Sk.coarse_full, agg_off);
    for (size_t q = 0; q < Sk.R_i.size(); q++) {
      out.R_i.push_back(Sk.R_i[q] + agg_off); out.R_j.push_back(Sk.R_j[q] + row_off);
      out.R_v.push_back(Sk.R_v[q]);
    }
    for (size_t q = 0; q < Sk.AC_i.size(); q++) {
      out.AC_i.push_back(Sk.AC_i[q] + cagg_off); out.AC_j.push_back(Sk.AC_j[q] + cagg_off);
      out.AC_v.push_back(Sk.AC_v[q]);
    }
    append_block(out.A, Sk.A);
    append_block(out.R, Sk.R);
    append_block(out.P, Sk.P);
    append_block(out.AC, Sk.AC);
    const int64_t sbase = out.sd_ptr.back();
    for (size_t q = 1; q < Sk.sd_ptr.size(); q++) out.sd_ptr.push_back(sbase + Sk.sd_ptr[q]);
    for (int v : Sk.sd_nodes) out.sd_nodes.push_back(v + row_off);
  }
  return true;
}

}  // namespace dg
