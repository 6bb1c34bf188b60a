// Setup of doug_geom on one process (src/main/geom.F90:62-116): no
// aggregation; the subdomains are all nodes (Partitionings_full_InitCoarse,
// Partitioning_full.F90:32-47) or an imported partition, grown by the
// overlap layers; with elemental input and levels 2 the coarse level is the
// geometric coarse grid of CoarsePreconditioner_geometric_Init
// (CoarsePreconditioner_geometric.F90:34-115):
//   CreateCoarse      coarse/geom/CreateCoarse.f90   box grid over the used
//                     nodes, refined by a max-heap of node counts (BHeap.f90)
//   SendCoarse        coarse/geom/TransmitCoarse.F90:574-799, the master's own
//                     part: the local grid in the order the local freedoms
//                     reach its elements
//   CreateRestrict    coarse/geom/CreateRestrict.F90, GeomInterp.f90:
//                     multilinear interpolation through the refinement path
//                     (interpolation_type 1), inverse distance (2), the
//                     reference's kriging values (3)
//   CleanCoarse       CoarseAllgathers.F90:331-507: unused coarse freedoms out
//   CoarseMtxBuild    CoarseMtx.F90:476-516: AC = R A R^T
// The arithmetic follows the reference operation by operation (no FMA
// contraction), so R and AC are bit-equal to the C restatement used as the
// test oracle.  Indices of nodes, elements and refinements are 1-based as in
// the reference; slot 0 of those arrays is unused.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "setup.hpp"

namespace dg {

namespace {

constexpr double kEps = 1.0e-9;  // globals.F90:41

struct GridElem {          // CoarseGridElem
  int nfs = 0, nref = 0, rbeg = -1, lbeg = 0;
  int n[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};
struct Refinement {        // RefinedElem (no hanging nodes)
  int level = 0, node = 0, next = -1, parent = 0, lbeg = 0, lend = -1;
};
struct Grid {
  int nsd = 0, ncti = 0, nct = 0, elnum = 0, refnum = 0, nlfc = 0, mlvl = 1;
  int nc[3] = {0, 0, 0};
  double h0[3] = {0, 0, 0}, minvg[3] = {0, 0, 0};
  std::vector<double> xyz;          // node v at [(v-1)*nsd]
  std::vector<GridElem> els;        // [1..elnum]
  std::vector<Refinement> refs;     // [1..refnum]
  std::vector<int> elmap;           // [1..] fine nodes
  const double *at(int v) const { return xyz.data() + (size_t)(v - 1) * nsd; }
  double *at(int v) { return xyz.data() + (size_t)(v - 1) * nsd; }
};

// BHeap.f90: max-heap keyed by count; a lone last left child is never
// compared in heapify, as in the reference
class CountHeap {
 public:
  explicit CountHeap(int cap) : cap_(cap), by_((size_t)cap + 1), ind_((size_t)cap + 1) {}
  void insert(int val, int ind) {
    if (size_ >= cap_) return;
    int cur = ++size_;
    for (; cur > 1 && by_[(size_t)cur / 2] < val; cur /= 2) {
      by_[(size_t)cur] = by_[(size_t)cur / 2];
      ind_[(size_t)cur] = ind_[(size_t)cur / 2];
    }
    by_[(size_t)cur] = val;
    ind_[(size_t)cur] = ind;
  }
  int top_value() const { return by_[1]; }
  int top_index() const { return ind_[1]; }
  void pop() {
    if (size_ < 1) return;
    by_[1] = by_[(size_t)size_];
    ind_[1] = ind_[(size_t)size_];
    size_--;
    sift(1);
  }

 private:
  void sift(int cur) {
    const int val = by_[(size_t)cur], ind = ind_[(size_t)cur];
    int best = cur;
    for (;;) {
      const int l = 2 * cur, r = l + 1;
      if (r <= size_) {
        if (by_[(size_t)best] < by_[(size_t)l]) best = l;
        if (by_[(size_t)best] < by_[(size_t)r]) best = r;
      } else if (l < size_) {
        if (by_[(size_t)best] < by_[(size_t)l]) best = l;
      }
      if (best == cur) break;
      by_[(size_t)cur] = by_[(size_t)best];
      ind_[(size_t)cur] = ind_[(size_t)best];
      cur = best;
      by_[(size_t)cur] = val;
    }
    ind_[(size_t)cur] = ind;
  }
  int cap_, size_ = 0;
  std::vector<int> by_, ind_;
};

// getDir (CoarseGrid.F90:498-509): 1 + (x<c) + 2 (y<c) + 4 (z<c)
int direction(const double *x, const double *c, int nsd) {
  int n = 1;
  if (x[0] - c[0] < 0) n += 1;
  if (x[1] - c[1] < 0) n += 2;
  if (nsd == 3 && x[2] - c[2] < 0) n += 4;
  return n;
}

struct Mesh {
  int nsd;
  const double *xyz;  // fine node v (1-based) at [(v-1)*nsd]
  const double *at(int v) const { return xyz + (size_t)(v - 1) * nsd; }
};

// ChooseGeometricCenter / ChooseMeanCenter with meanpow 1 (CreateCoarse.f90)
void choose_center(int type, double *pt, const Mesh &M, const std::vector<int> &elmap, int lo, int hi,
                   const double *mn, const double *mx) {
  const int nsd = M.nsd;
  if (type == 1) {
    for (int d = 0; d < nsd; d++) pt[d] = (mx[d] + mn[d]) / 2.0;
    return;
  }
  for (int d = 0; d < nsd; d++) pt[d] = 0.0;
  for (int i = lo; i <= hi; i++)
    for (int d = 0; d < nsd; d++) pt[d] = pt[d] + M.at(elmap[(size_t)i])[d];
  for (int d = 0; d < nsd; d++) pt[d] = pt[d] / (double)(hi - lo + 1);
  for (int d = 0; d < nsd; d++) {
    const double b = 0.25 * (mx[d] - mn[d]);
    if (pt[d] > mx[d] - b) pt[d] = mx[d] - b;
    else if (pt[d] < mn[d] + b) pt[d] = mn[d] + b;
  }
}

// getRefBounds (CoarseGrid.F90:427-473)
void refinement_bounds(const Grid &C, int refi, double *mn, double *mx) {
  bool lo_set[3] = {false, false, false}, hi_set[3] = {false, false, false};
  const Refinement *r = &C.refs[(size_t)refi];
  for (int k = 0; k < C.nsd; k++) mn[k] = mx[k] = C.at(r->node)[k];
  while (r->parent > 0) {
    r = &C.refs[(size_t)r->parent];
    const double *ct = C.at(r->node);
    for (int k = 0; k < C.nsd; k++) {
      if (!hi_set[k] && ct[k] > mx[k]) { mx[k] = ct[k]; hi_set[k] = true; }
      else if (!lo_set[k] && ct[k] <= mn[k]) { mn[k] = ct[k]; lo_set[k] = true; }
    }
  }
  const GridElem &el = C.els[(size_t)(-r->parent)];
  for (int i = 0; i < (1 << C.nsd); i++) {
    const double *p = C.at(el.n[i]);
    for (int k = 0; k < C.nsd; k++) {
      if (!lo_set[k] && p[k] < mn[k]) { mn[k] = p[k]; lo_set[k] = true; }
      else if (!hi_set[k] && p[k] > mx[k]) { mx[k] = p[k]; hi_set[k] = true; }
    }
  }
}

// CreateCoarseMesh + CreateCoarseFreemap (CreateCoarse.f90): one coarse
// freedom per coarse node
Grid create_grid(const Mesh &M, int nnode, const std::vector<char> &inuse, int maxcie, int maxnd, int cutbal,
                 int ctype) {
  Grid C;
  const int nsd = M.nsd, tn = 1 << nsd;
  C.nsd = nsd;
  double ln[3], mxg[3];
  for (int d = 0; d < nsd; d++) {
    bool first = true;
    double lo = 0, hi = 0;
    for (int v = 1; v <= nnode; v++)
      if (inuse[(size_t)v]) {
        const double x = M.at(v)[d];
        if (first || x < lo) lo = x;
        if (first || x > hi) hi = x;
        first = false;
      }
    C.minvg[d] = lo;
    mxg[d] = hi;
    ln[d] = mxg[d] - C.minvg[d];
    C.minvg[d] = C.minvg[d] - ln[d] * 0.005;
    mxg[d] = mxg[d] + ln[d] * 0.005;
    ln[d] = ln[d] * 1.01;
  }
  if (nsd == 2) {
    C.nc[0] = (int)std::round(std::pow((double)maxcie * (ln[0] / ln[1]), 0.5));
    C.nc[1] = (int)std::round(std::pow((double)maxcie * (ln[1] / ln[0]), 0.5));
  } else {
    for (int d = 0; d < 3; d++) {
      const double den = d == 0 ? ln[1] * ln[2] : d == 1 ? ln[0] * ln[2] : ln[0] * ln[1];
      C.nc[d] = (int)std::round(std::pow((double)maxcie * ln[d] * ln[d] / den, 0.33));
    }
  }
  C.elnum = 1;
  for (int d = 0; d < nsd; d++) {
    C.nc[d] = std::max(C.nc[d], 1);
    C.h0[d] = ln[d] / (double)C.nc[d];
    C.elnum *= C.nc[d];
  }
  C.ncti = 1;
  for (int d = 0; d < nsd; d++) C.ncti *= ++C.nc[d];
  const int refmax = std::max(maxnd - C.ncti, 0);
  C.nct = std::max(maxnd, C.ncti);
  C.xyz.assign((size_t)C.nct * nsd, 0.0);
  C.els.assign((size_t)C.elnum + 1, GridElem());
  C.refs.assign((size_t)refmax + 1, Refinement());
  C.elmap.assign((size_t)nnode + 1, 0);
  int v = 1;
  const int n0 = C.nc[0], n1 = C.nc[1], n2 = nsd == 3 ? C.nc[2] : 1;
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++)
      for (int k = 0; k < n2; k++, v++) {
        C.at(v)[0] = i * C.h0[0] + C.minvg[0];
        C.at(v)[1] = j * C.h0[1] + C.minvg[1];
        if (nsd == 3) C.at(v)[2] = k * C.h0[2] + C.minvg[2];
      }
  int el = 1;
  for (int i = 1; i < n0; i++)
    for (int j = 1; j < n1; j++)
      for (int k = 1; k < (nsd == 3 ? n2 : 2); k++, el++) {
        GridElem &E = C.els[(size_t)el];
        if (nsd == 2) {
          const int nb = (i - 1) * n1 + j;
          const int c2[4] = {nb, nb + 1, nb + n1, nb + n1 + 1};
          std::copy(c2, c2 + 4, E.n);
        } else {
          const int nb = ((i - 1) * n1 + (j - 1)) * n2 + k;
          const int c3[8] = {nb, nb + 1, nb + n2, nb + n2 + 1, nb + n2 * n1, nb + n2 * n1 + 1,
                             nb + n2 * (n1 + 1), nb + n2 * (n1 + 1) + 1};
          std::copy(c3, c3 + 8, E.n);
        }
      }
  // getelem (CoarseGrid.F90:403-424)
  auto elem_of = [&](const double *x) {
    double rx[3] = {0, 0, 0};
    for (int d = 0; d < nsd; d++) rx[d] = (x[d] - C.minvg[d]) / C.h0[d];
    int ind = (int)std::trunc(rx[0]);
    for (int d = 1; d < nsd; d++) ind = (int)((double)(ind * (C.nc[d] - 1)) + std::trunc(rx[d]));
    return ind + 1;
  };
  std::vector<int> owner((size_t)nnode + 1, 0);
  for (int u = 1; u <= nnode; u++)
    if (inuse[(size_t)u]) {
      owner[(size_t)u] = elem_of(M.at(u));
      if (owner[(size_t)u] < 1 || owner[(size_t)u] > C.elnum) throw std::runtime_error("fine node outside the coarse grid");
      C.els[(size_t)owner[(size_t)u]].nfs++;
    }
  C.els[1].lbeg = 1;
  for (int i = 2; i <= C.elnum; i++) C.els[(size_t)i].lbeg = C.els[(size_t)i - 1].lbeg + C.els[(size_t)i - 1].nfs;
  for (int u = 1; u <= nnode; u++)
    if (inuse[(size_t)u]) C.elmap[(size_t)C.els[(size_t)owner[(size_t)u]].lbeg++] = u;
  CountHeap heap(C.elnum + refmax);
  const double root = std::sqrt((double)nsd);
  C.els[1].lbeg = 1;
  for (int i = 1; i <= C.elnum; i++) {
    if (i > 1) C.els[(size_t)i].lbeg = C.els[(size_t)i - 1].lbeg + C.els[(size_t)i - 1].nfs;
    if (C.els[(size_t)i].nfs > 0) heap.insert((int)std::lround(root * C.els[(size_t)i].nfs), i);
  }
  C.mlvl = 1;
  int refpt = 1;
  const int last_node = C.nct;
  double pt[3], p2[3], mn[3], mx[3];
  while (C.ncti + refpt <= last_node) {
    const int top = heap.top_index(), pcnt = heap.top_value();
    heap.pop();
    if (pcnt <= 2 * cutbal) break;
    if (top <= C.elnum) {  // split an initial element at its centre
      GridElem &E = C.els[(size_t)top];
      Refinement &nw = C.refs[(size_t)refpt];
      nw.level = 1;
      nw.node = C.ncti + refpt;
      nw.parent = -top;
      nw.next = -1;
      nw.lbeg = E.lbeg;
      nw.lend = E.lbeg + E.nfs - 1;
      for (int d = 0; d < nsd; d++) { mn[d] = C.at(E.n[0])[d]; mx[d] = C.at(E.n[tn - 1])[d]; }
      choose_center(ctype, pt, M, C.elmap, nw.lbeg, nw.lend, mn, mx);
      std::copy(pt, pt + nsd, C.at(nw.node));
      E.rbeg = refpt;
      heap.insert(E.nfs, C.elnum + refpt);
      refpt++;
      continue;
    }
    // split off the fullest orthant of a refined element
    const int er = top - C.elnum;
    Refinement &cur = C.refs[(size_t)er];
    Refinement &nw = C.refs[(size_t)refpt];
    nw.level = cur.level + 1;
    nw.node = C.ncti + refpt;
    nw.parent = er;
    std::copy(C.at(cur.node), C.at(cur.node) + nsd, pt);
    refinement_bounds(C, er, mn, mx);
    int counts[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = cur.lbeg; i <= cur.lend; i++) counts[direction(M.at(C.elmap[(size_t)i]), pt, nsd)]++;
    int flag = 1;
    for (int i = 2; i <= tn; i++) if (counts[i] > counts[flag]) flag = i;
    const int cnt = counts[flag];
    if (cnt <= cutbal) break;
    // the orthant's nodes to the end of the range, two-sided swap scan
    int a = cur.lbeg, b = cur.lend;
    for (;;) {
      while (a <= b && direction(M.at(C.elmap[(size_t)a]), pt, nsd) != flag) a++;
      while (b >= a && direction(M.at(C.elmap[(size_t)b]), pt, nsd) == flag) b--;
      if (a >= b) break;
      std::swap(C.elmap[(size_t)a], C.elmap[(size_t)b]);
    }
    nw.lbeg = a;
    nw.lend = cur.lend;
    nw.next = cur.next;
    cur.next = refpt;
    cur.lend = a - 1;
    std::copy(M.at(C.elmap[(size_t)nw.lbeg]), M.at(C.elmap[(size_t)nw.lbeg]) + nsd, p2);
    for (int d = 0; d < nsd; d++) {  // adjustBounds (CoarseGrid.F90:477-491)
      if (pt[d] <= p2[d]) mn[d] = pt[d];
      else mx[d] = pt[d];
    }
    choose_center(ctype, pt, M, C.elmap, nw.lbeg, nw.lend, mn, mx);
    std::copy(pt, pt + nsd, C.at(nw.node));
    heap.insert(cnt, C.elnum + refpt);
    heap.insert(pcnt - cnt, C.elnum + er);
    C.mlvl = std::max(C.mlvl, nw.level);
    refpt++;
  }
  C.refnum = refpt - 1;
  C.refs.resize((size_t)C.refnum + 1);
  // grid nodes of empty elements go; refinement centres are numbered
  // element by element in list order
  std::vector<int> keep((size_t)C.ncti + 1, 0);
  for (int i = 1; i <= C.elnum; i++)
    if (C.els[(size_t)i].nfs != 0)
      for (int k = 0; k < tn; k++) keep[(size_t)C.els[(size_t)i].n[k]] = 1;
  int dropped = 0;
  for (int i = 1; i <= C.ncti; i++) dropped += keep[(size_t)i] == 0;
  const int nct = C.ncti - dropped + C.refnum;
  std::vector<double> nx((size_t)nct * nsd, 0.0);
  int kept = 0;
  for (int i = 1; i <= C.ncti; i++) {
    if (keep[(size_t)i]) {
      keep[(size_t)i] = ++kept;
      std::copy(C.at(i), C.at(i) + nsd, nx.begin() + (ptrdiff_t)(kept - 1) * nsd);
    } else {
      keep[(size_t)i] = kept;
    }
  }
  if (dropped > 0)
    for (int i = 1; i <= C.elnum; i++)
      for (int k = 0; k < tn; k++)
        C.els[(size_t)i].n[k] = C.els[(size_t)i].nfs > 0 ? keep[(size_t)C.els[(size_t)i].n[k]] : 0;
  C.ncti = kept;
  int next_node = C.ncti + 1;
  for (int i = 1; i <= C.elnum; i++) {
    const int first = next_node;
    for (int j = C.els[(size_t)i].rbeg; j != -1; j = C.refs[(size_t)j].next) {
      std::copy(C.at(C.refs[(size_t)j].node), C.at(C.refs[(size_t)j].node) + nsd,
                nx.begin() + (ptrdiff_t)(next_node - 1) * nsd);
      C.refs[(size_t)j].node = next_node++;
    }
    C.els[(size_t)i].nref = next_node - first;
  }
  C.xyz.swap(nx);
  C.nct = nct;
  C.nlfc = C.nct;
  return C;
}

// SendCoarse, the master's own part (TransmitCoarse.F90:574-799), one
// process.  node_of_local[l] (1-based l) = fine node of local freedom l.
Grid local_grid(const Grid &C, int nnode, const std::vector<int> &node_of_local, int nlf) {
  const int nsd = C.nsd, tn = 1 << nsd;
  std::vector<int> home((size_t)nnode + 1, 0);  // -element or refinement holding the node
  for (int el = 1; el <= C.elnum; el++) {
    const GridElem &E = C.els[(size_t)el];
    if (E.rbeg <= 0) {
      for (int j = E.lbeg; j < E.lbeg + E.nfs; j++) home[(size_t)C.elmap[(size_t)j]] = -el;
    } else {
      for (int r = E.rbeg; r > 0; r = C.refs[(size_t)r].next)
        for (int j = C.refs[(size_t)r].lbeg; j <= C.refs[(size_t)r].lend; j++) home[(size_t)C.elmap[(size_t)j]] = r;
    }
  }
  std::vector<char> refmark((size_t)C.refnum + 1, 0), elmark((size_t)C.elnum + 1, 0), present((size_t)nnode + 1, 0);
  std::vector<int> order;  // initial elements in the order the freedoms reach them
  Grid L;
  L.nsd = nsd;
  int lnnode = 0;
  for (int l = 1; l <= nlf; l++) {
    const int v = node_of_local[(size_t)l];
    if (v == 0 || home[(size_t)v] == 0) continue;
    if (!present[(size_t)v]) { present[(size_t)v] = 1; lnnode++; }
    int k = home[(size_t)v];
    while (k > 0 && !refmark[(size_t)k]) {
      refmark[(size_t)k] = 1;
      L.refnum++;
      k = C.refs[(size_t)k].parent;
    }
    if (k < 0 && !elmark[(size_t)-k]) { elmark[(size_t)-k] = 1; order.push_back(-k); }
  }
  L.elnum = (int)order.size();
  std::vector<int> g2l((size_t)C.nct + 1, 0), l2g(1, 0);
  for (int el : order)
    for (int j = 0; j < tn; j++) {
      const int g = C.els[(size_t)el].n[j];
      if (!g2l[(size_t)g]) { l2g.push_back(g); g2l[(size_t)g] = (int)l2g.size() - 1; }
    }
  L.ncti = (int)l2g.size() - 1;
  for (int el : order)
    for (int r = C.els[(size_t)el].rbeg; r != -1; r = C.refs[(size_t)r].next)
      if (refmark[(size_t)r]) { l2g.push_back(C.refs[(size_t)r].node); g2l[(size_t)C.refs[(size_t)r].node] = (int)l2g.size() - 1; }
  L.nct = L.ncti + L.refnum;
  L.nlfc = L.nct;
  L.mlvl = C.mlvl;
  L.xyz.resize((size_t)L.nct * nsd);
  for (int i = 1; i <= L.nct; i++) std::copy(C.at(l2g[(size_t)i]), C.at(l2g[(size_t)i]) + nsd, L.at(i));
  L.els.assign((size_t)L.elnum + 1, GridElem());
  L.refs.assign((size_t)L.refnum + 1, Refinement());
  L.elmap.assign((size_t)lnnode + 1, 0);
  int nd = 1, rel = 1;
  std::vector<int> path;  // most recent local refinement per level
  for (int f = 1; f <= L.elnum; f++) {
    const GridElem &E = C.els[(size_t)order[(size_t)f - 1]];
    GridElem &LE = L.els[(size_t)f];
    LE.nref = E.nref;
    for (int j = 0; j < tn; j++) LE.n[j] = g2l[(size_t)E.n[j]];
    LE.lbeg = nd;
    LE.nfs = 0;
    if (E.rbeg == -1) {
      LE.rbeg = -1;
      for (int j = E.lbeg; j < E.lbeg + E.nfs; j++)
        if (present[(size_t)C.elmap[(size_t)j]]) { LE.nfs++; L.elmap[(size_t)nd++] = C.elmap[(size_t)j]; }
      continue;
    }
    LE.rbeg = rel;
    path.assign(1, -f);
    int last = 0;
    for (int r = E.rbeg; r != -1; r = C.refs[(size_t)r].next) {
      if (!refmark[(size_t)r]) continue;
      const Refinement &old = C.refs[(size_t)r];
      Refinement &nr = L.refs[(size_t)rel];
      nr.level = old.level;
      nr.node = g2l[(size_t)old.node];
      if ((int)path.size() < nr.level) throw std::runtime_error("refinement list out of order");
      nr.parent = path[(size_t)nr.level - 1];
      nr.next = rel + 1;
      nr.lbeg = nd;
      for (int j = old.lbeg; j <= old.lend; j++)
        if (present[(size_t)C.elmap[(size_t)j]]) { LE.nfs++; L.elmap[(size_t)nd++] = C.elmap[(size_t)j]; }
      nr.lend = nd - 1;
      path.resize((size_t)nr.level + 1);
      path[(size_t)nr.level] = rel;
      last = rel++;
    }
    L.refs[(size_t)last].next = -1;
  }
  return L;
}

// BuildMults (GeomInterp.f90:472-560): polynomial coefficients (1, x, y,
// [z, yz, xz,] xy[, xyz]) of every coarse node over the box [mn, mx];
// coef(corner a, column c) at [(c-1)*tn + a-1], mult likewise
void build_mults(const double *mn, const double *mx, const double *coef, int csz, int nsd, double *mult, int ncols) {
  const int tn = 1 << nsd;
  std::fill(mult, mult + (size_t)tn * ncols, 0.0);
  double prd = 1.0;
  for (int d = 0; d < nsd; d++) prd = prd * (mx[d] - mn[d]);
  prd = 1.0 / prd;
  double m[8];
  for (int a = 1; a <= tn; a++) {
    if (nsd == 2) {
      const double X = (a == 2 || a == 4) ? mx[0] : mn[0], Y = (a >= 3) ? mx[1] : mn[1];
      const bool plus = a == 1 || a == 4;
      m[0] = plus ? X * Y : -(X * Y);
      m[1] = plus ? -Y : Y;
      m[2] = plus ? -X : X;
      m[3] = plus ? 1.0 : -1.0;
    } else {
      // corner a: bound of each factor (max where the corner bit is set),
      // and whether the factors enter negated (then the term sign is +)
      const bool negated = a == 1 || a == 4 || a == 6 || a == 7;
      double f[3];
      for (int d = 0; d < 3; d++) {
        const double b = (((a - 1) >> d) & 1) ? mx[d] : mn[d];
        f[d] = negated ? -b : b;
      }
      m[4] = f[0]; m[5] = f[1]; m[6] = f[2];
      m[0] = m[4] * m[5] * m[6];
      for (int d = 0; d < 3; d++) m[1 + d] = negated ? m[0] / m[4 + d] : -m[0] / m[4 + d];
      m[7] = negated ? 1.0 : -1.0;
    }
    for (int r = 0; r < tn; r++) m[r] = m[r] * prd;
    for (int c = 1; c <= csz; c++) {
      const double w = coef[(size_t)(c - 1) * tn + a - 1];
      double *mc = mult + (size_t)(c - 1) * tn;
      for (int r = 0; r < tn; r++) mc[r] = mc[r] + w * m[r];
    }
  }
}

// MlinInterpolate (GeomInterp.f90:563-582)
double interpolate(const double *p, int nsd, const double *m) {
  if (nsd == 2) return m[0] + m[1] * p[0] + m[2] * p[1] + m[3] * p[0] * p[1];
  return m[0] + m[1] * p[0] + m[2] * p[1] + m[3] * p[2] + m[4] * p[1] * p[2] + m[5] * p[0] * p[2] +
         m[6] * p[0] * p[1] + m[7] * p[0] * p[1] * p[2];
}

// CalcNextCoefs (GeomInterp.f90:244-468), no hanging nodes: the corner
// coefficients of the sub-box of [mn, mx] cut at the centre ct towards pt.
// The reference weighs the 2-D edge corners drev-rev(i) and the 3-D face
// centres with the multipliers as written there (exact for box centres,
// where every multiplier is 1/2).
void next_coefs(const double *ct, int ci, const double *mn, const double *mx, const double *coef, const int *cind,
                int csz, int nsd, const double *pt, double *out, int *oind, int &osz) {
  const int tn = 1 << nsd;
  auto CF = [&](int a, int c) { return coef[(size_t)(c - 1) * tn + a - 1]; };
  auto CO = [&](int a, int c) -> double & { return out[(size_t)(c - 1) * tn + a - 1]; };
  double m[3];
  for (int d = 0; d < nsd; d++) m[d] = (mx[d] - ct[d]) / (mx[d] - mn[d]);
  osz = csz;
  std::copy(cind, cind + csz, oind);
  int dir = 1, drev = 1, rev[3] = {0, 0, 0};
  for (int d = 0, k = 1; d < nsd; d++, k *= 2) {
    if (pt[d] < ct[d]) { dir += k; rev[d] = -k; }
    else { drev += k; rev[d] = k; }
  }
  for (int c = 1; c <= csz; c++) { CO(dir, c) = CF(dir, c); CO(drev, c) = 0.0; }
  if (nsd == 2) {
    for (int d = 0; d < 2; d++) {
      const int a = drev - rev[d];
      for (int c = 1; c <= csz; c++)
        CO(a, c) = rev[d] > 0 ? m[d] * CF(a, c) + (1 - m[d]) * CF(dir, c) : m[d] * CF(dir, c) + (1 - m[d]) * CF(a, c);
    }
  } else {
    for (int d = 0; d < 3; d++) {
      const int a = dir + rev[d];
      for (int c = 1; c <= csz; c++)
        CO(a, c) = rev[d] > 0 ? m[d] * CF(a, c) + (1 - m[d]) * CF(dir, c) : m[d] * CF(dir, c) + (1 - m[d]) * CF(a, c);
    }
    // face centre across direction d: bilinear in the two other directions
    // (u, w) with corner offsets su, sw from the first corner on that face
    const int U[3] = {1, 0, 0}, W[3] = {2, 2, 1}, SU[3] = {2, 1, 1}, SW[3] = {4, 4, 2};
    for (int d = 0; d < 3; d++) {
      const int a = drev - rev[d], k0 = std::max(0, -rev[d]) + 1;
      const double p = m[U[d]], q = m[W[d]];
      for (int c = 1; c <= csz; c++)
        CO(a, c) = p * q * CF(k0, c) + p * (1 - q) * CF(k0 + SW[d], c) + (1 - p) * q * CF(k0 + SU[d], c) +
                   (1 - p) * (1 - q) * CF(k0 + SU[d] + SW[d], c);
    }
  }
  // the new centre takes a column whose coefficients all vanished, else the
  // last column closes the gap; a centre left over is appended
  int pending = 1;
  for (int c = csz; c >= 1; c--) {
    bool zero = true;
    for (int a = 1; a <= tn && zero; a++) zero = CO(a, c) == 0.0;
    if (!zero) continue;
    if (pending > 0) {
      CO(drev, c) = 1.0;
      oind[c - 1] = ci;
      pending--;
    } else {
      for (int a = 1; a <= tn; a++) CO(a, c) = CO(a, osz);
      oind[c - 1] = oind[osz - 1];
      osz--;
    }
  }
  if (pending > 0) {
    osz++;
    for (int a = 1; a <= tn; a++) CO(a, osz) = 0.0;
    CO(drev, osz) = 1.0;
    oind[osz - 1] = ci;
  }
}

struct Entry { int fine, coarse; double v; };

// CalcMlinearInterp (GeomInterp.f90:585-825): (fine node, coarse node,
// value), node after node in element and list order
void multilinear(const Grid &C, const Mesh &M, std::vector<Entry> &np) {
  const int nsd = C.nsd, tn = 1 << nsd, L = C.mlvl, maxc = tn + L + nsd;
  std::vector<double> lo((size_t)nsd * (L + 2)), hi((size_t)nsd * (L + 2));
  std::vector<double> coefs((size_t)tn * maxc * (L + 1)), cur((size_t)tn * maxc * 9), fin((size_t)tn * maxc * 9);
  std::vector<double> mult((size_t)tn * maxc);
  std::vector<int> cinds((size_t)maxc * (L + 1)), cszs((size_t)L + 2), curi((size_t)maxc * 9);
  int cursz[9];
  auto LO = [&](int lv) { return lo.data() + (size_t)lv * nsd; };
  auto HI = [&](int lv) { return hi.data() + (size_t)lv * nsd; };
  auto COEF = [&](int lv) { return coefs.data() + (size_t)lv * tn * maxc; };
  auto CIND = [&](int lv) { return cinds.data() + (size_t)lv * maxc; };
  auto sub_bounds = [&](const double *ct, const double *pt, int lv) {
    for (int d = 0; d < nsd; d++) {
      if (ct[d] <= pt[d]) { LO(lv + 1)[d] = ct[d]; HI(lv + 1)[d] = HI(lv)[d]; }
      else { LO(lv + 1)[d] = LO(lv)[d]; HI(lv + 1)[d] = ct[d]; }
    }
  };
  // initial box: corner a (getDir order) is the coarse node in column col[a]
  static const int col2[4] = {4, 2, 3, 1}, col3[8] = {8, 4, 6, 2, 7, 3, 5, 1};
  for (int e = 1; e <= C.elnum; e++) {
    const GridElem &E = C.els[(size_t)e];
    std::copy(C.at(E.n[0]), C.at(E.n[0]) + nsd, LO(1));
    std::copy(C.at(E.n[tn - 1]), C.at(E.n[tn - 1]) + nsd, HI(1));
    cszs[1] = tn;
    std::copy(E.n, E.n + tn, CIND(1));
    std::fill(COEF(1), COEF(1) + (size_t)tn * tn, 0.0);
    for (int a = 0; a < tn; a++) COEF(1)[(size_t)((nsd == 2 ? col2[a] : col3[a]) - 1) * tn + a] = 1.0;
    if (E.rbeg == -1) {
      build_mults(LO(1), HI(1), COEF(1), cszs[1], nsd, mult.data(), maxc);
      for (int j = E.lbeg; j < E.lbeg + E.nfs; j++) {
        const int pn = C.elmap[(size_t)j];
        for (int c = 1; c <= cszs[1]; c++)
          np.push_back({pn, CIND(1)[c - 1], interpolate(M.at(pn), nsd, mult.data() + (size_t)(c - 1) * tn)});
      }
      continue;
    }
    for (int r = E.rbeg; r != -1; r = C.refs[(size_t)r].next) {
      const Refinement &R = C.refs[(size_t)r];
      if (R.parent > 0) {
        const int ci = C.refs[(size_t)R.parent].node, lv = R.level - 1;
        const double *ct = C.at(ci), *pt = C.at(R.node);
        next_coefs(ct, ci, LO(lv), HI(lv), COEF(lv), CIND(lv), cszs[(size_t)lv], nsd, pt, COEF(lv + 1), CIND(lv + 1),
                   cszs[(size_t)lv + 1]);
        sub_bounds(ct, pt, lv);
      }
      if (R.lbeg > R.lend) continue;
      const int ci = R.node, lv = R.level;
      const double *ct = C.at(ci);
      bool have[9] = {false, false, false, false, false, false, false, false, false};
      for (int k = R.lbeg; k <= R.lend; k++) {
        const int pn = C.elmap[(size_t)k];
        const double *pt = M.at(pn);
        const int d = direction(pt, ct, nsd);
        double *cc = cur.data() + (size_t)d * tn * maxc, *ff = fin.data() + (size_t)d * tn * maxc;
        int *ii = curi.data() + (size_t)d * maxc;
        if (!have[d]) {
          next_coefs(ct, ci, LO(lv), HI(lv), COEF(lv), CIND(lv), cszs[(size_t)lv], nsd, pt, cc, ii, cursz[d]);
          sub_bounds(ct, pt, lv);
          build_mults(LO(lv + 1), HI(lv + 1), cc, cursz[d], nsd, ff, maxc);
          have[d] = true;
        }
        for (int c = 1; c <= cursz[d]; c++) np.push_back({pn, ii[c - 1], interpolate(pt, nsd, ff + (size_t)(c - 1) * tn)});
      }
    }
  }
}

// CreatePathRestrict's values (CreateRestrict.F90:95-213, 219-276): every
// node against its element's corners and the centres on its refinement
// path; type 2 inverse distance, type 3 the distances (the reference's
// kriging values).  Rows by fine node number.
void path_weights(const Grid &C, const Mesh &M, int nnode, int type, std::vector<Entry> &np) {
  const int nsd = C.nsd, tn = 1 << nsd;
  std::vector<int> start((size_t)nnode + 2, 0);
  for (int e = 1; e <= C.elnum; e++)
    if (C.els[(size_t)e].rbeg == -1)
      for (int j = C.els[(size_t)e].lbeg; j < C.els[(size_t)e].lbeg + C.els[(size_t)e].nfs; j++)
        start[(size_t)C.elmap[(size_t)j] + 1] = tn;
  for (int r = 1; r <= C.refnum; r++)
    for (int j = C.refs[(size_t)r].lbeg; j <= C.refs[(size_t)r].lend; j++)
      start[(size_t)C.elmap[(size_t)j] + 1] = tn + C.refs[(size_t)r].level;
  start[1] = 1;
  for (int v = 1; v <= nnode; v++) start[(size_t)v + 1] += start[(size_t)v];
  np.assign((size_t)start[(size_t)nnode + 1] - 1, Entry{0, 0, 0.0});
  std::vector<const double *> pts((size_t)tn + C.mlvl + 1);
  std::vector<int> pid((size_t)tn + C.mlvl + 1);
  std::vector<double> w((size_t)tn + C.mlvl + 1);
  auto weigh = [&](int lo, int hi, int csz) {
    for (int j = lo; j <= hi; j++) {
      const int pn = C.elmap[(size_t)j];
      const double *x = M.at(pn);
      for (int q = 1; q <= csz; q++) {
        double s = 0.0;
        for (int d = 0; d < nsd; d++) {
          const double t = pts[(size_t)q][d] - x[d];
          s = s + t * t;
        }
        w[(size_t)q] = std::pow(s, 0.5);
      }
      if (type == 2) {
        for (int q = 1; q <= csz; q++) {
          if (w[(size_t)q] <= kEps) {
            std::fill(w.begin() + 1, w.begin() + csz + 1, 0.0);
            w[(size_t)q] = 1.0;
            break;
          }
          w[(size_t)q] = 1.0 / w[(size_t)q];
        }
        double sum = 0.0;
        for (int q = 1; q <= csz; q++) sum = sum + w[(size_t)q];
        for (int q = 1; q <= csz; q++) w[(size_t)q] = w[(size_t)q] / sum;
      }
      for (int q = 1; q <= csz; q++) np[(size_t)(start[(size_t)pn] + q - 2)] = {pn, pid[(size_t)q], w[(size_t)q]};
    }
  };
  for (int e = 1; e <= C.elnum; e++) {
    const GridElem &E = C.els[(size_t)e];
    for (int a = 0; a < tn; a++) { pts[(size_t)a + 1] = C.at(E.n[a]); pid[(size_t)a + 1] = E.n[a]; }
    if (E.rbeg == -1) {
      weigh(E.lbeg, E.lbeg + E.nfs - 1, tn);
      continue;
    }
    for (int r = E.rbeg; r != -1; r = C.refs[(size_t)r].next) {
      const Refinement &R = C.refs[(size_t)r];
      const int csz = tn + R.level;
      pts[(size_t)csz] = C.at(R.node);
      pid[(size_t)csz] = R.node;
      weigh(R.lbeg, R.lend, csz);
    }
  }
}

}  // namespace

bool geometric_restriction(const Controls &c, const std::vector<int> &efree, const NodeGeometry &G,
                           const std::vector<int> &lg_fmap, Coo &R, std::vector<double> &coarse_xyz,
                           std::string &err) {
  const int nsd = G.nsd, nnode = G.nnode;
  if (nsd != 2 && nsd != 3) { err = "the geometric coarse grid needs 2-D or 3-D node coordinates"; return false; }
  if (c.hanging_nodes) { err = "hanging_nodes: not supported by the geometric coarse grid here"; return false; }
  const int maxcie = c.maxcie == -1 ? 75 : c.maxcie, maxnd = c.maxnd == -1 ? 500 : c.maxnd;
  const int cutbal = c.cutbal <= 0 ? 1 : c.cutbal, ctype = c.center_type == -1 ? 1 : c.center_type;
  const int itype = c.interpolation_type == -1 ? 1 : c.interpolation_type;
  if (ctype != 1 && ctype != 2) { err = "center_type " + std::to_string(ctype) + ": box (1) and mean (2) centres are supported"; return false; }
  if (itype < 1 || itype > 3) { err = "interpolation_type " + std::to_string(itype) + ": 1, 2 or 3"; return false; }
  if ((int64_t)G.coords.size() < (int64_t)nsd * nnode) { err = "node coordinates: too few values"; return false; }
  const Mesh M{nsd, G.coords.data()};
  // nodes of the freedoms of the elements of this process (all elements)
  std::vector<char> inuse((size_t)nnode + 1, 0);
  for (int f : efree) {
    if (f < 1 || f > (int)G.freemap.size()) { err = "freedom " + std::to_string(f) + " has no node in the freemap"; return false; }
    const int v = G.freemap[(size_t)f - 1];
    if (v < 1 || v > nnode) { err = "freemap: node " + std::to_string(v) + " out of range"; return false; }
    inuse[(size_t)v] = 1;
  }
  const int nlf = (int)lg_fmap.size();
  std::vector<int> node_of_local((size_t)nlf + 1, 0);
  for (int l = 0; l < nlf; l++) node_of_local[(size_t)l + 1] = G.freemap[(size_t)lg_fmap[(size_t)l] - 1];
  try {
    Grid C = create_grid(M, nnode, inuse, maxcie, maxnd, cutbal, ctype);
    Grid L = local_grid(C, nnode, node_of_local, nlf);
    std::vector<Entry> np;
    std::vector<int64_t> lo((size_t)nnode + 1, 0), hi((size_t)nnode + 1, -1);
    if (itype == 1) {
      multilinear(L, M, np);
      // the entries of a node are consecutive (GeomInterp.f90:178-190)
      for (size_t k = 0; k < np.size(); k++) {
        const int v = np[k].fine;
        if (k == 0 || np[k - 1].fine != v) {
          if (hi[(size_t)v] >= 0) { err = "Node restriction matrix not consolidated"; return false; }
          lo[(size_t)v] = (int64_t)k;
        }
        hi[(size_t)v] = (int64_t)k;
      }
    } else {
      path_weights(L, M, nnode, itype, np);
      for (size_t k = 0; k < np.size(); k++) {
        const int v = np[k].fine;
        if (hi[(size_t)v] < 0) lo[(size_t)v] = (int64_t)k;
        hi[(size_t)v] = (int64_t)k;
      }
    }
    // R: coarse freedom x local fine freedom, column after column, values
    // above eps (GeomInterp.f90:192-214); then CleanCoarse renumbers the
    // coarse freedoms that R uses, in order
    Coo Rb;
    for (int l = 1; l <= nlf; l++) {
      const int v = node_of_local[(size_t)l];
      if (v == 0) continue;
      for (int64_t k = lo[(size_t)v]; k <= hi[(size_t)v]; k++)
        if (np[(size_t)k].v > kEps) { Rb.i.push_back(np[(size_t)k].coarse); Rb.j.push_back(l - 1); Rb.v.push_back(np[(size_t)k].v); }
    }
    std::vector<int> used((size_t)L.nlfc + 1, 0);
    for (int a : Rb.i) used[(size_t)a] = 1;
    int nk = 0;
    for (int a = 1; a <= L.nlfc; a++) used[(size_t)a] = used[(size_t)a] ? ++nk : 0;
    R = Coo();
    R.nrows = nk;
    R.ncols = nlf;
    R.i.resize(Rb.i.size());
    for (size_t k = 0; k < Rb.i.size(); k++) R.i[k] = used[(size_t)Rb.i[k]] - 1;
    R.j = std::move(Rb.j);
    R.v = std::move(Rb.v);
    coarse_xyz.assign((size_t)nk * nsd, 0.0);
    for (int a = 1; a <= L.nlfc; a++)
      if (used[(size_t)a]) std::copy(L.at(a), L.at(a) + nsd, coarse_xyz.begin() + (ptrdiff_t)(used[(size_t)a] - 1) * nsd);
  } catch (const std::exception &e) {
    err = e.what();
    return false;
  }
  return true;
}

std::vector<int> independent_coarse(const Csr &AC) {
  const int nc = AC.nrows;
  std::vector<int> keep((size_t)nc, 0);
  if (nc > 4000) {
    for (int i = 0; i < nc; i++) keep[(size_t)i] = i + 1;
    return keep;
  }
  std::vector<double> a((size_t)nc * nc, 0.0);
  for (int r = 0; r < nc; r++)
    for (int64_t k = AC.ptr[(size_t)r]; k < AC.ptr[(size_t)r + 1]; k++)
      a[(size_t)r * nc + AC.col[(size_t)k]] = a[(size_t)r * nc + AC.col[(size_t)k]] + AC.val[(size_t)k];
  int nk = 0;
  for (int j = 0; j < nc; j++) {
    double *rj = a.data() + (size_t)j * nc;
    double d = rj[j];
    const double d0 = d;
    for (int k = 0; k < j; k++) if (keep[(size_t)k]) d = d - rj[k] * rj[k];
    if (!(d > 1.0e-10 * d0)) {
      for (int i = j; i < nc; i++) a[(size_t)i * nc + j] = 0.0;
      continue;
    }
    keep[(size_t)j] = ++nk;
    const double l = std::sqrt(d);
    rj[j] = l;
    for (int i = j + 1; i < nc; i++) {
      double *ri = a.data() + (size_t)i * nc;
      double t = ri[j];
      for (int k = 0; k < j; k++) if (keep[(size_t)k]) t = t - ri[k] * rj[k];
      ri[j] = t / l;
    }
  }
  return keep;
}

}  // namespace dg
