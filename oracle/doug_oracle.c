/*
 * doug_oracle.c -- CPU restatement of DOUG's solve path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
 * baseline of the benchmark use this file as the checker.  The product
 * (doug_gb300/) never links, loads or calls it.
 *
 * Every routine below cites the reference routine it restates
 * (file:line relative to the DOUG source tree).  Arrays are 1-based (element
 * 0 unused) so that each loop maps one-to-one onto the Fortran it follows.
 * Compile with -ffp-contract=off: the reference arithmetic is evaluated in
 * source order without fused multiply-adds, and the aggregation of the coarse
 * level depends on the exact bits of the Galerkin product.
 *
 * Parity pin: tests/test_oracle.py checks the solutions of the reference
 * fixtures tests/assembled/lap4x4 and tests/assembled/lap16x16.
 */
#include "doug_oracle.h"
#include "spchol.h"

#include <ctype.h>
#include <limits.h>
#include <math.h>
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* error handling: DOUG_abort (DOUG_utils.F90:254-286) becomes a longjmp */
/* back to the API entry, which returns a negative status.              */
/* ------------------------------------------------------------------ */
static jmp_buf g_jmp;
static char g_err[512];

static void orc_abort(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  longjmp(g_jmp, 1);
}

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) orc_abort("out of memory (%zu x %zu)", n, sz);
  return p;
}
#define NEWI(n) ((int *)xcalloc((size_t)(n) + 1, sizeof(int)))
#define NEWD(n) ((double *)xcalloc((size_t)(n) + 1, sizeof(double)))
#define NEWB(n) ((char *)xcalloc((size_t)(n) + 1, 1))

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* parameters.F90:99-102 */
#define D_MAXINT 2147483647
#define D_AGGREGATED D_MAXINT
#define D_PENDING (D_MAXINT / 2)

enum { ARR_NO = 0, ARR_ROWS = 1, ARR_COLS = 2 };
enum { SCALE_UNDEF = -1, SCALE_NO = 0, SCALE_DIAG = 1 };

/* ------------------------------------------------------------------ */
/* control data: globals.F90:85-154, controls.F90:159-246               */
/* ------------------------------------------------------------------ */
typedef struct {
  int solver, method, fine_method, num_iters, coarse_method, num_subdomains,
      levels, overlap, smoothers, input_type, grid_size, matrix_type,
      initial_guess, number_of_blocks, radius1, radius2, minasize1, minasize2,
      maxasize1, maxasize2, debug, verbose, plotting;
  double strong1, strong2, solve_tolerance;
  int solve_maxiters;
  int symmstruct, symmnumeric;
  int interpolation_type;
  int maxcie, maxnd, cutbal, center_type, hanging_nodes;
  int executable; /* extension word: -1/0 doug_aggr, 1 doug_geom */
  double omega;   /* extension word: prolongator smoother weight (the reference's 1/3 when unset) */
  /* master data */
  char assembled_mtx_file[300];
  int assembled_mtx_format;
  char assembled_rhs_file[300];
  int assembled_rhs_format;
  char solution_file[300];
  int solution_format;
  int start_vec_type;
  char info_file[300], freedom_lists_file[300], elemmat_rhs_file[300];
  char coords_file[300], freemap_file[300];
} ctl_t;

static void ctl_defaults(ctl_t *c) {
  memset(c, 0, sizeof *c);
  c->solver = c->method = c->fine_method = c->num_iters = c->coarse_method = -1;
  c->num_subdomains = c->levels = c->overlap = c->smoothers = -1;
  c->input_type = c->grid_size = c->matrix_type = c->initial_guess = -1;
  c->number_of_blocks = c->radius1 = c->radius2 = c->minasize1 = -1;
  c->minasize2 = c->maxasize1 = c->maxasize2 = c->debug = c->verbose = -1;
  c->plotting = -1;
  c->strong1 = c->strong2 = c->solve_tolerance = -1.0;
  c->solve_maxiters = -1;
  c->interpolation_type = -1;
  c->maxcie = c->maxnd = c->cutbal = c->center_type = -1;
  c->hanging_nodes = 0;
  c->executable = -1;
  c->omega = -1.0;
  c->assembled_mtx_format = -1;
  c->assembled_rhs_format = -1;
  c->solution_format = -1;
  c->start_vec_type = -1;
}

/* Fortran internal READ with edit descriptor I10: the first 10 characters,
 * blanks ignored (BLANK='NULL'), optional sign. DOUG_utils.F90:731ff. */
int orc_parse_i10(const char *s, int *out) {
  char buf[11];
  int k = 0, i;
  for (i = 0; i < 10 && s[i]; i++)
    if (s[i] != ' ') buf[k++] = s[i];
  buf[k] = 0;
  if (k == 0) { *out = 0; return 0; }
  char *end;
  long v = strtol(buf, &end, 10);
  if (*end) return -1;
  *out = (int)v;
  return 0;
}

/* Fortran internal READ with F10.5: first 10 characters, blanks ignored;
 * without a decimal point the digits carry 5 implied decimals
 * (so "8" reads as 8e-5). Used for strong1/strong2/solve_tolerance
 * (DOUG_utils.F90:914-936). */
int orc_parse_f10_5(const char *s, double *out) {
  char buf[11];
  int k = 0, i;
  for (i = 0; i < 10 && s[i]; i++)
    if (s[i] != ' ') buf[k++] = s[i];
  buf[k] = 0;
  if (k == 0) { *out = 0.0; return 0; }
  /* split mantissa / exponent */
  int p = 0, neg = 0;
  if (buf[p] == '+' || buf[p] == '-') { neg = buf[p] == '-'; p++; }
  char mant[16]; int m = 0, has_dot = 0, ndig = 0;
  while (buf[p] && (isdigit((unsigned char)buf[p]) || buf[p] == '.')) {
    if (buf[p] == '.') { if (has_dot) return -1; has_dot = 1; }
    else ndig++;
    mant[m++] = buf[p++];
  }
  mant[m] = 0;
  int expo = 0;
  if (buf[p]) {
    if (buf[p] == 'e' || buf[p] == 'E' || buf[p] == 'd' || buf[p] == 'D') p++;
    if (!(buf[p] == '+' || buf[p] == '-' || isdigit((unsigned char)buf[p]))) return -1;
    char *end;
    long e = strtol(buf + p, &end, 10);
    if (*end) return -1;
    expo = (int)e;
  }
  if (ndig == 0) return -1;
  char num[48];
  if (has_dot)
    snprintf(num, sizeof num, "%se%d", mant, expo);
  else
    snprintf(num, sizeof num, "%se%d", mant, expo - 5);
  double v = strtod(num, NULL);
  *out = neg ? -v : v;
  return 0;
}

/* L1: first character T/t true, F/f false. */
int orc_parse_l1(const char *s, int *out) {
  char c = s[0];
  if (c == 'T' || c == 't') { *out = 1; return 0; }
  if (c == 'F' || c == 'f') { *out = 0; return 0; }
  if (c == '.' && (s[1] == 'T' || s[1] == 't')) { *out = 1; return 0; }
  if (c == '.' && (s[1] == 'F' || s[1] == 'f')) { *out = 0; return 0; }
  return -1;
}

/* getword (DOUG_utils.F90:1518-1544): words are separated by blanks only. */
static int getword(const char *line, int num, char *word, size_t wsz) {
  int n = (int)strlen(line);
  while (n > 0 && (line[n - 1] == ' ' || line[n - 1] == '\n' || line[n - 1] == '\r')) n--;
  int j = 0, k = 0, i;
  for (i = 1; i <= num; i++) {
    while (j < n && line[j] == ' ') j++;
    if (j >= n) { word[0] = 0; return 0; }
    k = j;
    while (j < n && line[j] != ' ') j++;
  }
  int len = j - k;
  if ((size_t)len >= wsz) len = (int)wsz - 1;
  memcpy(word, line + k, (size_t)len);
  word[len] = 0;
  return len;
}

/* util_actionOnCtrlArg (DOUG_utils.F90:703-1150): the first occurrence of a
 * word wins (later repeats only warn); unknown words are ignored. */
#define SETI(name) if (!strcmp(w1, #name)) { if (c->name == -1) { if (orc_parse_i10(w2, &c->name)) orc_abort("bad integer for %s: '%s'", w1, w2); } return; }
#define SETR(name) if (!strcmp(w1, #name)) { if (c->name == -1.0) { if (orc_parse_f10_5(w2, &c->name)) orc_abort("bad real for %s: '%s'", w1, w2); } return; }
#define SETL(name) if (!strcmp(w1, #name)) { int _v; if (orc_parse_l1(w2, &_v)) orc_abort("bad logical for %s: '%s'", w1, w2); c->name = _v; return; }
#define SETS(name) if (!strcmp(w1, #name)) { if (!c->name[0]) snprintf(c->name, sizeof c->name, "%s", w2); return; }
static void ctl_action(ctl_t *c, const char *w1, const char *w2) {
  SETI(solver) SETI(method) SETI(fine_method) SETI(num_iters) SETI(grid_size)
  SETI(coarse_method) SETI(num_subdomains) SETI(levels) SETI(overlap)
  SETI(smoothers) SETI(input_type) SETI(matrix_type) SETI(initial_guess)
  SETI(number_of_blocks) SETI(radius1) SETI(radius2) SETI(minasize1)
  SETI(minasize2) SETI(maxasize1) SETI(maxasize2) SETI(debug) SETI(verbose)
  SETI(plotting)
  SETR(strong1) SETR(strong2) SETR(solve_tolerance)
  SETI(solve_maxiters)
  SETL(symmstruct) SETL(symmnumeric)
  SETI(interpolation_type)
  SETS(assembled_mtx_file) SETI(assembled_mtx_format)
  SETS(assembled_rhs_file) SETI(assembled_rhs_format)
  SETS(solution_file) SETI(solution_format) SETI(start_vec_type)
  SETS(info_file) SETS(freedom_lists_file) SETS(elemmat_rhs_file)
  SETS(coords_file) SETS(freemap_file)
  SETI(maxcie) SETI(maxnd) SETI(cutbal) SETI(center_type) SETL(hanging_nodes)
  if (!strcmp(w1, "omega")) { /* not a reference word: parsed as a C double, first value wins */
    if (c->omega == -1.0) {
      char *end = NULL;
      double v = strtod(w2, &end);
      if (!end || *end || !(v > 0)) orc_abort("bad omega: '%s'", w2);
      c->omega = v;
    }
    return;
  }
  if (!strcmp(w1, "executable")) { /* not a reference word: which of the reference's drivers */
    if (c->executable == -1) {
      if (!strcmp(w2, "aggr")) c->executable = 0;
      else if (!strcmp(w2, "geom")) c->executable = 1;
      else orc_abort("executable must be aggr or geom: '%s'", w2);
    }
    return;
  }
}

/* CtrlData_initFromFile (DOUG_utils.F90:629-696), on text. */
static void ctl_parse_text(ctl_t *c, const char *text) {
  const char *p = text;
  char line[512], w1[320], w2[320];
  while (p && *p) {
    const char *e = strchr(p, '\n');
    size_t len = e ? (size_t)(e - p) : strlen(p);
    if (len > 300) len = 300;
    memcpy(line, p, len);
    line[len] = 0;
    p = e ? e + 1 : NULL;
    int lt = (int)strlen(line);
    while (lt > 0 && (line[lt - 1] == ' ' || line[lt - 1] == '\r')) lt--;
    line[lt] = 0;
    if (lt > 0 && line[0] != '#') {
      getword(line, 1, w1, sizeof w1);
      for (char *q = w1; *q; q++)
        if (*q >= 'A' && *q <= 'Z') *q = (char)(*q + 32);
      getword(line, 2, w2, sizeof w2);
      ctl_action(c, w1, w2);
    }
  }
}

static void ctl_finish(ctl_t *c) {
  if (c->solve_maxiters == -1) c->solve_maxiters = 100; /* DOUG_utils.F90:676-678 */
}

/* ------------------------------------------------------------------ */
/* sparse matrix in DOUG's COO + bounds form (SpMtx_class.F90:69-146)  */
/* ------------------------------------------------------------------ */
typedef struct {
  int nnz, nrows, ncols;
  int *indi, *indj;
  double *val;
  int arrange;
  int *mbound;
  int mbound_len; /* number of entries in mbound (n+1) */
  double *diag;
  int scaling;
  char *strong;
  int *srow, *scol;
  int symmstruct, symmnumeric;
} spm;

static spm spm_new(int nnz, int nrows, int ncols) {
  spm m;
  memset(&m, 0, sizeof m);
  m.nnz = nnz; m.nrows = nrows; m.ncols = ncols;
  m.indi = NEWI(nnz); m.indj = NEWI(nnz); m.val = NEWD(nnz);
  m.arrange = ARR_NO;
  m.scaling = SCALE_NO;
  return m;
}

static void spm_free(spm *m) {
  free(m->indi); free(m->indj); free(m->val); free(m->mbound); free(m->diag);
  free(m->strong); free(m->srow); free(m->scol);
  memset(m, 0, sizeof *m);
}

static spm spm_copy(const spm *a) { /* SpMtx_Copy, SpMtx_class.F90:680-699 */
  spm m = spm_new(a->nnz, a->nrows, a->ncols);
  memcpy(m.indi + 1, a->indi + 1, sizeof(int) * (size_t)a->nnz);
  memcpy(m.indj + 1, a->indj + 1, sizeof(int) * (size_t)a->nnz);
  memcpy(m.val + 1, a->val + 1, sizeof(double) * (size_t)a->nnz);
  m.arrange = a->arrange;
  if (a->arrange != ARR_NO) {
    m.mbound_len = a->mbound_len;
    m.mbound = NEWI(a->mbound_len);
    memcpy(m.mbound + 1, a->mbound + 1, sizeof(int) * (size_t)a->mbound_len);
  }
  return m;
}

static int imax_arr(const int *a, int n) {
  int m = INT_MIN, i;
  for (i = 1; i <= n; i++) if (a[i] > m) m = a[i];
  return m;
}

/* SpMtx_arrange (SpMtx_arrangement.F90:58-252): stable bucketing by row or
 * column; with sort=.true. an insertion sort by the other index. */
static void spm_arrange(spm *M, int at, int sort, int nnz_o, int nrows_o, int ncols_o) {
  int Mnnz = nnz_o > 0 ? nnz_o : M->nnz;
  int Mnrows = nrows_o > 0 ? nrows_o : M->nrows;
  int Mncols = ncols_o > 0 ? ncols_o : M->ncols;
  int columnwise = (at == ARR_COLS);
  int ok = (M->arrange == at);
  if (ok) {
    int need = columnwise ? Mncols + 1 : Mnrows + 1;
    if (!M->mbound || M->mbound_len != need) ok = 0;
  }
  if (ok) return; /* "arrange not needed" */
  M->arrange = at;
  int nb = columnwise ? Mncols : Mnrows;
  int *el = NEWI(nb);
  free(M->mbound);
  M->mbound = NEWI(nb + 1);
  M->mbound_len = nb + 1;
  int i, k;
  for (i = 1; i <= Mnnz; i++) {
    k = columnwise ? M->indj[i] : M->indi[i];
    if (k < 1 || k > nb) orc_abort("arrange: index %d out of range 1..%d", k, nb);
    el[k]++;
  }
  M->mbound[1] = 1;
  for (i = 1; i <= nb; i++) M->mbound[i + 1] = M->mbound[i] + el[i];
  int *ni = NEWI(Mnnz), *nj = NEWI(Mnnz);
  double *nv = NEWD(Mnnz);
  if (sort) {
    int *sortref = NEWI(Mnnz);
    memset(el, 0, sizeof(int) * (size_t)(nb + 1));
    for (i = 1; i <= Mnnz; i++) {
      k = columnwise ? M->indj[i] : M->indi[i];
      int ind_beg = M->mbound[k];
      if (el[k] == 0) {
        sortref[ind_beg] = i;
        el[k] = 1;
      } else {
        int ind = M->mbound[k] + el[k];
        int j = ind_beg;
        for (;;) {
          if (j == ind) { sortref[j] = i; el[k]++; break; }
          int other_i = columnwise ? M->indi[i] : M->indj[i];
          int other_s = columnwise ? M->indi[sortref[j]] : M->indj[sortref[j]];
          if (other_i < other_s) {
            int kk;
            for (kk = ind; kk >= j + 1; kk--) sortref[kk] = sortref[kk - 1];
            sortref[j] = i;
            el[k]++;
            break;
          }
          j++;
        }
      }
    }
    for (i = 1; i <= Mnnz; i++) {
      int ind = sortref[i];
      ni[i] = M->indi[ind]; nj[i] = M->indj[ind]; nv[i] = M->val[ind];
    }
    free(sortref);
  } else {
    memset(el, 0, sizeof(int) * (size_t)(nb + 1));
    for (i = 1; i <= Mnnz; i++) {
      k = columnwise ? M->indj[i] : M->indi[i];
      int ind = M->mbound[k] + el[k];
      el[k]++;
      ni[ind] = M->indi[i]; nj[ind] = M->indj[i]; nv[ind] = M->val[i];
    }
  }
  memcpy(M->indi + 1, ni + 1, sizeof(int) * (size_t)Mnnz);
  memcpy(M->indj + 1, nj + 1, sizeof(int) * (size_t)Mnnz);
  memcpy(M->val + 1, nv + 1, sizeof(double) * (size_t)Mnnz);
  free(ni); free(nj); free(nv); free(el);
  free(M->strong); M->strong = NULL; /* "destroy strong" :249-250 */
}

/* SpMtx_scale (SpMtx_arrangement.F90:298-346). */
static void spm_scale(spm *M) {
  if (!(M->scaling == SCALE_NO || M->scaling == SCALE_UNDEF)) return;
  int ndiags = M->nrows > M->ncols ? M->nrows : M->ncols;
  int i;
  if (!M->diag) M->diag = NEWD(ndiags);
  double *s = NEWD(ndiags);
  for (i = 1; i <= M->nnz; i++)
    if (M->indi[i] == M->indj[i]) M->diag[M->indi[i]] = M->val[i];
  if (M->symmstruct && M->symmnumeric) {
    for (i = 1; i <= ndiags; i++) s[i] = sqrt(fabs(M->diag[i]));
    for (i = 1; i <= M->nnz; i++) {
      M->val[i] = M->val[i] / s[M->indi[i]];
      M->val[i] = M->val[i] / s[M->indj[i]];
    }
  } else {
    for (i = 1; i <= ndiags; i++) s[i] = fabs(M->diag[i]);
    for (i = 1; i <= M->nnz; i++) M->val[i] = M->val[i] / s[M->indi[i]];
  }
  free(s);
  M->scaling = SCALE_DIAG;
}

/* SpMtx_unscale (SpMtx_arrangement.F90:350-388). */
static void spm_unscale(spm *M) {
  if (M->scaling != SCALE_DIAG) return;
  int ndiags = M->nrows > M->ncols ? M->nrows : M->ncols;
  int i;
  double *s = NEWD(ndiags);
  if (M->symmstruct && M->symmnumeric) {
    for (i = 1; i <= ndiags; i++) s[i] = sqrt(fabs(M->diag[i]));
    for (i = 1; i <= M->nnz; i++) {
      M->val[i] = M->val[i] * s[M->indi[i]];
      M->val[i] = M->val[i] * s[M->indj[i]];
    }
  } else {
    for (i = 1; i <= ndiags; i++) s[i] = fabs(M->diag[i]);
    for (i = 1; i <= M->nnz; i++) M->val[i] = M->val[i] * s[M->indi[i]];
  }
  free(s);
  free(M->diag); M->diag = NULL;
  M->scaling = SCALE_NO;
}

/* SpMtx_find_strong (SpMtx_aggregation.F90:829-900), symmetrise off. */
static void spm_find_strong(spm *A, double alpha) {
  if (A->scaling == SCALE_NO || A->scaling == SCALE_UNDEF) spm_scale(A);
  spm_arrange(A, ARR_ROWS, 0, 0, 0, 0);
  if (!A->strong) A->strong = NEWB(A->nnz);
  int i, j;
  for (i = 1; i <= A->nrows; i++) {
    int start = A->mbound[i], ending = A->mbound[i + 1] - 1;
    double maxndiag = (double)(-1.0e15f); /* default-real literal */
    for (j = start; j <= ending; j++)
      if (A->indj[j] != i) {
        double aa = fabs(A->val[j]);
        if (maxndiag < aa) maxndiag = aa;
      }
    maxndiag = maxndiag * alpha;
    for (j = start; j <= ending; j++) {
      double aa = fabs(A->val[j]);
      if (A->indj[j] != i)
        A->strong[j] = aa > maxndiag;
      else
        A->strong[j] = A->diag[i] > maxndiag; /* unscaled diagonal, :886 */
    }
  }
}

/* SpMtx_build_refs_symm with sortdown (SpMtx_arrangement.F90:461-568). */
static void spm_build_refs_symm(spm *A) {
  int nn = A->nrows, nnz = A->nnz, i;
  int *cnt = NEWI(nn);
  for (i = 1; i <= nnz; i++)
    if (A->strong[i]) {
      int ii = A->indi[i], jj = A->indj[i];
      if (ii != jj && jj <= nn) cnt[ii]++;
    }
  free(A->srow);
  A->srow = NEWI(nn + 1);
  A->srow[1] = 1;
  for (i = 1; i <= nn; i++) A->srow[i + 1] = A->srow[i] + cnt[i];
  int noff = A->srow[nn + 1] - 1;
  free(A->scol);
  A->scol = NEWI(noff);
  memset(cnt, 0, sizeof(int) * (size_t)(nn + 1));
  int *sortref = NEWI(noff);
  for (i = 1; i <= nnz; i++) {
    if (!A->strong[i]) continue;
    int ii = A->indi[i], jj = A->indj[i];
    if (ii == jj || jj > nn) continue;
    int ind_beg = A->srow[ii];
    if (cnt[ii] == 0) {
      sortref[ind_beg] = i;
      cnt[ii] = 1;
    } else {
      int ind = A->srow[ii] + cnt[ii] - 1;
      int j = ind_beg;
      for (;;) {
        if (j == ind + 1) { sortref[j] = i; cnt[ii]++; break; }
        if (fabs(A->val[i]) > fabs(A->val[sortref[j]])) {
          int k;
          for (k = ind + 1; k >= j + 1; k--) sortref[k] = sortref[k - 1];
          sortref[j] = i;
          cnt[ii]++;
          break;
        }
        j++;
      }
    }
  }
  for (i = 1; i <= noff; i++) A->scol[i] = A->indj[sortref[i]];
  free(sortref);
  free(cnt);
}

/* ------------------------------------------------------------------ */
/* aggregates (Aggregate_mod.F90)                                       */
/* ------------------------------------------------------------------ */
typedef struct {
  int nagr, radius, nisolated, n;
  int *num, *starts, *nodes;
} aggrs;

static void aggrs_free(aggrs *a) {
  free(a->num); free(a->starts); free(a->nodes);
  memset(a, 0, sizeof *a);
}

/* Form_Aggr (Aggregate_mod.F90:82-125). */
static void form_aggr(aggrs *ag, int nagrs, int n, int radius, int nisolated,
                      const int *aggrnum) {
  int i, j;
  int *starts = NEWI(nagrs + 1), *stat = NEWI(nagrs);
  for (i = 1; i <= n; i++) {
    j = aggrnum[i];
    if (j > 0) stat[j]++;
  }
  starts[1] = 1;
  for (i = 1; i <= nagrs; i++) {
    starts[i + 1] = starts[i] + stat[i];
    stat[i] = starts[i];
  }
  int *nodes = NEWI(starts[nagrs + 1] - 1);
  for (i = 1; i <= n; i++) {
    j = aggrnum[i];
    if (j > 0) { nodes[stat[j]] = i; stat[j]++; }
  }
  ag->nagr = nagrs; ag->radius = radius; ag->nisolated = nisolated; ag->n = n;
  ag->num = NEWI(n);
  memcpy(ag->num + 1, aggrnum + 1, sizeof(int) * (size_t)n);
  ag->starts = starts;
  ag->nodes = nodes;
  free(stat);
}

/* SAVE variables of the reference that persist across calls. */
static int g_allmind = D_MAXINT;  /* Aggregate_mod.F90:348 (integer,save) */
static double g_beta = 1.0e-5;    /* SpMtx_aggregation.F90:81 (initialised => SAVE) */

typedef struct {
  int *inlayer, *newlayer, *roundernodes;
  int cap, rcap;
  int neighood, minasize, maxasize;
  int *stat, *distance, *rowstart, *colnrs, *nodes;
  int nodes_cap;
} colour_ctx;

#define CHK(idx, cap) do { if ((idx) > (cap)) orc_abort("aggregation work array overflow (%d > %d)", (idx), (cap)); } while (0)

/* can_add_roundlayer (Aggregate_mod.F90:323-497). */
static int can_add_roundlayer(colour_ctx *c, int layer, int *ninnodes, int *nneigs) {
  int nxtlayer = layer + 1, layerfits = 1, ntoadd = 0;
  int i, j, k, d, rs, re, cn, layernode, nrounders = 0, mind, maxd;
  int neighood = c->neighood, maxasize = c->maxasize;
  int *stat = c->stat, *distance = c->distance, *inlayer = c->inlayer,
      *newlayer = c->newlayer;
  if (layerfits && layer <= 2 * neighood) {
    for (k = 1; k <= *ninnodes; k++) {
      layernode = inlayer[k];
      rs = c->rowstart[layernode];
      re = c->rowstart[layernode + 1] - 1;
      for (i = rs; i <= re; i++) {
        cn = c->colnrs[i];
        if (stat[cn] <= 0) {
          if (stat[cn] == 0) {
            ntoadd++;
            CHK(ntoadd, c->cap);
            newlayer[ntoadd] = cn;
            distance[cn] = distance[layernode] + 1;
          }
          stat[cn] = stat[cn] - 1;
        }
      }
    }
  }
  if (layerfits && layer <= neighood) {
    nrounders = 0;
    mind = D_MAXINT;
    maxd = 0;
    for (k = 1; k <= ntoadd; k++) {
      d = -stat[newlayer[k]];
      if (d < mind) mind = d;
      if (d > maxd) maxd = d;
    }
    if (mind < g_allmind) g_allmind = mind;
    if (mind < maxd || mind > g_allmind) {
      for (k = 1; k <= ntoadd; k++) {
        if (stat[newlayer[k]] == -maxd) {
          nrounders++;
          if (*nneigs + *ninnodes + 1 > maxasize) { layerfits = 0; break; }
          (*ninnodes)++;
          CHK(*ninnodes, c->cap);
          inlayer[*ninnodes] = newlayer[k];
          CHK(nrounders, c->rcap);
          c->roundernodes[nrounders] = newlayer[k];
          newlayer[k] = -1;
        }
      }
    }
    if (!layerfits) nrounders = 0;
    j = 0;
    for (i = 1; i <= ntoadd; i++)
      if (newlayer[i] != -1) {
        j++;
        if (j < i) newlayer[j] = newlayer[i];
      }
    ntoadd = j;
    for (k = 1; k <= nrounders; k++) {
      layernode = c->roundernodes[k];
      rs = c->rowstart[layernode];
      re = c->rowstart[layernode + 1] - 1;
      for (i = rs; i <= re; i++) {
        cn = c->colnrs[i];
        if (stat[cn] == 0) {
          ntoadd++;
          CHK(ntoadd, c->cap);
          newlayer[ntoadd] = cn;
          distance[cn] = distance[layernode] + 1;
        }
      }
    }
  }
  if (layer <= neighood && *nneigs + *ninnodes > maxasize) layerfits = 0;
  if (layerfits) {
    for (k = 1; k <= *ninnodes; k++) {
      stat[inlayer[k]] = layer + 1;
      (*nneigs)++;
      CHK(*nneigs, c->nodes_cap);
      c->nodes[*nneigs] = inlayer[k];
    }
    if (layer <= 2 * neighood) {
      for (k = 1; k <= ntoadd; k++) stat[newlayer[k]] = D_PENDING - 1;
      *ninnodes = ntoadd;
      for (k = 1; k <= ntoadd; k++) inlayer[k] = newlayer[k];
      return can_add_roundlayer(c, nxtlayer, ninnodes, nneigs);
    }
    return 3;
  }
  for (k = 1; k <= *ninnodes; k++) distance[inlayer[k]] = 0;
  for (k = 1; k <= ntoadd; k++) distance[newlayer[k]] = 0;
  for (k = 1; k <= *nneigs; k++) distance[c->nodes[k]] = 0;
  for (k = 1; k <= *ninnodes; k++) {
    (*nneigs)++;
    CHK(*nneigs, c->nodes_cap);
    c->nodes[*nneigs] = inlayer[k];
  }
  if (*nneigs > 0) return layer > neighood ? 2 : 1;
  return 0;
}

/* lets_colour (Aggregate_mod.F90:287-321). */
static int lets_colour(colour_ctx *c, int innode, int *nneigs) {
  *nneigs = 0;
  long virt = 2L * c->maxasize * c->maxasize;
  if (virt > 50000000L) orc_abort("maxasize too large");
  if (!c->inlayer) { /* the reference's work arrays (Aggregate_mod.F90:305-310), allocated
                      * once per aggregation here and kept across calls: every entry is
                      * written before it is read */
    c->cap = (int)virt;
    c->rcap = c->maxasize;
    c->inlayer = (int *)malloc(sizeof(int) * ((size_t)c->cap + 1));
    c->newlayer = (int *)malloc(sizeof(int) * ((size_t)c->cap + 1));
    c->roundernodes = (int *)malloc(sizeof(int) * ((size_t)c->rcap + 1));
    if (!c->inlayer || !c->newlayer || !c->roundernodes) orc_abort("out of memory");
  }
  c->stat[innode] = 1;
  c->distance[innode] = 0;
  int ninnodes = 1;
  c->inlayer[1] = innode;
  return can_add_roundlayer(c, 0, &ninnodes, nneigs);
}

/* SpMtx_aggregate (SpMtx_aggregation.F90:49-641), numprocs==1. */
static void spm_aggregate(spm *A, aggrs *inner, aggrs *full, int neighood,
                          int minaggrsize, int maxaggrsize, double alpha,
                          int coarse) {
  int n = A->nrows, nn = n, i, j, k, kk, kkk, node;
  int toosmall = 0, nagrs = 0, nisolated = 0, unaggregated = 0;
  int *aggrnum = NEWI(nn), *fullaggrnum = NEWI(n);
  int sn = (int)sqrtf((float)n); /* default-real sqrt, :123 */
  int minasize, maxasize, maxasizelargest;
  (void)unaggregated;
  minasize = minaggrsize;
  maxasize = maxaggrsize;
  if (alpha >= 0 || sn * sn != n) {
    if (!A->srow) spm_build_refs_symm(A);
    /* nodes(n) in the reference; a node next to two rounder nodes is queued
     * twice (the rounder-neighbour scan does not mark it), so on small graphs
     * the list can outgrow n and the Fortran writes past the array end.  A
     * longer array gives that write somewhere to land. */
    int nodes_cap = 4 * n + 64;
    int *stat = NEWI(n), *nodes = NEWI(nodes_cap), *distance = NEWI(n);
    if (!coarse) maxasizelargest = maxasize + 4 * (2 * neighood);
    else maxasizelargest = 3 * maxasize;
    if (!coarse) g_beta = alpha / 4.0;
    int ngoodstarts = 0;
    int *nextgoodstart = NEWI(n);
    int *seen = NEWI(n), seen_stamp = 0;
    int firstwocol = 1;
    colour_ctx c;
    memset(&c, 0, sizeof c);
    c.neighood = neighood; c.minasize = minasize; c.maxasize = maxasize;
    c.stat = stat; c.distance = distance; c.rowstart = A->srow;
    c.colnrs = A->scol; c.nodes = nodes; c.nodes_cap = nodes_cap;
    while (firstwocol <= n) {
      int startnode, nneigs, ok, mindistance, nouters, next_start_layer;
      if (ngoodstarts > 0) {
        j = 0;
        for (i = 1; i <= ngoodstarts; i++)
          if (stat[nextgoodstart[i]] < D_PENDING) {
            j++;
            if (j < i) nextgoodstart[j] = nextgoodstart[i];
          }
        ngoodstarts = j;
      }
      if (ngoodstarts == 0) {
        int done = 0;
        while (stat[firstwocol] >= D_PENDING) {
          firstwocol++;
          if (firstwocol > n) { done = 1; break; }
        }
        if (done) break;
        startnode = firstwocol;
      } else {
        /* the first entry that repeats an earlier one (SpMtx_aggregation.F90:206-218), found with
         * a marker per node instead of the pairwise scan */
        startnode = 0;
        seen_stamp++;
        for (i = 1; i <= ngoodstarts; i++) {
          if (seen[nextgoodstart[i]] == seen_stamp) { startnode = nextgoodstart[i]; break; }
          seen[nextgoodstart[i]] = seen_stamp;
        }
        if (startnode == 0) startnode = nextgoodstart[1];
      }
      ok = lets_colour(&c, startnode, &nneigs);
      mindistance = D_MAXINT;
      if (ok <= 0) orc_abort("aggregation found nothing at node %d", startnode);
      nagrs++;
      nouters = 0;
      if (ok == 3) {
        int *layerlen = NEWI(2 * neighood + 2);
        int maxlayer = 0;
        if (!toosmall && nneigs < minasize) toosmall = 1;
        for (j = nneigs; j >= 1; j--) {
          k = stat[nodes[j]];
          if (k > maxlayer) maxlayer = k;
          if (k <= neighood + 1) break;
          if (k > 2 * neighood + 2) orc_abort("layer index out of range");
          layerlen[k]++;
        }
        next_start_layer = neighood + 2;
        k = layerlen[neighood + 2];
        for (j = neighood + 3; j <= maxlayer; j++)
          if (k < layerlen[j]) { k = layerlen[j]; next_start_layer = j; }
        free(layerlen);
      } else if (ok == 2) {
        next_start_layer = neighood + 2;
        if (!toosmall && nneigs < minasize) toosmall = 1;
      } else {
        next_start_layer = 0;
      }
      for (j = 1; j <= nneigs; j++) {
        node = nodes[j];
        if (stat[node] <= neighood + 1 && j <= maxasize) {
          stat[node] = D_AGGREGATED;
          aggrnum[node] = nagrs;
        } else if (next_start_layer > neighood + 1) {
          if (stat[node] == next_start_layer) {
            if (distance[node] < mindistance) mindistance = distance[node];
            nouters++;
            nextgoodstart[n - nouters + 1] = node;
          }
        }
      }
      for (j = 1; j <= nouters; j++)
        if (distance[nextgoodstart[n - j + 1]] == mindistance) {
          ngoodstarts++;
          nextgoodstart[ngoodstarts] = nextgoodstart[n - j + 1];
        }
      for (j = 1; j <= nneigs; j++) {
        node = nodes[j];
        if (stat[node] != D_AGGREGATED) { distance[node] = 0; stat[node] = 0; }
      }
    }
    free(c.inlayer); free(c.newlayer); free(c.roundernodes);
    free(seen);
    free(nextgoodstart); free(distance); free(nodes); free(stat);
  } else {
    /* Cartesian aggregates (:332-346); a radius below 1 is an integer
     * division fault in the reference */
    if (neighood < 1) orc_abort("Cartesian aggregation needs an aggregation radius >= 1 (radius %d)", neighood);
    int nsa = (sn + neighood - 1) / neighood;
    k = 0;
    for (i = 1; i <= sn; i++)
      for (j = 1; j <= sn; j++) {
        k++;
        aggrnum[k] = ((i + neighood - 1) / neighood - 1) * nsa + (j + neighood - 1) / neighood;
      }
    nagrs = imax_arr(aggrnum, n);
    nisolated = 0;
    maxasizelargest = maxasize + 4 * (2 * neighood);
  }
  int full_nagrs_new;
  if (!toosmall) {
    for (i = 1; i <= n; i++) fullaggrnum[i] = aggrnum[i];
    full_nagrs_new = imax_arr(fullaggrnum, n);
    if (full_nagrs_new < 0) full_nagrs_new = 0;
    form_aggr(inner, nagrs, n, neighood, nisolated, aggrnum);
  } else {
    /* repair of too small aggregates (:369-591) */
    int *aggrsize = NEWI(nagrs);
    for (i = 1; i <= n; i++) { j = aggrnum[i]; aggrsize[j]++; }
    int maxstructlen = maxasizelargest;
    for (i = 1; i <= nagrs; i++) if (aggrsize[i] > maxstructlen) maxstructlen = aggrsize[i];
    int **structnodes = (int **)xcalloc((size_t)nagrs + 1, sizeof(int *));
    for (i = 1; i <= nagrs; i++) structnodes[i] = NEWI(maxstructlen);
    memset(aggrsize, 0, sizeof(int) * (size_t)(nagrs + 1));
    for (i = 1; i <= n; i++) {
      j = aggrnum[i];
      aggrsize[j]++;
      structnodes[j][aggrsize[j]] = i;
    }
    int mnstructneigs = 4 * maxasize;
    spm_arrange(A, ARR_ROWS, 0, 0, 0, 0);
    int *colsaround = NEWI(mnstructneigs);
    double *connweightsums = NEWD(mnstructneigs);
    int nagrs_new = nagrs;
    for (i = 1; i <= nagrs; i++) {
      if (aggrsize[i] >= minasize) continue;
      int ncolsaround = 0;
      memset(colsaround, 0, sizeof(int) * (size_t)(mnstructneigs + 1));
      for (k = 1; k <= aggrsize[i]; k++) {
        kkk = structnodes[i][k];
        int rs = A->mbound[kkk], re = A->mbound[kkk + 1] - 1;
        for (j = rs; j <= re; j++) {
          int cn = A->indj[j];
          if (cn <= n) {
            int colr = aggrnum[cn];
            if (colr > 0 && colr != i) {
              for (kk = 1; kk <= ncolsaround; kk++)
                if (colr == colsaround[kk]) {
                  connweightsums[kk] = connweightsums[kk] + fabs(A->val[j]);
                  break;
                }
              if (kk > ncolsaround) {
                ncolsaround++;
                if (ncolsaround > mnstructneigs) orc_abort("mnstructneigs too small");
                connweightsums[kk] = fabs(A->val[j]);
                colsaround[kk] = colr;
              }
            }
          }
        }
      }
      double maxconnweightsum = 0.0;
      int eater = 0;
      for (j = 1; j <= ncolsaround; j++)
        if (maxconnweightsum < connweightsums[j])
          if (aggrsize[colsaround[j]] + aggrsize[i] <= maxasize) {
            maxconnweightsum = connweightsums[j];
            eater = colsaround[j];
          }
      if (maxconnweightsum >= alpha || (coarse && maxconnweightsum >= g_beta)) {
        if (eater == 0) orc_abort("aggregate repair without an eater (alpha <= 0)");
        for (j = 1; j <= aggrsize[i]; j++) {
          aggrsize[eater]++;
          if (aggrsize[eater] > maxstructlen) orc_abort("structnodes overflow");
          structnodes[eater][aggrsize[eater]] = structnodes[i][j];
          aggrnum[structnodes[i][j]] = eater;
        }
        aggrsize[i] = 0;
        nagrs_new--;
      } else {
        int nleft = aggrsize[i], reduced = 1;
        while (nleft > 0 && reduced) {
          reduced = 0;
          for (k = aggrsize[i]; k >= 1; k--) {
            kkk = structnodes[i][k];
            if (kkk > 0) {
              int rs = A->mbound[kkk], re = A->mbound[kkk + 1] - 1;
              for (j = rs; j <= re; j++) {
                int cn = A->indj[j];
                if (cn <= n) {
                  int colr = aggrnum[cn];
                  if (colr != i) {
                    if (colr < 1) orc_abort("repair: unaggregated neighbour");
                    if (aggrsize[colr] < maxasizelargest && fabs(A->val[j]) >= g_beta) {
                      aggrsize[colr]++;
                      if (aggrsize[colr] > maxstructlen) orc_abort("structnodes overflow");
                      structnodes[colr][aggrsize[colr]] = structnodes[i][k];
                      aggrnum[structnodes[i][k]] = colr;
                      structnodes[i][k] = -1;
                      nleft--;
                      reduced = 1;
                      break;
                    }
                  }
                }
              }
            }
          }
        }
        if (nleft > 0 && nleft < aggrsize[i]) {
          k = 0;
          for (j = 1; j <= aggrsize[i]; j++)
            if (structnodes[i][j] > 0) {
              k++;
              if (k > 0 && k < j) structnodes[i][k] = structnodes[i][j];
            }
          aggrsize[i] = nleft;
        } else if (nleft == 0) {
          aggrsize[i] = 0;
          nagrs_new--;
        }
      }
    }
    int naggregatednodes = 0;
    for (i = 1; i <= nagrs; i++) naggregatednodes += aggrsize[i];
    full_nagrs_new = nagrs_new;
    int cnt = imax_arr(aggrnum, n);
    if (cnt > nagrs_new) {
      int *st = NEWI(cnt), col = 0;
      for (i = 1; i <= n; i++)
        if (aggrnum[i] > 0) {
          int thiscol;
          if (st[aggrnum[i]] == 0) { col++; st[aggrnum[i]] = col; thiscol = col; }
          else thiscol = st[aggrnum[i]];
          aggrnum[i] = thiscol;
        }
      free(st);
    }
    if (n == naggregatednodes) {
      for (i = 1; i <= n; i++) fullaggrnum[i] = aggrnum[i];
      full_nagrs_new = imax_arr(fullaggrnum, n);
    } else {
      for (i = 1; i <= n; i++) {
        if (aggrnum[i] > 0) fullaggrnum[i] = aggrnum[i];
        else { full_nagrs_new++; fullaggrnum[i] = full_nagrs_new; }
      }
    }
    form_aggr(inner, nagrs_new, n, neighood, n - naggregatednodes, aggrnum);
    free(connweightsums); free(colsaround);
    for (i = 1; i <= nagrs; i++) free(structnodes[i]);
    free(structnodes); free(aggrsize);
    nagrs = nagrs_new;
  }
  form_aggr(full, full_nagrs_new, n, neighood, nisolated, fullaggrnum);
  free(fullaggrnum); free(aggrnum);
}

/* Get_aggregate_nodes (Aggregate_mod.F90:162-190). */
static int get_aggregate_nodes(int cAggr, const aggrs *cA, const aggrs *fA,
                               int maxnodes, int *nodes) {
  int *nodeLoc = NEWI(maxnodes), nnodes = 0, ifa, inode;
  for (ifa = cA->starts[cAggr]; ifa <= cA->starts[cAggr + 1] - 1; ifa++) {
    int fAggr = cA->nodes[ifa];
    for (inode = fA->starts[fAggr]; inode <= fA->starts[fAggr + 1] - 1; inode++) {
      int node = fA->nodes[inode];
      if (nodeLoc[node] == 0) {
        nnodes++;
        nodeLoc[node] = nnodes;
        nodes[nnodes] = node;
      }
    }
  }
  free(nodeLoc);
  return nnodes;
}

/* ------------------------------------------------------------------ */
/* SpMtx_AB (SpMtx_op_AB.f90:39-200): Gustavson row by row, dense       */
/* marker, output columns in first-touch order, zeros kept.             */
/* ------------------------------------------------------------------ */
static spm spm_AB(spm *A, spm *B, int AT, int BT) {
  int *Aindi, *Aindj, *Bindi, *Bindj;
  int Anrows, Ancols, Bnrows, Bncols;
  (void)Aindi; (void)Bindi;
  if (AT) {
    Aindi = A->indj; Aindj = A->indi;
    Anrows = A->ncols > imax_arr(A->indj, A->nnz) ? A->ncols : imax_arr(A->indj, A->nnz);
    Ancols = A->nrows > imax_arr(A->indi, A->nnz) ? A->nrows : imax_arr(A->indi, A->nnz);
    spm_arrange(A, ARR_COLS, 0, A->nnz, Ancols, Anrows);
  } else {
    Aindi = A->indi; Aindj = A->indj;
    Anrows = A->nrows > imax_arr(A->indi, A->nnz) ? A->nrows : imax_arr(A->indi, A->nnz);
    Ancols = A->ncols > imax_arr(A->indj, A->nnz) ? A->ncols : imax_arr(A->indj, A->nnz);
    spm_arrange(A, ARR_ROWS, 0, A->nnz, Anrows, Ancols);
  }
  if (BT) {
    Bindi = B->indj; Bindj = B->indi;
    Bnrows = B->ncols > imax_arr(B->indj, B->nnz) ? B->ncols : imax_arr(B->indj, B->nnz);
    Bncols = B->nrows > imax_arr(B->indi, B->nnz) ? B->nrows : imax_arr(B->indi, B->nnz);
    spm_arrange(B, ARR_COLS, 0, B->nnz, Bncols, Bnrows);
  } else {
    Bindi = B->indi; Bindj = B->indj;
    Bnrows = B->nrows > imax_arr(B->indi, B->nnz) ? B->nrows : imax_arr(B->indi, B->nnz);
    Bncols = B->ncols > imax_arr(B->indj, B->nnz) ? B->ncols : imax_arr(B->indj, B->nnz);
    spm_arrange(B, ARR_ROWS, 0, B->nnz, Bnrows, Bncols);
  }
  if (Ancols != Bnrows) orc_abort("A*B is impossible: %d vs %d", Ancols, Bnrows);
  /* after arrange the index pointers may have moved */
  if (AT) { Aindj = A->indi; } else { Aindj = A->indj; }
  if (BT) { Bindj = B->indi; } else { Bindj = B->indj; }
  int *indeces = NEWI(Bncols), *coladder = NEWI(Bncols);
  /* first pass: count output nnz (the reference grows its estimate and
   * retries; the result is the same) */
  long total = 0;
  int i, k, j;
  for (i = 1; i <= Anrows; i++) {
    int nind = 0;
    for (k = A->mbound[i]; k <= A->mbound[i + 1] - 1; k++) {
      int kk = Aindj[k];
      for (j = B->mbound[kk]; j <= B->mbound[kk + 1] - 1; j++) {
        int jj = Bindj[j];
        if (coladder[jj] != i) { coladder[jj] = i; nind++; }
      }
    }
    total += nind;
  }
  if (total > INT_MAX / 2) orc_abort("SpMtx_AB output too large");
  int nnz = (int)total;
  spm AB = spm_new(nnz, Anrows, Bncols);
  AB.arrange = ARR_ROWS;
  AB.mbound = NEWI(Anrows + 1);
  AB.mbound_len = Anrows + 1;
  memset(coladder, 0, sizeof(int) * (size_t)(Bncols + 1));
  int counter = 1;
  for (i = 1; i <= Anrows; i++) {
    AB.mbound[i] = counter;
    int nind = 0;
    for (k = A->mbound[i]; k <= A->mbound[i + 1] - 1; k++) {
      int kk = Aindj[k];
      for (j = B->mbound[kk]; j <= B->mbound[kk + 1] - 1; j++) {
        int jj = Bindj[j];
        if (coladder[jj] != i) {
          coladder[jj] = i;
          nind++;
          indeces[jj] = nind;
          AB.indi[counter + nind - 1] = i;
          AB.indj[counter + nind - 1] = jj;
          AB.val[counter + nind - 1] = A->val[k] * B->val[j];
        } else {
          int kkk = indeces[jj];
          AB.val[counter + kkk - 1] = AB.val[counter + kkk - 1] + A->val[k] * B->val[j];
        }
      }
    }
    counter += nind;
  }
  AB.mbound[Anrows + 1] = counter;
  free(indeces); free(coladder);
  return AB;
}

/* KeepGivenColumnIndeces (SpMtx_util.f90:232-286) for inds = 1..ninner. */
static void keep_columns_upto(spm *A, int ninner, int keepShape) {
  int i, nz = 0;
  for (i = 1; i <= A->nnz; i++)
    if (A->indj[i] >= 1 && A->indj[i] <= ninner) {
      nz++;
      A->indi[nz] = A->indi[i]; A->indj[nz] = A->indj[i]; A->val[nz] = A->val[i];
    }
  if (nz < A->nnz) {
    A->nnz = nz;
    if (!keepShape) A->ncols = imax_arr(A->indj, nz);
  }
  if (A->arrange != ARR_NO) {
    free(A->mbound); A->mbound = NULL; A->mbound_len = 0;
    A->arrange = ARR_NO;
  }
}

/* Build one Jacobi-type smoother S (CoarseMtx.F90:154-233 for S with
 * diag accumulated from 0; :236-301 for S2 whose diagonal is assigned). */
static spm build_smoother(const spm *A, double omega, int assign_diag) {
  int N = A->nrows > A->ncols ? A->nrows : A->ncols, i;
  double *diag = NEWD(N);
  for (i = 1; i <= A->nnz; i++) {
    if (A->indi[i] == A->indj[i]) {
      if (assign_diag) diag[A->indi[i]] = A->val[i];
      else diag[A->indi[i]] = diag[A->indi[i]] + A->val[i];
    } else if (!A->strong[i]) {
      diag[A->indi[i]] = diag[A->indi[i]] + A->val[i];
    }
  }
  spm S = spm_new(A->nnz, A->nrows, A->nrows);
  int nz = 0;
  for (i = 1; i <= A->nnz; i++) {
    nz++;
    S.indi[nz] = A->indi[i];
    S.indj[nz] = A->indj[i];
    if (A->indi[i] == A->indj[i]) S.val[nz] = 1.0 - omega;
    else if (A->strong[i]) S.val[nz] = -(omega / diag[A->indi[i]] * A->val[i]);
    else S.val[nz] = 0.0;
  }
  free(diag);
  return S;
}

/* IntRestBuild (CoarseMtx.F90:50-474), np=1 (no ghost matrix). */
static spm int_rest_build(const spm *A, const aggrs *ag, int smoothers, double w) {
  const double omega = w > 0 ? w : 0.33333333333333;   /* :64 */
  const double omega2 = w > 0 ? w : 0.33333333333333;  /* :67 */
  int Tnrows = A->nrows, i, j, k;
  int nz = ag->starts[ag->nagr + 1] - 1, nagr = ag->nagr;
  spm T = spm_new(nz, nagr, Tnrows);
  for (i = 1; i <= nagr; i++)
    for (j = ag->starts[i]; j <= ag->starts[i + 1] - 1; j++) T.indi[j] = i;
  for (k = 1; k <= nz; k++) { T.indj[k] = ag->nodes[k]; T.val[k] = 1.0; }
  if (smoothers == 0) return T; /* :82-127, arrange_type NO */
  if (smoothers < 0) orc_abort("smoothers=%d not supported", smoothers);
  spm S = build_smoother(A, omega, 0);
  spm R;
  if (smoothers == 1) {
    R = spm_AB(&T, &S, 0, 1);
  } else {
    spm S2 = build_smoother(A, omega2, 1);
    spm SS = spm_AB(&S2, &S, 0, 0);
    if (smoothers == 3) {
      spm SSS = spm_AB(&SS, &S2, 0, 0);
      R = spm_AB(&T, &SSS, 0, 0);
      spm_free(&SSS);
    } else if (smoothers == 4) {
      spm SSSS = spm_AB(&SS, &SS, 0, 0);
      R = spm_AB(&T, &SSSS, 0, 0);
      spm_free(&SSSS);
    } else if (smoothers == 5) {
      spm SSSS = spm_AB(&SS, &SS, 0, 0);
      spm SSS = spm_AB(&SSSS, &S2, 0, 0);
      R = spm_AB(&T, &SSS, 0, 0);
      spm_free(&SSSS); spm_free(&SSS);
    } else if (smoothers == 6) {
      spm SSSS = spm_AB(&SS, &SS, 0, 0);
      spm SSS = spm_AB(&SSSS, &SS, 0, 0);
      R = spm_AB(&T, &SSS, 0, 0);
      spm_free(&SSSS); spm_free(&SSS);
    } else if (smoothers == 7) {
      spm SSSS = spm_AB(&SS, &SS, 0, 0);
      spm SSS = spm_AB(&SSSS, &SS, 0, 0);
      spm_free(&SSSS);
      SSSS = spm_AB(&SSS, &S2, 0, 0);
      spm_free(&SSS);
      R = spm_AB(&T, &SSSS, 0, 0);
      spm_free(&SSSS);
    } else if (smoothers == 8) {
      spm SSSS = spm_AB(&SS, &SS, 0, 0);
      spm SSS = spm_AB(&SSSS, &SSSS, 0, 0);
      R = spm_AB(&T, &SSS, 0, 0);
      spm_free(&SSSS); spm_free(&SSS);
    } else { /* 2, and >8 which the reference performs as 2 */
      R = spm_AB(&T, &SS, 0, 1);
    }
    spm_free(&SS); spm_free(&S2);
  }
  spm_free(&S); spm_free(&T);
  return R;
}

/* Dense lower Cholesky in place (n x n, column-major, 0-based); 0 if not SPD. */
static int dense_chol(int n, double *a) {
  int i, j, k;
  for (j = 0; j < n; j++) {
    double d = a[(size_t)j * n + j];
    for (k = 0; k < j; k++) d -= a[(size_t)k * n + j] * a[(size_t)k * n + j];
    if (!(d > 0.0)) return 0;
    d = sqrt(d);
    a[(size_t)j * n + j] = d;
    for (i = j + 1; i < n; i++) {
      double v = a[(size_t)j * n + i];
      for (k = 0; k < j; k++) v -= a[(size_t)k * n + i] * a[(size_t)k * n + j];
      a[(size_t)j * n + i] = v / d;
    }
  }
  return 1;
}
static void dense_chol_solve(int n, const double *l, double *x) {
  int i, k;
  for (i = 0; i < n; i++) {
    double v = x[i];
    for (k = 0; k < i; k++) v -= l[(size_t)k * n + i] * x[k];
    x[i] = v / l[(size_t)i * n + i];
  }
  for (i = n - 1; i >= 0; i--) {
    double v = x[i];
    for (k = i + 1; k < n; k++) v -= l[(size_t)i * n + k] * x[k];
    x[i] = v / l[(size_t)i * n + i];
  }
}

/* Robust coarse space (coarse_method 2): CoarsePreconditioner_robust_Init
 * (CoarsePreconditioner_robust.F90:34-63), CoarseProjectionMtxsBuild and
 * RobustRestrictMtxBuild (RobustCoarseMtx.f90:53-210).  The support S_i of
 * coarse node i is the column list of row i of the smoothed restriction R in
 * R's entry order; A_i = A(S_i, S_i); g solves B g = 1 with
 * B = sum_i R_i^T A_i^-1 R_i; row i of the new restriction holds
 * q_i = A_i^-1 g(S_i) on S_i, rows one after the other.  The reference reaches
 * g by preconditioned CG (pcg_forRCS, pcg_robust.f90:37-120, stopping on
 * ||r||/||r0|| <= tol^2); here B is formed densely and factored, an exact
 * solve for test-sized problems. */
static spm robust_restriction(const spm *A, const spm *R) {
  int n = A->nrows, nagr = R->nrows, k, i, j;
  spm Ar = spm_copy(A);
  spm_arrange(&Ar, ARR_ROWS, 0, 0, 0, 0);
  int *cnt = (int *)xcalloc((size_t)nagr + 2, sizeof(int));
  for (k = 1; k <= R->nnz; k++) cnt[R->indi[k]]++;
  int *start = (int *)xcalloc((size_t)nagr + 2, sizeof(int));
  for (i = 1; i <= nagr; i++) start[i + 1] = start[i] + cnt[i];
  int *supp = (int *)xcalloc((size_t)R->nnz + 1, sizeof(int));
  int *fill = (int *)xcalloc((size_t)nagr + 2, sizeof(int));
  for (k = 1; k <= R->nnz; k++) { i = R->indi[k]; supp[start[i] + fill[i]++] = R->indj[k]; }
  int *pos = (int *)xcalloc((size_t)n + 1, sizeof(int));
  for (i = 1; i <= n; i++) pos[i] = -1;
  double **Linv = (double **)xcalloc((size_t)nagr + 1, sizeof(double *));
  double *B = (double *)xcalloc((size_t)n * n, sizeof(double));
  for (i = 1; i <= nagr; i++) {
    int m = cnt[i], a, b;
    const int *S = supp + start[i];
    for (a = 0; a < m; a++) pos[S[a]] = a;
    double *Ai = (double *)xcalloc((size_t)m * m, sizeof(double));
    for (a = 0; a < m; a++) {
      int row = S[a];
      for (k = Ar.mbound[row]; k < Ar.mbound[row + 1]; k++) {
        int col = Ar.indj[k];
        if (col <= n && pos[col] >= 0) Ai[(size_t)pos[col] * m + a] += Ar.val[k];
      }
    }
    if (!dense_chol(m, Ai)) orc_abort("robust coarse space: a support matrix is not positive definite");
    double *col = (double *)xcalloc((size_t)m, sizeof(double));
    for (b = 0; b < m; b++) {  /* column b of A_i^-1 into B(S, S) */
      for (a = 0; a < m; a++) col[a] = a == b ? 1.0 : 0.0;
      dense_chol_solve(m, Ai, col);
      for (a = 0; a < m; a++) B[(size_t)(S[b] - 1) * n + (S[a] - 1)] += col[a];
    }
    free(col);
    Linv[i] = Ai;
    for (a = 0; a < m; a++) pos[S[a]] = -1;
  }
  if (!dense_chol(n, B)) orc_abort("robust coarse space: B is not positive definite");
  double *g = (double *)xcalloc((size_t)n, sizeof(double));
  for (j = 0; j < n; j++) g[j] = 1.0;
  dense_chol_solve(n, B, g);
  spm Rh = spm_new(R->nnz, nagr, R->ncols);
  int q = 0;
  for (i = 1; i <= nagr; i++) {
    int m = cnt[i], a;
    const int *S = supp + start[i];
    double *qi = (double *)xcalloc((size_t)m, sizeof(double));
    for (a = 0; a < m; a++) qi[a] = g[S[a] - 1];
    dense_chol_solve(m, Linv[i], qi);
    for (a = 0; a < m; a++) { q++; Rh.indi[q] = i; Rh.indj[q] = S[a]; Rh.val[q] = qi[a]; }
    free(qi);
    free(Linv[i]);
  }
  free(Linv); free(B); free(g); free(pos); free(fill); free(supp); free(start); free(cnt);
  spm_free(&Ar);
  return Rh;
}

/* CoarseMtxBuild (CoarseMtx.F90:476-516), np=1: T=A*R^T, AC=R*T. It
 * re-arranges R by columns as a side effect, exactly as the reference.
 * keep: assembled / structured input restrict R to the inner columns. */
static spm coarse_mtx_build(const spm *A, spm *R, int ninner, int keep) {
  spm TT = spm_copy(A);
  spm T = spm_AB(&TT, R, 0, 1);
  spm_free(&TT);
  spm RT = spm_copy(R);
  if (keep) keep_columns_upto(&RT, ninner, 1);
  spm AC = spm_AB(&RT, &T, 0, 0);
  spm_free(&RT); spm_free(&T);
  return AC;
}

/* Add_layers (Decomposition.f90:56-99). nodes has room for nlf entries. */
static int add_layers(const int *adjBounds, const int *adjValues, int *nodes,
                      int nnodes, int nlayers, int nlf) {
  int *frontstart = (int *)xcalloc((size_t)nlayers + 1, sizeof(int));
  int *frontend = (int *)xcalloc((size_t)nlayers + 1, sizeof(int));
  int *onfront = NEWI(nlf), i, j, layer;
  for (i = 1; i <= nnodes; i++) onfront[nodes[i]] = -1;
  frontstart[0] = 1;
  int nfront = nnodes;
  frontend[0] = nfront;
  for (layer = 1; layer <= nlayers; layer++) {
    frontstart[layer] = nfront;
    for (i = frontstart[layer - 1]; i <= frontend[layer - 1]; i++) {
      int node = nodes[i];
      for (j = adjBounds[node]; j <= adjBounds[node + 1] - 1; j++) {
        int neigh = adjValues[j];
        if (onfront[neigh] == 0) {
          onfront[neigh] = layer;
          nfront++;
          nodes[nfront] = neigh;
        }
      }
    }
    frontend[layer] = nfront;
  }
  int onn = frontend[nlayers];
  free(frontstart); free(frontend); free(onfront);
  return onn;
}

/* ------------------------------------------------------------------ */
/* exact SPD solves: spchol.c (nested dissection + multifrontal         */
/* Cholesky) stands in for UMFPACK's exact LU (Fact.F90:102-159); both   */
/* are exact solves, so results agree to rounding.                      */
/* ------------------------------------------------------------------ */
void *orc_spd_factor(int n, int nnz, const int *ii, const int *jj, const double *vv) {
  char err[256];
  return spchol_factor(n, nnz, ii, jj, vv, err, sizeof err);
}

int orc_spd_solve_factored(void *fact, const double *b, double *x) {
  spchol *f = (spchol *)fact;
  if (!f) return -1;
  double *w = (double *)malloc(sizeof(double) * (size_t)spchol_work_size(f));
  if (!w) return -1;
  spchol_solve(f, b, x, w);
  free(w);
  return 0;
}

void orc_spd_free(void *fact) { spchol_free((spchol *)fact); }

int orc_spd_solve(int n, int nnz, const int *ii, const int *jj, const double *vv,
                  const double *b, double *x) {
  void *f = orc_spd_factor(n, nnz, ii, jj, vv);
  if (!f) return -1;
  int rc = orc_spd_solve_factored(f, b, x);
  orc_spd_free(f);
  return rc;
}

/* ------------------------------------------------------------------ */
/* eigenvalues of the Lanczos tridiagonal: CalculateEigenvalues and the */
/* EISPACK QL method tql1 (pcg.F90:465-641; Bowdler, Martin, Reinsch &  */
/* Wilkinson, Num. Math. 11 (1968) 293-306).                            */
/* ------------------------------------------------------------------ */
static double pythag(double a, double b) {
  double p = fmax(fabs(a), fabs(b)), r, s, t, u;
  if (p == 0.0) return p;
  r = fmin(fabs(a), fabs(b)) / p;
  r = r * r;
  for (;;) {
    t = 4.0 + r;
    if (t == 4.0) break;
    s = r / t;
    u = 1.0 + 2.0 * s;
    p = u * p;
    r = (s / u) * (s / u) * r;
  }
  return p;
}

static int tql1(int n, double *d, double *e) { /* 1-based d, e */
  int i, j, l, m, ii, l1, l2, mml;
  double c, c2, c3 = 0, dl1, el1, f, g, h, p, r, s, s2 = 0, tst1, tst2;
  if (n == 1) return 0;
  for (i = 2; i <= n; i++) e[i - 1] = e[i];
  f = 0.0; tst1 = 0.0; e[n] = 0.0;
  for (l = 1; l <= n; l++) {
    j = 0;
    h = fabs(d[l]) + fabs(e[l]);
    if (tst1 < h) tst1 = h;
    for (m = l; m <= n; m++) {
      tst2 = tst1 + fabs(e[m]);
      if (tst2 == tst1) break;
    }
    if (m > n) m = n;
    if (m != l) {
      do {
        if (j == 30) return l;
        j++;
        l1 = l + 1; l2 = l1 + 1;
        g = d[l];
        p = (d[l1] - g) / (2.0 * e[l]);
        r = pythag(p, 1.0);
        d[l] = e[l] / (p + copysign(r, p));
        d[l1] = e[l] * (p + copysign(r, p));
        dl1 = d[l1];
        h = g - d[l];
        for (i = l2; i <= n; i++) d[i] -= h;
        f += h;
        p = d[m]; c = 1.0; c2 = c; el1 = e[l1]; s = 0.0;
        mml = m - l;
        for (ii = 1; ii <= mml; ii++) {
          c3 = c2; c2 = c; s2 = s;
          i = m - ii;
          g = c * e[i];
          h = c * p;
          r = pythag(p, e[i]);
          e[i + 1] = s * r;
          s = e[i] / r;
          c = p / r;
          p = c * d[i] - s * g;
          d[i + 1] = h + s * (c * g + s * d[i]);
        }
        p = -s * s2 * c3 * el1 * e[l] / dl1;
        e[l] = s * p;
        d[l] = c * p;
        tst2 = tst1 + fabs(e[l]);
      } while (tst2 > tst1);
    }
    p = d[l] + f;
    for (ii = 2; ii <= l; ii++) {
      i = l + 2 - ii;
      if (p >= d[i - 1]) goto found;
      d[i] = d[i - 1];
    }
    i = 1;
  found:
    d[i] = p;
  }
  return 0;
}

static double calc_cond(int it, const double *alpha, const double *beta) {
  if (it < 1) return 0.0;
  double *dd = NEWD(it), *ee = NEWD(it);
  int i;
  dd[1] = 1.0 / alpha[1];
  ee[1] = 0.0;
  for (i = 2; i <= it; i++) {
    if (alpha[i] == 0 || beta[i] < 0) { free(dd); free(ee); return 0.0; }
    dd[i] = 1.0 / alpha[i] + beta[i] / alpha[i - 1];
    ee[i] = -sqrt(beta[i]) / alpha[i - 1];
  }
  tql1(it, dd, ee);
  double c = dd[it] / dd[1];
  free(dd); free(ee);
  return c;
}

/* ------------------------------------------------------------------ */
/* geometric coarse grid of doug_geom on one process                    */
/* (CoarsePreconditioner_geometric.F90:34-115): CreateCoarse           */
/* (coarse/geom/CreateCoarse.f90), the master's own part of SendCoarse  */
/* (coarse/geom/TransmitCoarse.F90:574-799), CreateRestrict             */
/* (coarse/geom/CreateRestrict.F90, GeomInterp.f90) and CleanCoarse     */
/* (CoarseAllgathers.F90:331-507).  One coarse freedom per coarse node  */
/* (CreateCoarseFreemap); no hanging nodes (hanging_nodes .false., the  */
/* default); center_type 1 (box centre) and 2 (clamped mean); the       */
/* random median of center_type 3 is not restated.                     */
/* ------------------------------------------------------------------ */
typedef struct {
  int nsd, nnode, ngf, nell, mfrelt;
  double *coords;       /* coords(d, node) at [(node-1)*nsd + d-1] */
  int *freemap;         /* freemap(f) at [f], 1-based node numbers */
  int *nfrelt;          /* [e], e 1-based */
  int *mhead;           /* mhead(j, e) at [(e-1)*mfrelt + j-1] */
  int nlf, *lg_fmap;    /* local freedom -> global freedom, [l] */
} geom_mesh;

typedef struct { int nfs, n[8], nref, rbeg, lbeg; } cg_elem;           /* CoarseGridElem */
typedef struct { int level, node, next, parent, lbeg, lend; } cg_ref;  /* RefinedElem */
typedef struct {
  int nsd, ncti, nct, elnum, refnum, ngfc, nlfc, mlvl;
  int nc[3];
  double h0[3], minvg[3], maxvg[3];
  double *coords;       /* [(node-1)*nsd + d] */
  cg_elem *els;         /* [1..elnum] */
  cg_ref *refels;       /* [1..refnum] */
  int *elmap;           /* [1..] fine nodes */
} cgrid;

static void cgrid_free(cgrid *C) {
  free(C->coords ? C->coords - 1 : NULL); free(C->els); free(C->refels); free(C->elmap);
  memset(C, 0, sizeof *C);
}

/* BHeap.f90: max-heap of (by, ind); heapify never looks at a lone left child */
typedef struct { int size, cap; int *by, *inds; } bheap;
static void bh_insert(bheap *B, int val, int ind) {
  if (B->size < B->cap) {
    int cur = ++B->size;
    while (cur > 1) {
      if (B->by[cur / 2] >= val) break;
      B->by[cur] = B->by[cur / 2];
      B->inds[cur] = B->inds[cur / 2];
      cur /= 2;
    }
    B->by[cur] = val;
    B->inds[cur] = ind;
  }
}
static void bh_heapify(bheap *B, int cur) {
  int val = B->by[cur], ind = B->inds[cur], bt = cur;
  for (;;) {
    int l = 2 * cur, r = 2 * cur + 1;
    if (r <= B->size) {
      if (B->by[bt] < B->by[l]) bt = l;
      if (B->by[bt] < B->by[r]) bt = r;
    } else if (l < B->size) {
      if (B->by[bt] < B->by[l]) bt = l;
    }
    if (bt == cur) break;
    B->by[cur] = B->by[bt];
    B->inds[cur] = B->inds[bt];
    cur = bt;
    B->by[cur] = val;
  }
  B->inds[cur] = ind;
}
static void bh_delmax(bheap *B) {
  if (B->size >= 1) {
    B->by[1] = B->by[B->size];
    B->inds[1] = B->inds[B->size];
    B->size--;
    bh_heapify(B, 1);
  }
}

#define CGX(C, node) ((C)->coords + (size_t)((node) - 1) * (C)->nsd)
#define MGX(M, node) ((M)->coords + (size_t)((node) - 1) * (M)->nsd)

/* getelem (CoarseGrid.F90:403-424) */
static int cg_getelem(const double *x, const cgrid *C) {
  double rx[3] = {0.0, 0.0, 0.0};
  int i, ind;
  for (i = 0; i < C->nsd; i++) rx[i] = (x[i] - C->minvg[i]) / C->h0[i];
  ind = (int)trunc(rx[0]);
  for (i = 1; i < C->nsd; i++) ind = (int)((double)(ind * (C->nc[i] - 1)) + trunc(rx[i]));
  return ind + 1;
}

/* getDir (CoarseGrid.F90:498-509) on ds = x - c */
static int cg_getdir(const double *x, const double *c, int nsd) {
  int n = 1;
  if (x[0] - c[0] < 0) n += 1;
  if (x[1] - c[1] < 0) n += 2;
  if (nsd == 3 && x[2] - c[2] < 0) n += 4;
  return n;
}

/* getRefBounds (CoarseGrid.F90:427-473) */
static void cg_refbounds(const cgrid *C, int refi, double *minv, double *maxv) {
  int mi[3] = {0, 0, 0}, ma[3] = {0, 0, 0}, k, i;
  const cg_ref *ref = &C->refels[refi];
  const double *ct = CGX(C, ref->node);
  for (k = 0; k < C->nsd; k++) minv[k] = maxv[k] = ct[k];
  while (ref->parent > 0) {
    ref = &C->refels[ref->parent];
    ct = CGX(C, ref->node);
    for (k = 0; k < C->nsd; k++) {
      if (!ma[k] && ct[k] > maxv[k]) { maxv[k] = ct[k]; ma[k] = 1; }
      else if (!mi[k] && ct[k] <= minv[k]) { minv[k] = ct[k]; mi[k] = 1; }
    }
  }
  const cg_elem *el = &C->els[-ref->parent];
  for (i = 0; i < (1 << C->nsd); i++) {
    const double *p = CGX(C, el->n[i]);
    for (k = 0; k < C->nsd; k++) {
      if (!mi[k] && p[k] < minv[k]) { minv[k] = p[k]; mi[k] = 1; }
      else if (!ma[k] && p[k] > maxv[k]) { maxv[k] = p[k]; ma[k] = 1; }
    }
  }
}

/* ChooseGeometricCenter / ChooseMeanCenter with meanpow 1 (CreateCoarse.f90) */
static void cg_center(int type, double *pt, const geom_mesh *M, const int *elmap, int lo, int hi,
                      const double *minv, const double *maxv) {
  int d, i, nsd = M->nsd;
  if (type == 1) {
    for (d = 0; d < nsd; d++) pt[d] = (maxv[d] + minv[d]) / 2.0;
    return;
  }
  for (d = 0; d < nsd; d++) pt[d] = 0.0;
  for (i = lo; i <= hi; i++)
    for (d = 0; d < nsd; d++) pt[d] = pt[d] + MGX(M, elmap[i])[d];
  for (d = 0; d < nsd; d++) pt[d] = pt[d] / (double)(hi - lo + 1);
  for (d = 0; d < nsd; d++) {
    double bval = 0.25 * (maxv[d] - minv[d]);
    if (pt[d] > maxv[d] - bval) pt[d] = maxv[d] - bval;
    else if (pt[d] < minv[d] + bval) pt[d] = minv[d] + bval;
  }
}

/* CreateCoarseMesh + CreateCoarseFreemap (CreateCoarse.f90) */
static void cg_create(const geom_mesh *M, cgrid *C, int maxcie, int maxnd, int cutbal, int ctype) {
  int nsd = M->nsd, tn = 1 << nsd, i, j, k, e, nd, d;
  memset(C, 0, sizeof *C);
  C->nsd = nsd;
  char *inuse = (char *)xcalloc((size_t)M->nnode + 1, 1);
  for (e = 1; e <= M->nell; e++)
    for (j = 1; j <= M->nfrelt[e]; j++) inuse[M->freemap[M->mhead[(size_t)(e - 1) * M->mfrelt + j - 1]]] = 1;
  double ln[3];
  for (d = 0; d < nsd; d++) {
    int first = 1;
    double mn = 0, mx = 0;
    for (nd = 1; nd <= M->nnode; nd++)
      if (inuse[nd]) {
        double v = MGX(M, nd)[d];
        if (first || v < mn) mn = v;
        if (first || v > mx) mx = v;
        first = 0;
      }
    C->minvg[d] = mn;
    C->maxvg[d] = mx;
    ln[d] = C->maxvg[d] - C->minvg[d];
    C->minvg[d] = C->minvg[d] - ln[d] * 0.005;
    C->maxvg[d] = C->maxvg[d] + ln[d] * 0.005;
    ln[d] = ln[d] * 1.01;
  }
  if (nsd == 2) {
    C->nc[0] = (int)round(pow((double)maxcie * (ln[0] / ln[1]), 0.5));
    C->nc[1] = (int)round(pow((double)maxcie * (ln[1] / ln[0]), 0.5));
  } else {
    C->nc[0] = (int)round(pow((double)maxcie * ln[0] * ln[0] / (ln[1] * ln[2]), 0.33));
    C->nc[1] = (int)round(pow((double)maxcie * ln[1] * ln[1] / (ln[0] * ln[2]), 0.33));
    C->nc[2] = (int)round(pow((double)maxcie * ln[2] * ln[2] / (ln[0] * ln[1]), 0.33));
  }
  C->elnum = 1;
  for (d = 0; d < nsd; d++) {
    if (C->nc[d] < 1) C->nc[d] = 1;
    C->h0[d] = ln[d] / (double)C->nc[d];
    C->elnum *= C->nc[d];
  }
  C->ncti = 1;
  for (d = 0; d < nsd; d++) { C->nc[d] += 1; C->ncti *= C->nc[d]; }
  int refmax = maxnd - C->ncti > 0 ? maxnd - C->ncti : 0;
  C->nct = maxnd > C->ncti ? maxnd : C->ncti;
  double *coords = NEWD((size_t)C->nct * nsd);
  C->coords = coords + 1;
  C->els = (cg_elem *)xcalloc((size_t)C->elnum + 1, sizeof(cg_elem));
  C->refels = (cg_ref *)xcalloc((size_t)refmax + 1, sizeof(cg_ref));
  C->elmap = NEWI(M->nnode);
  nd = 1;
  if (nsd == 2) {
    for (i = 0; i <= C->nc[0] - 1; i++)
      for (j = 0; j <= C->nc[1] - 1; j++, nd++) {
        CGX(C, nd)[0] = i * C->h0[0] + C->minvg[0];
        CGX(C, nd)[1] = j * C->h0[1] + C->minvg[1];
      }
  } else {
    for (i = 0; i <= C->nc[0] - 1; i++)
      for (j = 0; j <= C->nc[1] - 1; j++)
        for (k = 0; k <= C->nc[2] - 1; k++, nd++) {
          CGX(C, nd)[0] = i * C->h0[0] + C->minvg[0];
          CGX(C, nd)[1] = j * C->h0[1] + C->minvg[1];
          CGX(C, nd)[2] = k * C->h0[2] + C->minvg[2];
        }
  }
  int el = 1;
  if (nsd == 2) {
    for (i = 1; i <= C->nc[0] - 1; i++)
      for (j = 1; j <= C->nc[1] - 1; j++, el++) {
        cg_elem *E = &C->els[el];
        int nb = (i - 1) * C->nc[1] + j;
        E->nfs = 0; E->nref = 0; E->rbeg = -1;
        E->n[0] = nb; E->n[1] = nb + 1; E->n[2] = nb + C->nc[1]; E->n[3] = nb + C->nc[1] + 1;
      }
  } else {
    for (i = 1; i <= C->nc[0] - 1; i++)
      for (j = 1; j <= C->nc[1] - 1; j++)
        for (k = 1; k <= C->nc[2] - 1; k++, el++) {
          cg_elem *E = &C->els[el];
          int nb = ((i - 1) * C->nc[1] + (j - 1)) * C->nc[2] + k, c3 = C->nc[2], c2 = C->nc[1];
          E->nfs = 0; E->nref = 0; E->rbeg = -1;
          E->n[0] = nb; E->n[1] = nb + 1; E->n[2] = nb + c3; E->n[3] = nb + c3 + 1;
          E->n[4] = nb + c3 * c2; E->n[5] = nb + c3 * c2 + 1;
          E->n[6] = nb + c3 * (c2 + 1); E->n[7] = nb + c3 * (c2 + 1) + 1;
        }
  }
  for (nd = 1; nd <= M->nnode; nd++)
    if (inuse[nd]) C->els[cg_getelem(MGX(M, nd), C)].nfs++;
  C->els[1].lbeg = 1;
  for (i = 2; i <= C->elnum; i++) C->els[i].lbeg = C->els[i - 1].lbeg + C->els[i - 1].nfs;
  for (nd = 1; nd <= M->nnode; nd++)
    if (inuse[nd]) {
      cg_elem *E = &C->els[cg_getelem(MGX(M, nd), C)];
      C->elmap[E->lbeg] = nd;
      E->lbeg++;
    }
  bheap B;
  B.size = 0;
  B.cap = C->elnum + refmax;
  B.by = NEWI(B.cap);
  B.inds = NEWI(B.cap);
  double buf = sqrt((double)nsd);
  C->els[1].lbeg = 1;
  if (C->els[1].nfs > 0) bh_insert(&B, (int)lround(buf * C->els[1].nfs), 1);
  for (i = 2; i <= C->elnum; i++) {
    C->els[i].lbeg = C->els[i - 1].lbeg + C->els[i - 1].nfs;
    if (C->els[i].nfs > 0) bh_insert(&B, (int)lround(buf * C->els[i].nfs), i);
  }
  C->mlvl = 1;
  int refpt = 1, hangpt = C->nct;
  double pt[3], pt2[3], minv[3], maxv[3];
  while (C->ncti + refpt <= hangpt) {
    el = B.inds[1];
    int pcnt = B.by[1];
    bh_delmax(&B);
    if (pcnt <= 2 * cutbal) break;
    if (el <= C->elnum) { /* refine an initial grid element */
      cg_ref *nw = &C->refels[refpt];
      cg_elem *E = &C->els[el];
      nw->level = 1;
      nw->node = C->ncti + refpt;
      nw->parent = -el;
      nw->next = -1;
      nw->lbeg = E->lbeg;
      nw->lend = E->lbeg + E->nfs - 1;
      for (d = 0; d < nsd; d++) { minv[d] = CGX(C, E->n[0])[d]; maxv[d] = CGX(C, E->n[tn - 1])[d]; }
      cg_center(ctype, pt, M, C->elmap, nw->lbeg, nw->lend, minv, maxv);
      for (d = 0; d < nsd; d++) CGX(C, nw->node)[d] = pt[d];
      E->rbeg = refpt;
      bh_insert(&B, E->nfs, C->elnum + refpt);
      refpt++;
    } else { /* refine a refined element */
      int er = el - C->elnum, counts[9] = {0}, flags, cnt;
      cg_ref *nw = &C->refels[refpt], *cur = &C->refels[er];
      nw->level = cur->level + 1;
      nw->node = C->ncti + refpt;
      nw->parent = er;
      for (d = 0; d < nsd; d++) pt[d] = CGX(C, cur->node)[d];
      cg_refbounds(C, er, minv, maxv);
      for (i = cur->lbeg; i <= cur->lend; i++) counts[cg_getdir(MGX(M, C->elmap[i]), pt, nsd)]++;
      flags = 1;
      for (i = 2; i <= tn; i++) if (counts[i] > counts[flags]) flags = i;
      cnt = counts[flags];
      if (cnt <= cutbal) break;
      i = cur->lbeg;
      k = cur->lend;
      for (;;) {
        for (; i <= k; i++) if (cg_getdir(MGX(M, C->elmap[i]), pt, nsd) == flags) break;
        for (; k >= i; k--) if (cg_getdir(MGX(M, C->elmap[k]), pt, nsd) != flags) break;
        if (i >= k) break;
        j = C->elmap[k]; C->elmap[k] = C->elmap[i]; C->elmap[i] = j;
      }
      nw->lbeg = i;
      nw->lend = cur->lend;
      nw->next = cur->next;
      cur->next = refpt;
      cur->lend = i - 1;
      for (d = 0; d < nsd; d++) pt2[d] = MGX(M, C->elmap[nw->lbeg])[d];
      for (d = 0; d < nsd; d++) { /* adjustBounds (CoarseGrid.F90:477-491) */
        if (pt[d] <= pt2[d]) minv[d] = pt[d];
        else maxv[d] = pt[d];
      }
      cg_center(ctype, pt, M, C->elmap, nw->lbeg, nw->lend, minv, maxv);
      for (d = 0; d < nsd; d++) CGX(C, nw->node)[d] = pt[d];
      bh_insert(&B, cnt, C->elnum + refpt);
      bh_insert(&B, pcnt - cnt, C->elnum + er);
      if (C->mlvl < nw->level) C->mlvl = nw->level;
      refpt++;
    }
  }
  free(B.by); free(B.inds);
  C->refnum = refpt - 1;
  C->nct = C->ncti + C->refnum;
  /* drop the grid nodes of empty elements, then number the refinement
   * centres element by element in list order */
  int *remap = (int *)xcalloc((size_t)C->ncti + 1, sizeof(int));
  for (i = 1; i <= C->elnum; i++)
    if (C->els[i].nfs != 0)
      for (k = 0; k < tn; k++) remap[C->els[i].n[k]] = 1;
  int pc = -1;
  for (i = 0; i <= C->ncti; i++) if (remap[i] == 0) pc++;
  C->nct -= pc;
  double *nco = NEWD((size_t)C->nct * nsd);
  double *ncoords = nco + 1;
  if (pc > 0) {
    for (i = 1; i <= C->ncti; i++) {
      if (remap[i] == 1) {
        remap[i] = remap[i - 1] + 1;
        memcpy(ncoords + (size_t)(remap[i] - 1) * nsd, CGX(C, i), sizeof(double) * (size_t)nsd);
      } else {
        remap[i] = remap[i - 1];
      }
    }
    C->ncti -= pc;
    for (i = 1; i <= C->elnum; i++)
      for (k = 0; k < tn; k++) C->els[i].n[k] = C->els[i].nfs > 0 ? remap[C->els[i].n[k]] : 0;
  } else {
    memcpy(ncoords, C->coords, sizeof(double) * (size_t)C->ncti * nsd);
  }
  free(remap);
  k = C->ncti + 1;
  for (i = 1; i <= C->elnum; i++) {
    C->els[i].nref = k;
    j = C->els[i].rbeg;
    while (j != -1) {
      memcpy(ncoords + (size_t)(k - 1) * nsd, CGX(C, C->refels[j].node), sizeof(double) * (size_t)nsd);
      C->refels[j].node = k;
      k++;
      j = C->refels[j].next;
    }
    C->els[i].nref = k - C->els[i].nref;
  }
  free(C->coords - 1);
  C->coords = ncoords;
  C->ngfc = C->nct;
  C->nlfc = C->ngfc;
  free(inuse);
}

/* the master's own part of SendCoarse (TransmitCoarse.F90:574-799) on one
 * process: the local grid LC holds the elements and refinements that own
 * local fine nodes, in the order the local freedoms first reach them.
 * lfreemap[l] (out) = fine node of local freedom l. */
static void cg_local(const geom_mesh *M, const cgrid *C, cgrid *LC, int *lfreemap) {
  int nsd = C->nsd, tn = 1 << nsd, i, j, k, f, nd;
  int *ndtoel = NEWI(M->nnode);
  for (int el = 1; el <= C->elnum; el++) {
    const cg_elem *E = &C->els[el];
    if (E->rbeg <= 0) {
      for (j = E->lbeg; j <= E->lbeg + E->nfs - 1; j++) ndtoel[C->elmap[j]] = -el;
    } else {
      for (j = E->rbeg; j > 0; j = C->refels[j].next)
        for (k = C->refels[j].lbeg; k <= C->refels[j].lend; k++) ndtoel[C->elmap[k]] = j;
    }
  }
  char *refmask = (char *)xcalloc((size_t)C->refnum + 1, 1), *elmask = (char *)xcalloc((size_t)C->elnum + 1, 1);
  char *have = (char *)xcalloc((size_t)M->nnode + 1, 1);
  int *ellist = NEWI(C->elnum);
  memset(LC, 0, sizeof *LC);
  LC->nsd = nsd;
  int lnnode = 0;
  for (i = 1; i <= M->nlf; i++) {
    f = M->lg_fmap[i];
    nd = M->freemap[f];
    if (ndtoel[nd] != 0) {
      lfreemap[i] = nd;
      if (!have[nd]) { lnnode++; have[nd] = 1; }
      k = ndtoel[nd];
      while (k > 0) {
        if (refmask[k]) break;
        refmask[k] = 1;
        LC->refnum++;
        k = C->refels[k].parent;
      }
      if (k < 0 && !elmask[-k]) {
        ellist[++LC->elnum] = -k;
        elmask[-k] = 1;
      }
    } else {
      lfreemap[i] = 0;
    }
  }
  int *gl_c = NEWI(C->nct), *lg_c = NEWI(C->nct);
  LC->ncti = 0;
  for (i = 1; i <= LC->elnum; i++)
    for (j = 0; j < tn; j++) {
      int cn = C->els[ellist[i]].n[j];
      if (gl_c[cn] == 0) { gl_c[cn] = ++LC->ncti; lg_c[LC->ncti] = cn; }
    }
  k = LC->ncti + 1;
  for (i = 1; i <= LC->elnum; i++)
    for (j = C->els[ellist[i]].rbeg; j != -1; j = C->refels[j].next)
      if (refmask[j]) { gl_c[C->refels[j].node] = k; lg_c[k] = C->refels[j].node; k++; }
  LC->nct = LC->ncti + LC->refnum;
  LC->ngfc = C->ngfc;
  LC->mlvl = C->mlvl;
  LC->nlfc = LC->nct; /* one freedom per coarse node */
  double *co = NEWD((size_t)LC->nct * nsd);
  LC->coords = co + 1;
  for (i = 1; i <= LC->nct; i++) memcpy(CGX(LC, i), CGX(C, lg_c[i]), sizeof(double) * (size_t)nsd);
  LC->els = (cg_elem *)xcalloc((size_t)LC->elnum + 1, sizeof(cg_elem));
  LC->refels = (cg_ref *)xcalloc((size_t)LC->refnum + 1, sizeof(cg_ref));
  LC->elmap = NEWI(lnnode);
  nd = 1;
  int rel = 1, pstack[64];
  for (f = 1; f <= LC->elnum; f++) {
    const cg_elem *E = &C->els[ellist[f]];
    cg_elem *L = &LC->els[f];
    L->nref = E->nref;
    for (j = 0; j < tn; j++) L->n[j] = gl_c[E->n[j]];
    L->lbeg = nd;
    L->nfs = 0;
    i = E->rbeg;
    if (i == -1) {
      L->rbeg = -1;
      for (j = E->lbeg; j <= E->lbeg + E->nfs - 1; j++)
        if (have[C->elmap[j]]) { L->nfs++; LC->elmap[nd++] = C->elmap[j]; }
    } else {
      int last = 0;
      L->rbeg = rel;
      pstack[0] = -f;
      while (i != -1) {
        const cg_ref *old = &C->refels[i];
        if (refmask[i]) {
          cg_ref *r = &LC->refels[rel];
          if (old->level >= 64) orc_abort("refinement deeper than 63 levels");
          r->level = old->level;
          r->node = gl_c[old->node];
          r->parent = pstack[r->level - 1];
          r->next = rel + 1;
          r->lbeg = nd;
          for (j = old->lbeg; j <= old->lend; j++)
            if (have[C->elmap[j]]) { L->nfs++; LC->elmap[nd++] = C->elmap[j]; }
          r->lend = nd - 1;
          pstack[r->level] = rel;
          last = rel;
          rel++;
        }
        i = old->next;
      }
      LC->refels[last].next = -1;
    }
  }
  free(ndtoel); free(refmask); free(elmask); free(have); free(ellist); free(gl_c); free(lg_c);
}

/* BuildMults (GeomInterp.f90:472-560): coefficients of the multilinear
 * polynomial of every coarse node over the box [minv, maxv].
 * coefs(corner, col) at [(col-1)*tn + corner-1]; mults(row, col) likewise. */
static void cg_buildmults(const double *minv, const double *maxv, const double *coefs, int csz, int nsd,
                          int ncols, double *mults) {
  int tn = 1 << nsd, i, r, c;
  double mbuf[8], prd = 1.0, fm[8];
  for (i = 0; i < tn * ncols; i++) mults[i] = 0.0;
  for (i = 0; i < nsd; i++) prd = prd * (maxv[i] - minv[i]);
  prd = 1.0 / prd;
  for (c = 1; c <= tn; c++) {
    if (nsd == 2) {
      switch (c) {
        case 1: mbuf[0] = minv[0] * minv[1]; mbuf[1] = -minv[1]; mbuf[2] = -minv[0]; mbuf[3] = 1.0; break;
        case 2: mbuf[0] = -(maxv[0] * minv[1]); mbuf[1] = minv[1]; mbuf[2] = maxv[0]; mbuf[3] = -1.0; break;
        case 3: mbuf[0] = -(minv[0] * maxv[1]); mbuf[1] = maxv[1]; mbuf[2] = minv[0]; mbuf[3] = -1.0; break;
        default: mbuf[0] = maxv[0] * maxv[1]; mbuf[1] = -maxv[1]; mbuf[2] = -maxv[0]; mbuf[3] = 1.0; break;
      }
    } else {
      /* corner c: signs of the factors (x - bound) and the sign of the term */
      static const int usemax[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                       {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
      static const int negf[8] = {1, 0, 0, 1, 0, 1, 1, 0}; /* factors negated, quotients kept */
      for (i = 0; i < 3; i++) {
        double b = usemax[c - 1][i] ? maxv[i] : minv[i];
        fm[i] = negf[c - 1] ? -b : b;
      }
      mbuf[4] = fm[0]; mbuf[5] = fm[1]; mbuf[6] = fm[2];
      mbuf[0] = mbuf[4] * mbuf[5] * mbuf[6];
      if (negf[c - 1]) {
        for (i = 0; i < 3; i++) mbuf[1 + i] = mbuf[0] / mbuf[4 + i];
        mbuf[7] = 1.0;
      } else {
        for (i = 0; i < 3; i++) mbuf[1 + i] = -mbuf[0] / mbuf[4 + i];
        mbuf[7] = -1.0;
      }
    }
    for (r = 0; r < tn; r++) mbuf[r] = mbuf[r] * prd;
    for (i = 1; i <= csz; i++)
      for (r = 0; r < tn; r++)
        mults[(size_t)(i - 1) * tn + r] = mults[(size_t)(i - 1) * tn + r] + coefs[(size_t)(i - 1) * tn + c - 1] * mbuf[r];
  }
}

/* MlinInterpolate (GeomInterp.f90:563-582) */
static double cg_interp(const double *p, int nsd, const double *m) {
  if (nsd == 2) return m[0] + m[1] * p[0] + m[2] * p[1] + m[3] * p[0] * p[1];
  return m[0] + m[1] * p[0] + m[2] * p[1] + m[3] * p[2] + m[4] * p[1] * p[2] + m[5] * p[0] * p[2] +
         m[6] * p[0] * p[1] + m[7] * p[0] * p[1] * p[2];
}

/* CalcNextCoefs (GeomInterp.f90:244-468) without hanging nodes: corner
 * coefficients of the sub-box of [minv, maxv] cut at the centre ct towards
 * pt, in terms of the coarse nodes cinds (+ the centre ci). */
static void cg_nextcoefs(const double *ct, int ci, const double *minv, const double *maxv, const double *coefs,
                         const int *cinds, int csz, int nsd, const double *pt, double *cfout, int *ciout,
                         int *ncsz_out) {
  int tn = 1 << nsd, i, k, r, ncnt = 1, ncsz, dir = 1, drev = 1, rev[3], nc[8], ni[8];
  double m[3];
#define CF(a, col) coefs[(size_t)((col) - 1) * tn + (a) - 1]
#define CO(a, col) cfout[(size_t)((col) - 1) * tn + (a) - 1]
  for (i = 0; i < nsd; i++) m[i] = (maxv[i] - ct[i]) / (maxv[i] - minv[i]);
  ncsz = csz;
  for (i = 1; i <= csz; i++) ciout[i - 1] = cinds[i - 1];
  k = 1;
  for (i = 0; i < nsd; i++) {
    if (pt[i] < ct[i]) { dir += k; rev[i] = -k; }
    else { drev += k; rev[i] = k; }
    k *= 2;
  }
  for (i = 1; i <= csz; i++) CO(dir, i) = CF(dir, i);
  for (i = 1; i <= csz; i++) CO(drev, i) = 0.0;
  nc[0] = drev;
  ni[0] = ci;
  if (nsd == 2) {
    for (r = 0; r < 2; r++) {
      int a = drev - rev[r];
      for (i = 1; i <= csz; i++) {
        if (rev[r] > 0) CO(a, i) = m[r] * CF(a, i) + (1 - m[r]) * CF(dir, i);
        else CO(a, i) = m[r] * CF(dir, i) + (1 - m[r]) * CF(a, i);
      }
    }
  } else {
    for (r = 0; r < 3; r++) {
      int a = dir + rev[r];
      for (i = 1; i <= csz; i++) {
        if (rev[r] > 0) CO(a, i) = m[r] * CF(a, i) + (1 - m[r]) * CF(dir, i);
        else CO(a, i) = m[r] * CF(dir, i) + (1 - m[r]) * CF(a, i);
      }
    }
    /* face centres: bilinear in the two other directions */
    static const int o1[3] = {1, 0, 0}, o2[3] = {2, 2, 1}, s1[3] = {2, 1, 1}, s2[3] = {4, 4, 2};
    for (r = 0; r < 3; r++) {
      int a = drev - rev[r], kk = (-rev[r] > 0 ? -rev[r] : 0) + 1;
      double p = m[o1[r]], q = m[o2[r]];
      for (i = 1; i <= csz; i++)
        CO(a, i) = p * q * CF(kk, i) + p * (1 - q) * CF(kk + s2[r], i) + (1 - p) * q * CF(kk + s1[r], i) +
                   (1 - p) * (1 - q) * CF(kk + s1[r] + s2[r], i);
    }
  }
  /* put the new centre into a column whose coefficients all vanished, or
   * close the gap with the last column */
  int n0 = ncsz;
  for (i = n0; i >= 1; i--) {
    int allz = 1;
    for (r = 1; r <= tn; r++) if (CO(r, i) != 0.0) { allz = 0; break; }
    if (!allz) continue;
    if (ncnt > 0) {
      CO(nc[ncnt - 1], i) = 1.0;
      ciout[i - 1] = ni[ncnt - 1];
      ncnt--;
    } else {
      for (r = 1; r <= tn; r++) CO(r, i) = CO(r, ncsz);
      ciout[i - 1] = ciout[ncsz - 1];
      ncsz--;
    }
  }
  for (i = 1; i <= ncnt; i++) {
    ncsz++;
    for (r = 1; r <= tn; r++) CO(r, ncsz) = 0.0;
    CO(nc[i - 1], ncsz) = 1.0;
    ciout[ncsz - 1] = ni[i - 1];
  }
  *ncsz_out = ncsz;
#undef CF
#undef CO
}

typedef struct { int n, cap; int *i, *j; double *v; } coo_buf;
static void coo_push(coo_buf *b, int i, int j, double v) {
  if (b->n == b->cap) {
    b->cap = b->cap ? 2 * b->cap : 1024;
    b->i = (int *)realloc(b->i, sizeof(int) * (size_t)(b->cap + 1));
    b->j = (int *)realloc(b->j, sizeof(int) * (size_t)(b->cap + 1));
    b->v = (double *)realloc(b->v, sizeof(double) * (size_t)(b->cap + 1));
    if (!b->i || !b->j || !b->v) orc_abort("out of memory");
  }
  b->n++;
  b->i[b->n] = i; b->j[b->n] = j; b->v[b->n] = v;
}

/* CalcMlinearInterp (GeomInterp.f90:585-825): node prolongation entries
 * (fine node, coarse node, value), fine node after fine node in element and
 * list order */
static void cg_mlinear(const cgrid *C, const geom_mesh *M, coo_buf *NP) {
  int nsd = C->nsd, tn = 1 << nsd, L = C->mlvl, maxc = tn + C->mlvl + nsd, i, j, k, l, d;
  double *mins = NEWD((size_t)nsd * (L + 1)), *maxs = NEWD((size_t)nsd * (L + 1));
  double *coefs = NEWD((size_t)tn * maxc * L), *curcfs = NEWD((size_t)tn * maxc * tn);
  double *finals = NEWD((size_t)tn * maxc * tn), *mults = NEWD((size_t)tn * maxc);
  int *cinds = NEWI((size_t)maxc * L), *cszs = NEWI(L), *curcis = NEWI((size_t)maxc * tn), curcsz[9];
  char have[9];
#define MN(lv) (mins + 1 + (size_t)((lv) - 1) * nsd)
#define MX(lv) (maxs + 1 + (size_t)((lv) - 1) * nsd)
#define COEF(lv) (coefs + 1 + (size_t)((lv) - 1) * tn * maxc)
#define CIND(lv) (cinds + 1 + (size_t)((lv) - 1) * maxc)
#define CURC(dd) (curcfs + 1 + (size_t)((dd) - 1) * tn * maxc)
#define CURI(dd) (curcis + 1 + (size_t)((dd) - 1) * maxc)
#define FIN(dd) (finals + 1 + (size_t)((dd) - 1) * tn * maxc)
  static const int c2[4] = {4, 2, 3, 1}, c3[8] = {8, 4, 6, 2, 7, 3, 5, 1};
  for (i = 1; i <= C->elnum; i++) {
    const cg_elem *E = &C->els[i];
    for (d = 0; d < nsd; d++) { MN(1)[d] = CGX(C, E->n[0])[d]; MX(1)[d] = CGX(C, E->n[tn - 1])[d]; }
    cszs[1] = tn;
    for (l = 0; l < tn; l++) CIND(1)[l] = E->n[l];
    for (l = 0; l < tn * tn; l++) COEF(1)[l] = 0.0;
    /* corner a of the box is the coarse node in column c(a) (getDir order) */
    for (l = 0; l < tn; l++) {
      int col = nsd == 2 ? c2[l] : c3[l];
      COEF(1)[(size_t)(col - 1) * tn + l] = 1.0;
    }
    if (E->rbeg == -1) {
      cg_buildmults(MN(1), MX(1), COEF(1), cszs[1], nsd, maxc, mults + 1);
      for (j = E->lbeg; j <= E->lbeg + E->nfs - 1; j++) {
        int pn = C->elmap[j];
        for (l = 1; l <= cszs[1]; l++)
          coo_push(NP, pn, CIND(1)[l - 1], cg_interp(MGX(M, pn), nsd, mults + 1 + (size_t)(l - 1) * tn));
      }
      continue;
    }
    for (j = E->rbeg; j != -1; j = C->refels[j].next) {
      const cg_ref *R = &C->refels[j];
      int lvl;
      if (R->parent > 0) {
        int ci = C->refels[R->parent].node;
        const double *ct = CGX(C, ci), *pt = CGX(C, R->node);
        lvl = R->level - 1;
        cg_nextcoefs(ct, ci, MN(lvl), MX(lvl), COEF(lvl), CIND(lvl), cszs[lvl], nsd, pt, COEF(lvl + 1),
                     CIND(lvl + 1), &cszs[lvl + 1]);
        for (d = 0; d < nsd; d++) {
          if (ct[d] <= pt[d]) { MN(lvl + 1)[d] = ct[d]; MX(lvl + 1)[d] = MX(lvl)[d]; }
          else { MN(lvl + 1)[d] = MN(lvl)[d]; MX(lvl + 1)[d] = ct[d]; }
        }
      }
      int ci = R->node;
      const double *ct = CGX(C, ci);
      lvl = R->level;
      if (R->lbeg > R->lend) continue;
      memset(have, 0, sizeof have);
      for (k = R->lbeg; k <= R->lend; k++) {
        int pn = C->elmap[k];
        const double *pt = MGX(M, pn);
        int dd = cg_getdir(pt, ct, nsd);
        if (!have[dd]) {
          cg_nextcoefs(ct, ci, MN(lvl), MX(lvl), COEF(lvl), CIND(lvl), cszs[lvl], nsd, pt, CURC(dd), CURI(dd),
                       &curcsz[dd]);
          for (d = 0; d < nsd; d++) {
            if (ct[d] <= pt[d]) { MN(lvl + 1)[d] = ct[d]; MX(lvl + 1)[d] = MX(lvl)[d]; }
            else { MN(lvl + 1)[d] = MN(lvl)[d]; MX(lvl + 1)[d] = ct[d]; }
          }
          cg_buildmults(MN(lvl + 1), MX(lvl + 1), CURC(dd), curcsz[dd], nsd, maxc, FIN(dd));
          have[dd] = 1;
        }
        for (l = 1; l <= curcsz[dd]; l++)
          coo_push(NP, pn, CURI(dd)[l - 1], cg_interp(pt, nsd, FIN(dd) + (size_t)(l - 1) * tn));
      }
    }
  }
#undef MN
#undef MX
#undef COEF
#undef CIND
#undef CURC
#undef CURI
#undef FIN
  free(mins); free(maxs); free(coefs); free(curcfs); free(finals); free(mults);
  free(cinds); free(cszs); free(curcis);
}

/* CreatePathRestrict's node prolongation (CreateRestrict.F90:95-213) for
 * interpolation_type 2 (inverse distance) and 3 (the reference's kriging,
 * which returns the distances themselves): rows by fine node number, every
 * node weighted against its element's corners and the refinement centres
 * on its path. */
static void cg_path(const cgrid *C, const geom_mesh *M, int itype, coo_buf *NP) {
  int nsd = C->nsd, tn = 1 << nsd, i, j, k, q, d;
  int *start = NEWI(M->nnode + 1);
  for (i = 1; i <= C->elnum; i++)
    if (C->els[i].rbeg == -1)
      for (j = C->els[i].lbeg; j <= C->els[i].lbeg + C->els[i].nfs - 1; j++) start[C->elmap[j] + 1] = tn;
  for (i = 1; i <= C->refnum; i++)
    for (j = C->refels[i].lbeg; j <= C->refels[i].lend; j++) start[C->elmap[j] + 1] = tn + C->refels[i].level;
  start[1] = 1;
  for (i = 1; i <= M->nnode; i++) start[i + 1] = start[i] + start[i + 1];
  int tot = start[M->nnode + 1] - 1;
  NP->n = NP->cap = tot;
  NP->i = NEWI(tot); NP->j = NEWI(tot); NP->v = NEWD(tot);
  double *pts = NEWD((size_t)nsd * (tn + C->mlvl));
  int *pinds = NEWI(tn + C->mlvl);
  double *w = NEWD(tn + C->mlvl);
  for (i = 1; i <= C->elnum; i++) {
    const cg_elem *E = &C->els[i];
    for (k = 0; k < tn; k++) {
      memcpy(pts + 1 + (size_t)k * nsd, CGX(C, E->n[k]), sizeof(double) * (size_t)nsd);
      pinds[k + 1] = E->n[k];
    }
    int lo0 = E->lbeg, hi0 = E->lbeg + E->nfs - 1, csz = tn, rj = E->rbeg;
    for (;;) {
      int lo, hi;
      if (E->rbeg == -1) { lo = lo0; hi = hi0; }
      else {
        if (rj == -1) break;
        const cg_ref *R = &C->refels[rj];
        csz = tn + R->level;
        memcpy(pts + 1 + (size_t)(csz - 1) * nsd, CGX(C, R->node), sizeof(double) * (size_t)nsd);
        pinds[csz] = R->node;
        lo = R->lbeg; hi = R->lend;
        rj = R->next;
      }
      for (j = lo; j <= hi; j++) {
        int pn = C->elmap[j];
        const double *x = MGX(M, pn);
        for (q = 1; q <= csz; q++) {
          double s = 0.0;
          for (d = 0; d < nsd; d++) {
            double t = pts[1 + (size_t)(q - 1) * nsd + d] - x[d];
            s = s + t * t;
          }
          w[q] = pow(s, 0.5);
        }
        if (itype == 2) { /* getInvDistVals (CreateRestrict.F90:232-251) */
          for (q = 1; q <= csz; q++) {
            if (w[q] <= 1.0e-9) {
              for (k = 1; k <= csz; k++) w[k] = 0.0;
              w[q] = 1.0;
              break;
            }
            w[q] = 1.0 / w[q];
          }
          double sum = 0.0;
          for (q = 1; q <= csz; q++) sum = sum + w[q];
          for (q = 1; q <= csz; q++) w[q] = w[q] / sum;
        }
        for (q = 1; q <= csz; q++) {
          int at = start[pn] + q - 1;
          NP->i[at] = pn; NP->j[at] = pinds[q]; NP->v[at] = w[q];
        }
      }
      if (E->rbeg == -1) break;
    }
  }
  free(start); free(pts); free(pinds); free(w);
}

/* CoarsePreconditioner_geometric_Init (CoarsePreconditioner_geometric.F90:
 * 34-115) up to CoarseMtxBuild, one process: the restriction R (local coarse
 * freedoms x local fine freedoms) in the reference's entry order, arranged
 * by columns; entries <= eps = 1e-9 dropped (GeomInterp.f90:200-214). */
static spm geom_restriction(const geom_mesh *M, const ctl_t *c, double **cxyz) {
  int maxcie = c->maxcie == -1 ? 75 : c->maxcie, maxnd = c->maxnd == -1 ? 500 : c->maxnd;
  int cutbal = c->cutbal <= 0 ? 1 : c->cutbal, ctype = c->center_type == -1 ? 1 : c->center_type;
  int itype = c->interpolation_type == -1 ? 1 : c->interpolation_type, i, j, k;
  if (M->nsd != 2 && M->nsd != 3) orc_abort("the geometric coarse grid needs 2-D or 3-D coordinates (nsd %d)", M->nsd);
  if (c->hanging_nodes) orc_abort("hanging_nodes: not restated");
  if (ctype != 1 && ctype != 2) orc_abort("No such center choosing method");
  if (itype < 1 || itype > 3) orc_abort("interpolation_type %d", itype);
  cgrid C, LC;
  cg_create(M, &C, maxcie, maxnd, cutbal, ctype);
  int *lfreemap = NEWI(M->nlf);
  cg_local(M, &C, &LC, lfreemap);
  cgrid_free(&C);
  coo_buf NP;
  memset(&NP, 0, sizeof NP);
  int *lb = NEWI(M->nnode), *ub = NEWI(M->nnode);
  if (itype == 1) { /* CreateGeneralRestrict (GeomInterp.f90:77-241) */
    cg_mlinear(&LC, M, &NP);
    if (NP.n > 0) {
      lb[NP.i[1]] = 1;
      for (k = 2; k <= NP.n; k++)
        if (NP.i[k - 1] != NP.i[k]) {
          if (ub[NP.i[k - 1]] != 0 || lb[NP.i[k]] != 0) orc_abort("Node restriction matrix not consolidated");
          ub[NP.i[k - 1]] = k - 1;
          lb[NP.i[k]] = k;
        }
      ub[NP.i[NP.n]] = NP.n;
    }
  } else { /* CreatePathRestrict: rows by fine node number */
    cg_path(&LC, M, itype, &NP);
    for (i = 1; i <= M->nnode; i++) { lb[i] = 0; ub[i] = -1; }
    for (k = 1; k <= NP.n; k++) {
      if (lb[NP.i[k]] == 0) lb[NP.i[k]] = k;
      ub[NP.i[k]] = k;
    }
  }
  coo_buf Rb;
  memset(&Rb, 0, sizeof Rb);
  for (i = 1; i <= M->nlf; i++) {
    int nd = lfreemap[i];
    if (nd == 0) continue;
    for (j = lb[nd]; j <= ub[nd] && j >= 1; j++)
      if (NP.v[j] > 1.0e-9) coo_push(&Rb, NP.j[j], i, NP.v[j]);
  }
  free(NP.i); free(NP.j); free(NP.v); free(lb); free(ub); free(lfreemap);
  /* CleanCoarse (CoarseAllgathers.F90:331-507), one process: coarse
   * freedoms that no entry of R uses are dropped, the rest renumbered in
   * order */
  int *used = NEWI(LC.nlfc);
  for (k = 1; k <= Rb.n; k++) used[Rb.i[k]] = 1;
  int nk = 0;
  for (i = 1; i <= LC.nlfc; i++) used[i] = used[i] ? ++nk : 0;
  spm R = spm_new(Rb.n, nk, M->nlf);
  for (k = 1; k <= Rb.n; k++) { R.indi[k] = used[Rb.i[k]]; R.indj[k] = Rb.j[k]; R.val[k] = Rb.v[k]; }
  *cxyz = (double *)xcalloc((size_t)nk * M->nsd + 1, sizeof(double));
  for (i = 1; i <= LC.nlfc; i++)
    if (used[i]) memcpy(*cxyz + (size_t)(used[i] - 1) * M->nsd, CGX(&LC, i), sizeof(double) * (size_t)M->nsd);
  free(used); free(Rb.i); free(Rb.j); free(Rb.v);
  cgrid_free(&LC);
  return R;
}

/* ------------------------------------------------------------------ */
/* the whole np=1 path                                                  */
/* ------------------------------------------------------------------ */
typedef struct {
  ctl_t ctl;
  spm A;
  double *rhs;
  int n;
  aggrs fine_inner, fine_full, coarse_inner, coarse_full;
  int have_coarse;
  spm R, AC;
  int have_R;
  int nsubd;
  int *sd_start, *sd_nodes; /* 0-based starts, 1-based node ids */
  int ol;
  double strong1, strong2;
  int r1, r2, min1, max1, min2, max2;
  const geom_mesh *geom; /* node coordinates of elemental input, or NULL */
  spm Rs, ACs;            /* the coarse level the solve uses when it differs from R, AC */
  int have_sub;
  int cnsd;
  double *cxyz;           /* coarse freedom coordinates (doug_geom) */
} state;

static void state_free(state *s) {
  spm_free(&s->A); free(s->rhs);
  aggrs_free(&s->fine_inner); aggrs_free(&s->fine_full);
  aggrs_free(&s->coarse_inner); aggrs_free(&s->coarse_full);
  spm_free(&s->R); spm_free(&s->AC);
  spm_free(&s->Rs); spm_free(&s->ACs); free(s->cxyz);
  free(s->sd_start); free(s->sd_nodes);
}

/* The multilinear basis functions of a geometric coarse grid can be
 * linearly dependent on the fine nodes (a coarse element whose fine nodes
 * lie on one line): AC is then singular but consistent, and the
 * reference's LU solve (UMFPACK with pivoting) returns one of its
 * solutions, whose prolongation R^T y is the same for all of them.  The
 * solve here keeps the coarse freedoms whose Cholesky pivot (natural order,
 * dependent ones skipped) stays above 1e-10 of their diagonal and solves on
 * those: the same projection onto the range of R^T.  Coarse levels of more
 * than 4000 freedoms are kept whole. */
static void geom_independent_coarse(state *s) {
  int nc = s->AC.nrows, i, j, k;
  if (nc <= 0 || nc > 4000) return;
  double *a = (double *)xcalloc((size_t)nc * nc, sizeof(double));
  for (k = 1; k <= s->AC.nnz; k++)
    a[(size_t)(s->AC.indi[k] - 1) * nc + (s->AC.indj[k] - 1)] = a[(size_t)(s->AC.indi[k] - 1) * nc + (s->AC.indj[k] - 1)] + s->AC.val[k];
  int *keep = NEWI(nc), nk = 0;
  for (j = 0; j < nc; j++) {
    double d = a[(size_t)j * nc + j], d0 = d;
    for (k = 0; k < j; k++) if (keep[k + 1]) d = d - a[(size_t)j * nc + k] * a[(size_t)j * nc + k];
    if (!(d > 1.0e-10 * d0)) {
      for (i = j; i < nc; i++) a[(size_t)i * nc + j] = 0.0;
      continue;
    }
    keep[j + 1] = ++nk;
    double l = sqrt(d);
    a[(size_t)j * nc + j] = l;
    for (i = j + 1; i < nc; i++) {
      double t = a[(size_t)i * nc + j];
      for (k = 0; k < j; k++) if (keep[k + 1]) t = t - a[(size_t)i * nc + k] * a[(size_t)j * nc + k];
      a[(size_t)i * nc + j] = t / l;
    }
  }
  free(a);
  if (nk == nc) { free(keep); return; }
  int nr = 0, na = 0;
  for (k = 1; k <= s->R.nnz; k++) if (keep[s->R.indi[k]]) nr++;
  for (k = 1; k <= s->AC.nnz; k++) if (keep[s->AC.indi[k]] && keep[s->AC.indj[k]]) na++;
  s->Rs = spm_new(nr, nk, s->R.ncols);
  s->ACs = spm_new(na, nk, nk);
  nr = na = 0;
  for (k = 1; k <= s->R.nnz; k++)
    if (keep[s->R.indi[k]]) { nr++; s->Rs.indi[nr] = keep[s->R.indi[k]]; s->Rs.indj[nr] = s->R.indj[k]; s->Rs.val[nr] = s->R.val[k]; }
  for (k = 1; k <= s->AC.nnz; k++)
    if (keep[s->AC.indi[k]] && keep[s->AC.indj[k]]) {
      na++;
      s->ACs.indi[na] = keep[s->AC.indi[k]]; s->ACs.indj[na] = keep[s->AC.indj[k]]; s->ACs.val[na] = s->AC.val[k];
    }
  s->have_sub = 1;
  free(keep);
}

/* main_geom (geom.F90:62-116) on one process: no aggregation; one
 * subdomain of all nodes (Partitionings_full_InitCoarse,
 * Partitioning_full.F90:32-47) or the imported parts, with ol layers
 * (FinePreconditioner_Init arranges A by rows); with elemental input and
 * levels 2 the geometric coarse grid gives R, and AC = R A R^T in the local
 * coarse numbering (the one-process allgather only renumbers it). */
static void run_setup_geom(state *s, const int *part, int nparts) {
  ctl_t *c = &s->ctl;
  int n = s->n, i, ip;
  s->fine_inner.n = s->fine_full.n = n;
  s->fine_inner.num = NEWI(n);
  s->fine_full.num = NEWI(n);
  s->ol = (c->overlap < 0) ? (c->smoothers > 0 ? c->smoothers : 0) : c->overlap;
  c->fine_method = 1; /* main_geom always applies exact subdomain solves (geom.F90:101-102) */
  if (c->levels > 2) orc_abort("doug_geom builds no coarse level for levels %d", c->levels);
  if (c->levels == 2 && (c->input_type != 1 || !s->geom))
    orc_abort("the geometric coarse grid needs elemental input with node coordinates");
  spm_arrange(&s->A, ARR_ROWS, 0, 0, 0, 0);
  int *nodes = NEWI(n);
  int np = part ? nparts : 1;
  s->nsubd = np;
  s->sd_start = (int *)xcalloc((size_t)np + 2, sizeof(int));
  long cap = 4L * n + 16, fill = 0;
  s->sd_nodes = (int *)xcalloc((size_t)cap, sizeof(int));
  for (ip = 1; ip <= np; ip++) {
    int nnodes = 0;
    for (i = 1; i <= n; i++)
      if (!part || part[i - 1] == ip) nodes[++nnodes] = i;
    int nexp = add_layers(s->A.mbound, s->A.indj, nodes, nnodes, s->ol, n);
    if (fill + nexp > cap) {
      cap = 2 * (fill + nexp);
      s->sd_nodes = (int *)realloc(s->sd_nodes, sizeof(int) * (size_t)cap);
      if (!s->sd_nodes) orc_abort("out of memory");
    }
    s->sd_start[ip - 1] = (int)fill;
    memcpy(s->sd_nodes + fill, nodes + 1, sizeof(int) * (size_t)nexp);
    fill += nexp;
  }
  s->sd_start[np] = (int)fill;
  free(nodes);
  if (c->levels == 2) {
    c->smoothers = 0; /* CoarsePreconditioner_geometric.F90:53 */
    s->R = geom_restriction(s->geom, c, &s->cxyz);
    s->cnsd = s->geom->nsd;
    s->have_R = 1;
    s->AC = coarse_mtx_build(&s->A, &s->R, n, 0);
    geom_independent_coarse(s);
  }
}

/* aggr.F90:131-215 for numprocs==1 (or an imported partition). */
/* Node geometry for coarse_method 3 (orc_set_geometry): the 1-based mesh
 * node of every unknown and the node coordinates (nsd per node). */
static int g_geo_nsd = 0, g_geo_n = 0, g_geo_nnode = 0;
static int *g_geo_unode = NULL;
static double *g_geo_xyz = NULL;

void orc_set_geometry(int nsd, int nnode, const double *coords, int n, const int *unode) {
  free(g_geo_unode); free(g_geo_xyz);
  g_geo_unode = NULL; g_geo_xyz = NULL;
  g_geo_nsd = 0; g_geo_n = 0; g_geo_nnode = 0;
  if (nsd <= 0 || !coords || !unode) return;
  g_geo_nsd = nsd; g_geo_n = n; g_geo_nnode = nnode;
  g_geo_unode = (int *)malloc(sizeof(int) * ((size_t)n + 1));
  g_geo_xyz = (double *)malloc(sizeof(double) * ((size_t)nsd * nnode + 1));
  memcpy(g_geo_unode + 1, unode, sizeof(int) * (size_t)n);
  memcpy(g_geo_xyz, coords, sizeof(double) * (size_t)nsd * nnode);
}

/* The three aggregation passes of smoothed aggregation on a weighted graph
 * (1-based: vertex v's neighbours col[ptr[v]..ptr[v+1]-1], weights val,
 * strong flags): (1) a vertex whose strong neighbours are all free starts an
 * aggregate with them; (2) a free vertex joins the phase-1 aggregate of its
 * strongest aggregated strong neighbour (first on ties); (3) the vertices
 * still free start aggregates with their free strong neighbours.  agg[v]:
 * 1-based aggregate; returns their number. */
static int three_phase(int nv, const int *ptr, const int *col, const double *val, const char *strong, int *agg) {
  int k, i, na = 0;
  int *agg1 = NEWI(nv);
  for (k = 1; k <= nv; k++) agg[k] = 0;
  for (k = 1; k <= nv; k++) {
    int freeall = 1;
    if (agg[k]) continue;
    for (i = ptr[k]; i < ptr[k + 1]; i++)
      if (strong[i] && col[i] != k && agg[col[i]]) { freeall = 0; break; }
    if (!freeall) continue;
    na++;
    agg[k] = na;
    for (i = ptr[k]; i < ptr[k + 1]; i++)
      if (strong[i]) agg[col[i]] = na;
  }
  for (k = 1; k <= nv; k++) agg1[k] = agg[k];
  for (k = 1; k <= nv; k++) {
    int best = 0;
    double bv = 0.0;
    if (agg1[k]) continue;
    for (i = ptr[k]; i < ptr[k + 1]; i++)
      if (strong[i] && agg1[col[i]] && (best == 0 || val[i] > bv)) { best = agg1[col[i]]; bv = val[i]; }
    if (best) agg[k] = best;
  }
  for (k = 1; k <= nv; k++) {
    if (agg[k]) continue;
    na++;
    agg[k] = na;
    for (i = ptr[k]; i < ptr[k + 1]; i++)
      if (strong[i] && agg[col[i]] == 0) agg[col[i]] = na;
  }
  free(agg1);
  return na;
}

/* coarse_method 3 (no counterpart in the reference, whose aggregation is
 * scalar): smoothed aggregation over mesh nodes with the rigid-body modes as
 * near-nullspace (Vanek, Mandel & Brezina, Computing 56 (1996) 179-196).
 * Nodes in order of first appearance over the unknowns, a node's unknowns
 * ascending being its components; block strength ||A_IJ||_F > theta *
 * sqrt(||A_II||_F ||A_JJ||_F); three aggregation passes (whole free
 * neighbourhoods, then joining the strongest phase-1 neighbour aggregate,
 * then new aggregates of the rest); per aggregate the translations and
 * rotations about its centroid, orthonormalised by modified Gram-Schmidt
 * applied twice, columns below 1e-8 of their norm dropped; radius1 rounds
 * of aggregation, the later ones over the previous aggregates; P = P_tent -
 * omega D^-1 A P_tent, omega = 4 / (3 rho(D^-1 A)) with rho from 20 power
 * steps; R = P^T and AC = R A R^T.  Subdomains: the imported parts with the
 * overlap layers. */
static void run_setup_rbm(state *s, const int *part, int nparts) {
  ctl_t *c = &s->ctl;
  int n = s->n, nsd = g_geo_nsd, i, k, u;
  if (!part) orc_abort("coarse_method 3 needs an imported partition");
  if (nsd != 2 && nsd != 3) orc_abort("coarse_method 3 needs node coordinates (orc_set_geometry)");
  if (g_geo_n != n) orc_abort("coarse_method 3: geometry for %d unknowns, matrix has %d", g_geo_n, n);
  if (c->method == 2 || c->method == 3)
    orc_abort("method %d restricts a residual the one-process reference never sets (pcg.F90:146-149)", c->method);
  s->strong1 = (c->strong1 != 0.0) ? c->strong1 : 0.67;
  double theta = s->strong1;
  spm_arrange(&s->A, ARR_ROWS, 0, 0, 0, 0);
  const spm *A = &s->A;
  /* nodes by first appearance */
  int *nid = NEWI(g_geo_nnode), *node_of = NEWI(n), *comp = NEWI(n);
  int *node_glob = NEWI(n), *ncomp = NEWI(n), nn = 0;
  for (u = 1; u <= n; u++) {
    int g = g_geo_unode[u];
    if (g < 1 || g > g_geo_nnode) orc_abort("coarse_method 3: node %d of unknown %d out of range", g, u);
    if (nid[g] == 0) { nn++; nid[g] = nn; node_glob[nn] = g; ncomp[nn] = 0; }
    node_of[u] = nid[g];
    comp[u] = ncomp[nid[g]]++;
  }
  for (k = 1; k <= nn; k++)
    if (ncomp[k] != nsd) orc_abort("coarse_method 3 needs all %d freedoms of every node", nsd);
  /* unknowns per node, ascending */
  int *nu_ptr = NEWI(nn + 1), *nu = NEWI(n), *fillp = NEWI(nn + 1);
  for (u = 1; u <= n; u++) nu_ptr[node_of[u] + 1]++;
  nu_ptr[1] = 1;
  for (k = 1; k <= nn; k++) nu_ptr[k + 1] += nu_ptr[k];
  for (k = 1; k <= nn; k++) fillp[k] = nu_ptr[k];
  for (u = 1; u <= n; u++) nu[fillp[node_of[u]]++] = u;
  /* block norms, neighbours in first-touch order */
  long cap = (long)A->nnz + 1;
  int *bptr = NEWI(nn + 1), *bcol = NEWI(cap);
  double *bval = NEWD(cap);
  int *posn = NEWI(nn), nb = 0;
  for (k = 1; k <= nn; k++) posn[k] = 0;
  bptr[1] = 1;
  for (k = 1; k <= nn; k++) {
    int q0 = nb + 1, t;
    for (t = nu_ptr[k]; t < nu_ptr[k + 1]; t++) {
      int uu = nu[t], e;
      for (e = A->mbound[uu]; e <= A->mbound[uu + 1] - 1; e++) {
        int J = node_of[A->indj[e]];
        double a = A->val[e];
        if (posn[J] == 0) { nb++; posn[J] = nb; bcol[nb] = J; bval[nb] = a * a; }
        else bval[posn[J]] = bval[posn[J]] + a * a;
      }
    }
    for (t = q0; t <= nb; t++) posn[bcol[t]] = 0;
    bptr[k + 1] = nb + 1;
  }
  double *dn = NEWD(nn);
  for (i = 1; i <= nb; i++) bval[i] = sqrt(bval[i]);
  for (k = 1; k <= nn; k++)
    for (i = bptr[k]; i < bptr[k + 1]; i++)
      if (bcol[i] == k) dn[k] = bval[i];
  char *strong = NEWB(nb);
  for (k = 1; k <= nn; k++)
    for (i = bptr[k]; i < bptr[k + 1]; i++) {
      int J = bcol[i];
      strong[i] = (J != k && bval[i] > theta * sqrt(dn[k] * dn[J])) ? 1 : 0;
    }
  /* aggregation: round 1 over the nodes, then radius1 - 1 rounds over the
   * previous aggregates (edges: strong node pairs between them, weight the
   * sum of their block norms); 1-based aggregate per node */
  int *agg = NEWI(nn), na;
  na = three_phase(nn, bptr, bcol, bval, strong, agg);
  {
    int rounds = c->radius1 > 0 ? c->radius1 : 1, round;
    for (round = 2; round <= rounds && na > 1; round++) {
      int *mptr = NEWI(na + 1), *mem = NEWI(nn), *f3 = NEWI(na + 1);
      for (k = 1; k <= nn; k++) mptr[agg[k] + 1]++;
      mptr[1] = 1;
      for (i = 1; i <= na; i++) mptr[i + 1] += mptr[i];
      for (i = 1; i <= na; i++) f3[i] = mptr[i];
      for (k = 1; k <= nn; k++) mem[f3[agg[k]]++] = k;
      int *gptr = NEWI(na + 1), *gcol = NEWI(nb), *gpos = NEWI(na), ng = 0, aa;
      double *gval = NEWD(nb);
      gptr[1] = 1;
      for (aa = 1; aa <= na; aa++) {
        int q0 = ng + 1, t, q;
        for (t = mptr[aa]; t < mptr[aa + 1]; t++) {
          int I = mem[t];
          for (q = bptr[I]; q < bptr[I + 1]; q++) {
            int bb;
            if (!strong[q]) continue;
            bb = agg[bcol[q]];
            if (bb == aa) continue;
            if (gpos[bb] == 0) { ng++; gpos[bb] = ng; gcol[ng] = bb; gval[ng] = bval[q]; }
            else gval[gpos[bb]] = gval[gpos[bb]] + bval[q];
          }
        }
        for (t = q0; t <= ng; t++) gpos[gcol[t]] = 0;
        gptr[aa + 1] = ng + 1;
      }
      char *gstrong = NEWB(ng);
      for (i = 1; i <= ng; i++) gstrong[i] = 1;
      int *agg2 = NEWI(na);
      int na2 = three_phase(na, gptr, gcol, gval, gstrong, agg2);
      for (k = 1; k <= nn; k++) agg[k] = agg2[agg[k]];
      na = na2;
      free(mptr); free(mem); free(f3); free(gptr); free(gcol); free(gpos); free(gval); free(gstrong); free(agg2);
    }
  }
  /* nodes per aggregate, ascending */
  int *ag_ptr = NEWI(na + 1), *ag_nodes = NEWI(nn), *pos_in = NEWI(nn);
  for (k = 1; k <= nn; k++) ag_ptr[agg[k] + 1]++;
  ag_ptr[1] = 1;
  for (i = 1; i <= na; i++) ag_ptr[i + 1] += ag_ptr[i];
  {
    int *f2 = NEWI(na + 1);
    for (i = 1; i <= na; i++) f2[i] = ag_ptr[i];
    for (k = 1; k <= nn; k++) { pos_in[k] = f2[agg[k]] - ag_ptr[agg[k]]; ag_nodes[f2[agg[k]]++] = k; }
    free(f2);
  }
  /* rigid-body modes, orthonormalised */
  int nmodes = nsd == 3 ? 6 : 3;
  int *cfirst = NEWI(na + 1);
  double **Q = (double **)xcalloc((size_t)na + 1, sizeof(double *));
  cfirst[1] = 1;
  for (int a = 1; a <= na; a++) {
    int m = ag_ptr[a + 1] - ag_ptr[a], rows = m * nsd, t, d, col, kept = 0;
    double cen[3] = {0.0, 0.0, 0.0};
    for (d = 0; d < nsd; d++) {
      for (t = ag_ptr[a]; t < ag_ptr[a + 1]; t++) cen[d] = cen[d] + g_geo_xyz[(size_t)(node_glob[ag_nodes[t]] - 1) * nsd + d];
      cen[d] = cen[d] / (double)m;
    }
    double *B = (double *)xcalloc((size_t)rows * nmodes + 1, sizeof(double));
    for (t = 0; t < m; t++) {
      int g = node_glob[ag_nodes[ag_ptr[a] + t]] - 1;
      double x = g_geo_xyz[(size_t)g * nsd] - cen[0], y = g_geo_xyz[(size_t)g * nsd + 1] - cen[1];
      double z = nsd == 3 ? g_geo_xyz[(size_t)g * nsd + 2] - cen[2] : 0.0;
      for (d = 0; d < nsd; d++) B[(size_t)d * rows + t * nsd + d] = 1.0;
      if (nsd == 2) {
        B[(size_t)2 * rows + t * 2] = -y; B[(size_t)2 * rows + t * 2 + 1] = x;
      } else {
        B[(size_t)3 * rows + t * 3 + 1] = -z; B[(size_t)3 * rows + t * 3 + 2] = y;
        B[(size_t)4 * rows + t * 3] = z; B[(size_t)4 * rows + t * 3 + 2] = -x;
        B[(size_t)5 * rows + t * 3] = -y; B[(size_t)5 * rows + t * 3 + 1] = x;
      }
    }
    double *q = (double *)xcalloc((size_t)rows * nmodes + 1, sizeof(double));
    double *v = (double *)xcalloc((size_t)rows + 1, sizeof(double));
    for (col = 0; col < nmodes; col++) {
      int r, pass, p2;
      double n0 = 0.0, nv = 0.0;
      for (r = 0; r < rows; r++) v[r] = B[(size_t)col * rows + r];
      for (r = 0; r < rows; r++) n0 = n0 + v[r] * v[r];
      n0 = sqrt(n0);
      for (pass = 0; pass < 2; pass++)
        for (p2 = 0; p2 < kept; p2++) {
          const double *qp = q + (size_t)p2 * rows;
          double h = 0.0;
          for (r = 0; r < rows; r++) h = h + qp[r] * v[r];
          for (r = 0; r < rows; r++) v[r] = v[r] - h * qp[r];
        }
      for (r = 0; r < rows; r++) nv = nv + v[r] * v[r];
      nv = sqrt(nv);
      if (!(nv > 1e-8 * n0)) continue;
      for (r = 0; r < rows; r++) q[(size_t)kept * rows + r] = v[r] / nv;
      kept++;
    }
    free(B); free(v);
    Q[a] = q;
    cfirst[a + 1] = cfirst[a] + kept;
  }
  int nc = cfirst[na + 1] - 1;
  /* tentative prolongator, unknown after unknown (n x nc) */
  spm Pt = spm_new(n * nmodes, n, nc);
  int np = 0;
  for (u = 1; u <= n; u++) {
    int K = node_of[u], a = agg[K], rows = (ag_ptr[a + 1] - ag_ptr[a]) * nsd, col;
    int r = pos_in[K] * nsd + comp[u];
    for (col = cfirst[a]; col < cfirst[a + 1]; col++) {
      np++;
      Pt.indi[np] = u; Pt.indj[np] = col; Pt.val[np] = Q[a][(size_t)(col - cfirst[a]) * rows + r];
    }
  }
  Pt.nnz = np;
  /* omega from the power method on D^-1 A */
  double *dg = NEWD(n), *xv = NEWD(n), *yv = NEWD(n), rho = 0.0;
  for (u = 1; u <= n; u++)
    for (k = A->mbound[u]; k <= A->mbound[u + 1] - 1; k++)
      if (A->indj[k] == u) dg[u] = A->val[k];
  for (u = 1; u <= n; u++)
    if (!(dg[u] > 0.0)) orc_abort("coarse_method 3: non-positive diagonal at unknown %d", u);
  for (u = 1; u <= n; u++) xv[u] = 1.0 + (double)((u - 1) % 7) / 7.0;
  for (int it = 0; it < 20; it++) {
    double ny = 0.0, nx = 0.0;
    for (u = 1; u <= n; u++) {
      double sacc = 0.0;
      for (k = A->mbound[u]; k <= A->mbound[u + 1] - 1; k++) sacc = sacc + A->val[k] * xv[A->indj[k]];
      yv[u] = sacc / dg[u];
    }
    for (u = 1; u <= n; u++) { ny = ny + yv[u] * yv[u]; nx = nx + xv[u] * xv[u]; }
    ny = sqrt(ny);
    rho = ny / sqrt(nx);
    for (u = 1; u <= n; u++) xv[u] = yv[u] / ny;
  }
  double omega = 4.0 / (3.0 * rho);
  /* A P_tent (first-touch), then P = P_tent - omega D^-1 A P_tent as R = P^T */
  spm AA = spm_copy(A);
  spm AP = spm_AB(&AA, &Pt, 0, 0);
  spm_free(&AA);
  spm_arrange(&AP, ARR_ROWS, 0, 0, 0, 0);
  spm_arrange(&Pt, ARR_ROWS, 0, 0, 0, 0);
  spm R = spm_new(AP.nnz, nc, n);
  {
    double *ptv = NEWD(nc);
    int nr = 0;
    for (u = 1; u <= n; u++) {
      for (k = Pt.mbound[u]; k <= Pt.mbound[u + 1] - 1; k++) ptv[Pt.indj[k]] = Pt.val[k];
      double w = omega / dg[u];
      for (k = AP.mbound[u]; k <= AP.mbound[u + 1] - 1; k++) {
        int col = AP.indj[k];
        nr++;
        R.indi[nr] = col; R.indj[nr] = u; R.val[nr] = ptv[col] - w * AP.val[k];
      }
      for (k = Pt.mbound[u]; k <= Pt.mbound[u + 1] - 1; k++) ptv[Pt.indj[k]] = 0.0;
    }
    R.nnz = nr;
    free(ptv);
  }
  s->R = R;
  s->have_R = 1;
  s->AC = coarse_mtx_build(&s->A, &s->R, n, 0);
  /* aggregates per unknown for export */
  int *num = NEWI(n);
  for (u = 1; u <= n; u++) num[u] = agg[node_of[u]];
  form_aggr(&s->fine_inner, na, n, 0, 0, num);
  form_aggr(&s->fine_full, na, n, 0, 0, num);
  free(num);
  s->have_coarse = 0;
  /* subdomains: imported parts + overlap (Get_nodes, Add_layers) */
  s->ol = (c->overlap < 0) ? (c->smoothers > 0 ? c->smoothers : 0) : c->overlap;
  spm_arrange(&s->A, ARR_ROWS, 0, 0, 0, 0);
  int *nodes = NEWI(n);
  s->nsubd = nparts;
  s->sd_start = (int *)xcalloc((size_t)nparts + 2, sizeof(int));
  long scap = 16L * n + 16, fill = 0;
  s->sd_nodes = (int *)xcalloc((size_t)scap, sizeof(int));
  for (int ip = 1; ip <= nparts; ip++) {
    int nnodes = 0;
    for (i = 1; i <= n; i++) if (part[i - 1] == ip) nodes[++nnodes] = i;
    int nexp = add_layers(s->A.mbound, s->A.indj, nodes, nnodes, s->ol, n);
    if (fill + nexp > scap) {
      scap = 2 * (fill + nexp);
      s->sd_nodes = (int *)realloc(s->sd_nodes, sizeof(int) * (size_t)scap);
      if (!s->sd_nodes) orc_abort("out of memory");
    }
    s->sd_start[ip - 1] = (int)fill;
    memcpy(s->sd_nodes + fill, nodes + 1, sizeof(int) * (size_t)nexp);
    fill += nexp;
  }
  s->sd_start[nparts] = (int)fill;
  free(nodes);
  for (int a = 1; a <= na; a++) free(Q[a]);
  free(Q); free(cfirst); spm_free(&Pt); spm_free(&AP);
  free(dg); free(xv); free(yv); free(agg); free(ag_ptr); free(ag_nodes); free(pos_in);
  free(bptr); free(bcol); free(bval); free(posn); free(dn); free(strong);
  free(nu_ptr); free(nu); free(fillp); free(nid); free(node_of); free(comp); free(node_glob); free(ncomp);
}

static void run_setup(state *s, const int *part, int nparts) {
  ctl_t *c = &s->ctl;
  int n = s->n, i;
  if (c->executable == 1) {
    run_setup_geom(s, part, nparts);
    return;
  }
  if (c->coarse_method == 3) {
    run_setup_rbm(s, part, nparts);
    return;
  }
  /* Partitionings_aggr_InitFine (Partitioning_aggr.F90:33-117) */
  s->strong1 = (c->strong1 != 0.0) ? c->strong1 : 0.67;
  s->r1 = (c->radius1 > 0) ? c->radius1 : 2;
  s->min1 = (c->minasize1 > 0) ? c->minasize1 : (int)(0.5 * (double)((2 * s->r1 + 1) * (2 * s->r1 + 1)));
  s->max1 = (c->maxasize1 > 0) ? c->maxasize1 : (2 * s->r1 + 1) * (2 * s->r1 + 1);
  g_allmind = D_MAXINT;
  g_beta = 1.0e-5;
  spm_find_strong(&s->A, s->strong1);
  spm_aggregate(&s->A, &s->fine_inner, &s->fine_full, s->r1, s->min1, s->max1, s->strong1, 0);
  spm_unscale(&s->A);
  /* CoarsePreconditioner_smooth_Init (CoarsePreconditioner_smooth.F90:47-89) */
  if (c->coarse_method > 2) orc_abort("Wrong coarse method %d", c->coarse_method);
  if (c->smoothers > c->radius1) c->smoothers = c->radius1; /* CoarseMtx.F90:75-78 */
  s->R = int_rest_build(&s->A, &s->fine_inner, c->smoothers, c->omega);
  if (c->coarse_method == 2) { /* aggr.F90:158-160 */
    spm Rh = robust_restriction(&s->A, &s->R);
    spm_free(&s->R);
    s->R = Rh;
  }
  s->have_R = 1;
  s->AC = coarse_mtx_build(&s->A, &s->R, n, c->input_type != 1);
  /* Partitionings_aggr_InitCoarse (Partitioning_aggr.F90:120-193) */
  s->strong2 = (c->strong2 > 0) ? c->strong2 : s->strong1 / 2.0;
  spm_find_strong(&s->AC, s->strong2);
  if (c->radius2 > 0) s->r2 = c->radius2;
  else {
    int nn = (int)sqrt(1.0 * (double)s->A.nrows);
    s->r2 = (int)lround(3.0 * sqrt((double)nn) / (double)(2 * s->r1 + 1) - 1.0);
  }
  if (c->minasize2 > 0) s->min2 = c->minasize2;
  else if (c->radius2 > 0) s->min2 = 2 * c->radius2 + 1;
  else s->min2 = (int)(0.5 * (double)((2 * s->r2 + 1) * (2 * s->r2 + 1)));
  s->max2 = (c->maxasize2 > 0) ? c->maxasize2 : (2 * s->r2 + 1) * (2 * s->r2 + 1);
  spm_aggregate(&s->AC, &s->coarse_inner, &s->coarse_full, s->r2, s->min2, s->max2, s->strong2, 1);
  spm_unscale(&s->AC);
  s->have_coarse = 1;
  /* subdomains: coarse partitions (+ overlap), Preconditioner_base.F90:96-123 */
  s->ol = (c->overlap < 0) ? (c->smoothers > 0 ? c->smoothers : 0) : c->overlap;
  spm_arrange(&s->A, ARR_ROWS, 0, 0, 0, 0);
  int *nodes = NEWI(n);
  int np = part ? nparts : s->coarse_full.nagr;
  s->nsubd = np;
  s->sd_start = (int *)xcalloc((size_t)np + 2, sizeof(int));
  long cap = 16L * n + 16;
  s->sd_nodes = (int *)xcalloc((size_t)cap, sizeof(int));
  long fill = 0;
  int ip;
  for (ip = 1; ip <= np; ip++) {
    int nnodes = 0;
    if (part) { /* Get_nodes (Decomposition.f90:35-53) on an imported partition */
      for (i = 1; i <= n; i++) if (part[i - 1] == ip) nodes[++nnodes] = i;
    } else {
      nnodes = get_aggregate_nodes(ip, &s->coarse_full, &s->fine_full, n, nodes);
    }
    int nexp = add_layers(s->A.mbound, s->A.indj, nodes, nnodes, s->ol, n);
    if (fill + nexp > cap) {
      cap = 2 * (fill + nexp);
      s->sd_nodes = (int *)realloc(s->sd_nodes, sizeof(int) * (size_t)cap);
      if (!s->sd_nodes) orc_abort("out of memory");
    }
    s->sd_start[ip - 1] = (int)fill;
    memcpy(s->sd_nodes + fill, nodes + 1, sizeof(int) * (size_t)nexp);
    fill += nexp;
  }
  s->sd_start[np] = (int)fill;
  free(nodes);
}

/* y = A x with DOUG's row-arranged loop (SpMtx_op_Ax.f90:82-87) */
static void spmv_rows(const spm *A, const double *x, double *y) {
  int i, j;
  for (i = 1; i <= A->nrows; i++) {
    double s = 0.0;
    for (j = A->mbound[i]; j <= A->mbound[i + 1] - 1; j++) s = s + A->val[j] * x[A->indj[j]];
    y[i] = s;
  }
}

/* restriction / prolongation with R in its final (column-arranged or
 * unarranged) form, following SpMtx_Ax (SpMtx_op_Ax.f90:44-101). */
static void spmv_R(const spm *R, const double *x, double *y, int transp, int ny) {
  int i, j;
  for (i = 1; i <= ny; i++) y[i] = 0.0;
  int at = R->arrange;
  const int *indi = transp ? R->indj : R->indi;
  const int *indj = transp ? R->indi : R->indj;
  if (transp) at = (at == ARR_ROWS) ? ARR_COLS : (at == ARR_COLS ? ARR_ROWS : at);
  if (at == ARR_NO) {
    for (j = 1; j <= R->nnz; j++) y[indi[j]] = y[indi[j]] + R->val[j] * x[indj[j]];
  } else if (at == ARR_ROWS) {
    int nr = transp ? R->ncols : R->nrows;
    for (i = 1; i <= nr; i++)
      for (j = R->mbound[i]; j <= R->mbound[i + 1] - 1; j++) y[i] = y[i] + R->val[j] * x[indj[j]];
  } else {
    int nc = transp ? R->nrows : R->ncols;
    for (j = 1; j <= nc; j++)
      for (i = R->mbound[j]; i <= R->mbound[j + 1] - 1; i++) y[indi[i]] = y[indi[i]] + R->val[i] * x[j];
  }
}

static double dotp(const double *a, const double *b, int n) {
  double s = 0.0;
  int i;
  for (i = 1; i <= n; i++) s = s + a[i] * b[i];
  return s;
}

/* Host threads of the oracle's factorisations, subdomain solves and vector
 * loops (orc_set_threads).  Every parallel loop is over independent
 * subdomains, rows or entries, and the subdomain results are summed in
 * subdomain order afterwards, so the results do not depend on the count. */
static int g_threads = 1;

void orc_set_threads(int t) { g_threads = t > 0 ? t : 1; }

typedef struct {
  spchol **sd;     /* per subdomain (fine_method 1) */
  spchol *coarse;  /* levels > 1 */
  int nsd;
  long work;       /* doubles of work a subdomain solve needs */
} factors;

static void factors_free(factors *F) {
  if (F->sd) {
    int sd;
    for (sd = 0; sd < F->nsd; sd++) spchol_free(F->sd[sd]);
    free(F->sd);
  }
  spchol_free(F->coarse);
  memset(F, 0, sizeof *F);
}

/* Factorise_subdomains (subsolvers.F90:78-163): the principal submatrix
 * A(inds, inds) of every subdomain, and the coarse matrix, which the
 * reference factorises lazily on the first coarse solve (pcg.F90:166-178).
 * Task 0 is the coarse matrix, tasks 1..nsd the subdomains. */
static void factor_all(state *s, factors *F) {
  ctl_t *c = &s->ctl;
  int n = s->n;
  const spm *ACp = s->have_sub ? &s->ACs : &s->AC;
  F->nsd = c->fine_method == 1 ? s->nsubd : 0;
  F->sd = (spchol **)xcalloc((size_t)F->nsd + 1, sizeof(spchol *));
  int have_coarse = c->levels > 1;
  int ntask = F->nsd + 1, failed = 0, t;
  char msg[256];
  msg[0] = 0;
#pragma omp parallel num_threads(g_threads) if (g_threads > 1)
  {
    int *floc = (int *)calloc((size_t)n + 2, sizeof(int));
    if (!floc) {
#pragma omp atomic write
      failed = 1;
    }
#pragma omp for schedule(dynamic, 1)
    for (t = 0; t < ntask; t++) {
      char err[256];
      err[0] = 0;
      if (!floc || failed) continue;
      if (t == 0) {
        if (!have_coarse) continue;
        long nz = ACp->nnz, k;
        int *ci = (int *)malloc(sizeof(int) * ((size_t)nz + 1));
        int *cj = (int *)malloc(sizeof(int) * ((size_t)nz + 1));
        spchol *f = NULL;
        if (ci && cj) {
          for (k = 0; k < nz; k++) { ci[k] = ACp->indi[k + 1] - 1; cj[k] = ACp->indj[k + 1] - 1; }
          f = spchol_factor(ACp->nrows, nz, ci, cj, ACp->val + 1, err, sizeof err);
        } else {
          snprintf(err, sizeof err, "out of memory");
        }
        free(ci); free(cj);
        if (!f) {
#pragma omp critical(orc_fail)
          { failed = 1; snprintf(msg, sizeof msg, "coarse factorisation: %s", err); }
        }
        F->coarse = f;
        continue;
      }
      int sd = t - 1;
      int b0 = s->sd_start[sd], m = s->sd_start[sd + 1] - b0, k;
      const int *nodes = s->sd_nodes + b0;
      long cnt = 0, q;
      for (k = 0; k < m; k++) floc[nodes[k]] = k + 1;
      for (k = 0; k < m; k++) {
        int i = nodes[k];
        for (q = s->A.mbound[i]; q <= s->A.mbound[i + 1] - 1; q++)
          if (floc[s->A.indj[q]] > 0) cnt++;
      }
      int *si = (int *)malloc(sizeof(int) * ((size_t)cnt + 1));
      int *sj = (int *)malloc(sizeof(int) * ((size_t)cnt + 1));
      double *sv = (double *)malloc(sizeof(double) * ((size_t)cnt + 1));
      spchol *f = NULL;
      if (si && sj && sv) {
        cnt = 0;
        for (k = 0; k < m; k++) {
          int i = nodes[k];
          for (q = s->A.mbound[i]; q <= s->A.mbound[i + 1] - 1; q++) {
            int l = floc[s->A.indj[q]];
            if (l > 0) { si[cnt] = k; sj[cnt] = l - 1; sv[cnt] = s->A.val[q]; cnt++; }
          }
        }
        f = spchol_factor(m, cnt, si, sj, sv, err, sizeof err);
      } else {
        snprintf(err, sizeof err, "out of memory");
      }
      free(si); free(sj); free(sv);
      for (k = 0; k < m; k++) floc[nodes[k]] = 0;
      if (!f) {
#pragma omp critical(orc_fail)
        { failed = 1; snprintf(msg, sizeof msg, "subdomain %d: %s", sd + 1, err); }
      }
      F->sd[sd] = f;
    }
    free(floc);
  }
  if (failed) {
    factors_free(F);
    orc_abort("%s", msg[0] ? msg : "out of memory");
  }
  F->work = 1;
  for (t = 0; t < F->nsd; t++) {
    long w = spchol_work_size(F->sd[t]);
    if (w > F->work) F->work = w;
  }
}

/* y = A x over row blocks (the same per-row sums as spmv_rows) */
static void spmv_rows_par(const spm *A, const double *x, double *y) {
  int i;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1) schedule(static)
  for (i = 1; i <= A->nrows; i++) {
    double s = 0.0;
    int j;
    for (j = A->mbound[i]; j <= A->mbound[i + 1] - 1; j++) s = s + A->val[j] * x[A->indj[j]];
    y[i] = s;
  }
}

/* pcg_weigs (pcg.F90:289-462) with preconditioner (pcg.F90:216-270). */
static void run_pcg(state *s, orc_result *res) {
  ctl_t *c = &s->ctl;
  int n = s->n, i, sd;
  int levels = c->levels;
  int method = c->method;
  if (c->fine_method != 1 && c->fine_method != 0 && c->fine_method != 2)
    orc_abort("Wrong fine method %d", c->fine_method); /* aggr.F90:216-226 */
  if (method == 2 || method == 3)
    orc_abort("method %d restricts a residual the one-process reference never sets (pcg.F90:146-149)", method);
  int sgs_iters = c->num_iters <= 0 ? 3 : c->num_iters; /* aggr.F90:221 */
  unsigned char *sgs_in = (unsigned char *)xcalloc((size_t)n + 1, 1);
  double *sgs_diag = NEWD(n), *sgs_x = NEWD(n);
  double t0 = now_s();
  factors F;
  memset(&F, 0, sizeof F);
  factor_all(s, &F);
  const spm *ACp = s->have_sub ? &s->ACs : &s->AC, *Rp = s->have_sub ? &s->Rs : &s->R;
  int nc = ACp->nrows;
  double t1 = now_s();
  res->t_factor = t1 - t0;

  int nthr = g_threads > 1 ? g_threads : 1;
  double *x = NEWD(n), *r = NEWD(n), *p = NEWD(n), *q = NEWD(n), *z = NEWD(n);
  long sdtot = s->sd_start[s->nsubd];
  double *subsol = NEWD(sdtot);
  double *works = (double *)xcalloc((size_t)F.work * nthr + 1, sizeof(double));
  double *crhs = NEWD(nc), *csol = NEWD(nc), *tmpsol = NEWD(n);
  double *cw = levels > 1 ? NEWD(spchol_work_size(F.coarse)) : NEWD(1);
  double tol = c->solve_tolerance;
  int maxit = c->solve_maxiters;
  if (maxit == -1) maxit = 100000;
  double *alpha = NEWD(maxit + 1), *beta = NEWD(maxit + 1);
  res->res_hist = (double *)xcalloc((size_t)maxit + 1, sizeof(double));
  spmv_rows_par(&s->A, x, r);
  for (i = 1; i <= n; i++) r[i] = s->rhs[i - 1] - r[i];
  double init_norm = dotp(r, r, n);
  if (init_norm == 0.0) init_norm = 1.0;
  res->init_norm = sqrt(init_norm);
  int it = 0;
  double ratio_norm = 1.0, rho_prev = 0.0;
  while (ratio_norm > tol * tol && it < maxit) {
    it++;
    /* preconditioner */
    if (method == 0) {
      for (i = 1; i <= n; i++) z[i] = r[i];
    } else {
      for (i = 1; i <= n; i++) z[i] = 0.0;
      if (c->fine_method == 0) { /* FinePreconditioner_Apply, type NONE (Preconditioner.F90:38-39) */
        for (i = 1; i <= n; i++) z[i] = r[i];
      } else if (c->fine_method == 2) {
        /* FinePreconditioner_sgs_Apply (FinePreconditioner_sgs.F90:69-86): per
         * subdomain, SymGaussSeidel (stationary.F90:33-88) on the entries of A
         * with row and column in the subdomain, rows in global order, x0 = 0;
         * the subdomain results are added in subdomain order */
        for (sd = 0; sd < s->nsubd; sd++) {
          int b0 = s->sd_start[sd], m = s->sd_start[sd + 1] - b0, k, it2, jj;
          for (k = 0; k < m; k++) sgs_in[s->sd_nodes[b0 + k]] = 1;
          for (i = 1; i <= n; i++) { sgs_diag[i] = 0.0; sgs_x[i] = 0.0; }
          for (i = 1; i <= n; i++)
            if (sgs_in[i])
              for (jj = s->A.mbound[i]; jj <= s->A.mbound[i + 1] - 1; jj++)
                if (s->A.indj[jj] == i) sgs_diag[i] = s->A.val[jj];
          for (it2 = 1; it2 <= sgs_iters; it2++) {
            int dir;
            for (dir = 0; dir < 2; dir++) {
              int i0 = dir == 0 ? 1 : n, i1 = dir == 0 ? n + 1 : 0, di = dir == 0 ? 1 : -1;
              for (i = i0; i != i1; i += di) {
                if (sgs_diag[i] == 0) continue;
                sgs_x[i] = r[i];
                for (jj = s->A.mbound[i]; jj <= s->A.mbound[i + 1] - 1; jj++) {
                  int j = s->A.indj[jj];
                  if (!sgs_in[j] || j == i) continue;
                  sgs_x[i] = sgs_x[i] - s->A.val[jj] * sgs_x[j];
                }
                sgs_x[i] = sgs_x[i] / sgs_diag[i];
              }
            }
          }
          for (k = 0; k < m; k++) z[s->sd_nodes[b0 + k]] = z[s->sd_nodes[b0 + k]] + sgs_x[s->sd_nodes[b0 + k]];
          for (k = 0; k < m; k++) sgs_in[s->sd_nodes[b0 + k]] = 0;
        }
      }
      /* Solve_subdomains (subsolvers.F90:54-76) beside prec2Level's coarse
       * solve (pcg.F90:144-209): task 0 restricts, solves the coarse system
       * and prolongs; task sd+1 solves subdomain sd into its own slice */
      int nsolve = c->fine_method == 1 ? s->nsubd : 0, t;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1) schedule(dynamic, 1)
      for (t = 0; t < nsolve + 1; t++) {
        if (t == 0) {
          if (levels > 1) {
            spmv_R(Rp, r, crhs, 0, nc);
            spchol_solve(F.coarse, crhs + 1, csol + 1, cw);
            spmv_R(Rp, csol, tmpsol, 1, n);
          }
          continue;
        }
        int sdi = t - 1, b0 = s->sd_start[sdi], m = s->sd_start[sdi + 1] - b0, k;
#ifdef _OPENMP
        double *w = works + (size_t)F.work * (size_t)omp_get_thread_num();
#else
        double *w = works;
#endif
        double *v = subsol + 1 + b0;
        for (k = 0; k < m; k++) v[k] = r[s->sd_nodes[b0 + k]];
        spchol_solve(F.sd[sdi], v, v, w);
      }
      for (sd = 0; sd < nsolve; sd++) {
        int b0 = s->sd_start[sd], m = s->sd_start[sd + 1] - b0, k;
        const double *v = subsol + 1 + b0;
        for (k = 0; k < m; k++) z[s->sd_nodes[b0 + k]] = z[s->sd_nodes[b0 + k]] + v[k];
      }
      if (levels > 1 && (method == 1 || method == 5)) /* pcg.F90:191-193, 205-208 */
        for (i = 1; i <= n; i++) z[i] = z[i] + tmpsol[i];
    }
    double rho_curr = dotp(r, z, n);
    if (it == 1) {
      for (i = 1; i <= n; i++) p[i] = z[i];
    } else {
      double bt = rho_curr / rho_prev;
      beta[it] = bt;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1) schedule(static)
      for (i = 1; i <= n; i++) p[i] = z[i] + bt * p[i];
    }
    spmv_rows_par(&s->A, p, q);
    double al = rho_curr / dotp(p, q, n);
    alpha[it] = al;
#pragma omp parallel for num_threads(g_threads) if (g_threads > 1) schedule(static)
    for (i = 1; i <= n; i++) {
      x[i] = x[i] + al * p[i];
      r[i] = r[i] - al * q[i];
    }
    rho_prev = rho_curr;
    double res_norm = dotp(r, r, n);
    ratio_norm = res_norm / init_norm;
    res->res_hist[it - 1] = sqrt(res_norm);
  }
  res->t_solve = now_s() - t1;
  res->iterations = it;
  res->cond_num = calc_cond(it, alpha, beta);
  res->x = (double *)xcalloc((size_t)n, sizeof(double));
  memcpy(res->x, x + 1, sizeof(double) * (size_t)n);
  factors_free(&F);
  free(x); free(r); free(p); free(q); free(z); free(subsol); free(works);
  free(crhs); free(csol); free(cw); free(tmpsol); free(alpha); free(beta);
  free(sgs_in); free(sgs_diag); free(sgs_x);
}

static int *dup0(const int *a1, int n) { /* 1-based -> 0-based copy */
  int *o = (int *)xcalloc((size_t)n + 1, sizeof(int));
  if (n > 0) memcpy(o, a1 + 1, sizeof(int) * (size_t)n);
  return o;
}
static double *dupd0(const double *a1, int n) {
  double *o = (double *)xcalloc((size_t)n + 1, sizeof(double));
  if (n > 0) memcpy(o, a1 + 1, sizeof(double) * (size_t)n);
  return o;
}

static void export_setup(const state *s, orc_result *r) {
  r->n = s->n;
  r->nagr_fine = s->fine_inner.nagr;
  r->aggr_fine = dup0(s->fine_inner.num, s->n);
  r->nagr_fine_full = s->fine_full.nagr;
  r->aggr_fine_full = dup0(s->fine_full.num, s->n);
  if (s->have_coarse) {
    r->nagr_coarse = s->coarse_inner.nagr;
    r->aggr_coarse = dup0(s->coarse_inner.num, s->coarse_inner.n);
    r->nagr_coarse_full = s->coarse_full.nagr;
    r->aggr_coarse_full = dup0(s->coarse_full.num, s->coarse_full.n);
  }
  r->nsubd = s->nsubd;
  r->subd_starts = (int *)xcalloc((size_t)s->nsubd + 1, sizeof(int));
  memcpy(r->subd_starts, s->sd_start, sizeof(int) * (size_t)(s->nsubd + 1));
  int tot = s->sd_start[s->nsubd];
  r->subd_nodes = (int *)xcalloc((size_t)tot + 1, sizeof(int));
  memcpy(r->subd_nodes, s->sd_nodes, sizeof(int) * (size_t)tot);
  r->R_nrows = s->R.nrows; r->R_ncols = s->R.ncols; r->R_nnz = s->R.nnz;
  r->R_i = dup0(s->R.indi, s->R.nnz); r->R_j = dup0(s->R.indj, s->R.nnz);
  r->R_v = dupd0(s->R.val, s->R.nnz);
  r->AC_n = s->AC.nrows; r->AC_nnz = s->AC.nnz;
  r->AC_i = dup0(s->AC.indi, s->AC.nnz); r->AC_j = dup0(s->AC.indj, s->AC.nnz);
  r->AC_v = dupd0(s->AC.val, s->AC.nnz);
  r->overlap = s->ol; r->smoothers = s->ctl.smoothers; r->levels = s->ctl.levels;
  r->method = s->ctl.method;
  r->strong1 = s->strong1; r->strong2 = s->strong2;
  r->radius1 = s->r1; r->radius2 = s->r2;
  r->minasize1 = s->min1; r->maxasize1 = s->max1;
  r->minasize2 = s->min2; r->maxasize2 = s->max2;
  r->tol = s->ctl.solve_tolerance; r->maxit = s->ctl.solve_maxiters;
  if (s->cxyz) {
    r->cnsd = s->cnsd;
    r->cxyz = (double *)xcalloc((size_t)s->cnsd * s->AC.nrows + 1, sizeof(double));
    memcpy(r->cxyz, s->cxyz, sizeof(double) * (size_t)s->cnsd * s->AC.nrows);
  }
}

static void load_coo(state *s, int n, int nnz, const int *ii, const int *jj,
                     const double *vv) {
  /* ReadInSparseAssembled (SpMtx_class.F90:410-453) after the file read */
  if (n > nnz) { int t = n; n = nnz; nnz = t; }
  s->n = n;
  s->A = spm_new(nnz, n, n);
  int k, shift = (nnz > 0 && ii[0] == 0) ? 1 : 0;
  for (k = 0; k < nnz; k++) {
    s->A.indi[k + 1] = ii[k] + shift;
    s->A.indj[k + 1] = jj[k] + shift;
    s->A.val[k + 1] = vv[k];
    if (s->A.indi[k + 1] < 1 || s->A.indi[k + 1] > n || s->A.indj[k + 1] < 1 ||
        s->A.indj[k + 1] > n)
      orc_abort("matrix index out of range at entry %d", k + 1);
  }
  s->A.symmstruct = s->ctl.symmstruct;
  s->A.symmnumeric = s->A.symmstruct ? s->ctl.symmnumeric : 0;
  s->A.scaling = SCALE_NO;
}

static int run_common(int n, int nnz, const int *ii, const int *jj, const double *vv,
                      const double *rhs, const char *ctl_text, const int *part,
                      int nparts, int do_solve, const geom_mesh *G, orc_result **out) {
  orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
  state *s = (state *)calloc(1, sizeof(state));
  *out = r;
  s->geom = G;
  if (setjmp(g_jmp)) {
    r->status = -1;
    snprintf(r->errmsg, sizeof r->errmsg, "%s", g_err);
    state_free(s); free(s);
    return -1;
  }
  ctl_defaults(&s->ctl);
  ctl_parse_text(&s->ctl, ctl_text ? ctl_text : "");
  ctl_finish(&s->ctl);
  load_coo(s, n, nnz, ii, jj, vv);
  s->rhs = (double *)xcalloc((size_t)s->n + 1, sizeof(double));
  int i;
  for (i = 0; i < s->n; i++) s->rhs[i] = rhs ? rhs[i] : 1.0;
  double t0 = now_s();
  run_setup(s, part, nparts);
  r->t_setup = now_s() - t0;
  export_setup(s, r);
  r->b = (double *)xcalloc((size_t)s->n + 1, sizeof(double));
  memcpy(r->b, s->rhs, sizeof(double) * (size_t)s->n);
  if (do_solve) run_pcg(s, r);
  state_free(s); free(s);
  return 0;
}

int orc_run_coo(int n, int nnz, const int *ii, const int *jj, const double *vv,
                const double *rhs, const char *ctl_text, const int *part,
                int nparts, orc_result **out) {
  return run_common(n, nnz, ii, jj, vv, rhs, ctl_text, part, nparts, 1, NULL, out);
}

int orc_setup_coo(int n, int nnz, const int *ii, const int *jj, const double *vv,
                  const char *ctl_text, const int *part, int nparts,
                  orc_result **out) {
  return run_common(n, nnz, ii, jj, vv, NULL, ctl_text, part, nparts, 0, NULL, out);
}

/* A setup kept for repeated factorisations + solves (the benchmark's CPU
 * timing: the setup once, then per step what the GPU step does). */
struct orc_session {
  state s;
};

int orc_session_new(int n, int nnz, const int *ii, const int *jj, const double *vv,
                    const char *ctl_text, const int *part, int nparts, orc_session **sess,
                    orc_result **out) {
  orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
  orc_session *S = (orc_session *)calloc(1, sizeof(orc_session));
  *out = r;
  *sess = NULL;
  state *s = &S->s;
  if (setjmp(g_jmp)) {
    r->status = -1;
    snprintf(r->errmsg, sizeof r->errmsg, "%s", g_err);
    state_free(s); free(S);
    return -1;
  }
  ctl_defaults(&s->ctl);
  ctl_parse_text(&s->ctl, ctl_text ? ctl_text : "");
  ctl_finish(&s->ctl);
  load_coo(s, n, nnz, ii, jj, vv);
  s->rhs = (double *)xcalloc((size_t)s->n + 1, sizeof(double));
  double t0 = now_s();
  run_setup(s, part, nparts);
  r->t_setup = now_s() - t0;
  export_setup(s, r);
  *sess = S;
  return 0;
}

int orc_session_solve(orc_session *S, const double *rhs, orc_result **out) {
  orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
  *out = r;
  state *s = &S->s;
  if (setjmp(g_jmp)) {
    r->status = -1;
    snprintf(r->errmsg, sizeof r->errmsg, "%s", g_err);
    return -1;
  }
  int i;
  for (i = 0; i < s->n; i++) s->rhs[i] = rhs ? rhs[i] : 1.0;
  r->n = s->n;
  r->b = (double *)xcalloc((size_t)s->n + 1, sizeof(double));
  memcpy(r->b, s->rhs, sizeof(double) * (size_t)s->n);
  run_pcg(s, r);
  return 0;
}

void orc_session_free(orc_session *S) {
  if (!S) return;
  state_free(&S->s);
  free(S);
}

void orc_free(orc_result *r) {
  if (!r) return;
  free(r->x); free(r->b); free(r->res_hist); free(r->aggr_fine);
  free(r->aggr_fine_full); free(r->aggr_coarse); free(r->aggr_coarse_full);
  free(r->subd_starts); free(r->subd_nodes); free(r->R_i); free(r->R_j);
  free(r->R_v); free(r->AC_i); free(r->AC_j); free(r->AC_v); free(r->cxyz);
  free(r);
}

/* ------------------------------------------------------------------ */
/* file formats (SpMtx_class.F90:410-617, Vect.F90:840-947,             */
/* DOUG_utils.F90:1598-1700)                                            */
/* ------------------------------------------------------------------ */
static unsigned char *slurp(const char *path, long *len) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  long L = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char *buf = (unsigned char *)malloc((size_t)L + 1);
  if (!buf) { fclose(f); return NULL; }
  if (L > 0 && fread(buf, 1, (size_t)L, f) != (size_t)L) { fclose(f); free(buf); return NULL; }
  buf[L] = 0;
  fclose(f);
  *len = L;
  return buf;
}

static uint32_t be32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static double bed(const unsigned char *p) {
  uint64_t u = ((uint64_t)be32(p) << 32) | be32(p + 4);
  double d;
  memcpy(&d, &u, 8);
  return d;
}
static uint32_t le32(const unsigned char *p) {
  return ((uint32_t)p[3] << 24) | ((uint32_t)p[2] << 16) | ((uint32_t)p[1] << 8) | p[0];
}
static double led(const unsigned char *p) {
  uint64_t u = ((uint64_t)le32(p + 4) << 32) | le32(p);
  double d;
  memcpy(&d, &u, 8);
  return d;
}

/* Fortran unformatted sequential record (4-byte little-endian markers,
 * gfortran sub-records for lengths beyond 2^31-1). */
static const unsigned char *fort_record(const unsigned char *buf, long len, long *pos,
                                        long *rlen, unsigned char **owned) {
  *owned = NULL;
  if (*pos + 4 > len) return NULL;
  int32_t m = (int32_t)le32(buf + *pos);
  if (m >= 0) {
    if (*pos + 8 + m > len) return NULL;
    const unsigned char *d = buf + *pos + 4;
    *rlen = m;
    *pos += 8 + m;
    return d;
  }
  /* sub-records: concatenate */
  long total = 0, p = *pos;
  unsigned char *acc = NULL;
  for (;;) {
    if (p + 4 > len) { free(acc); return NULL; }
    int32_t mm = (int32_t)le32(buf + p);
    long l = mm < 0 ? -(long)mm : mm;
    if (p + 8 + l > len) { free(acc); return NULL; }
    acc = (unsigned char *)realloc(acc, (size_t)(total + l + 1));
    memcpy(acc + total, buf + p + 4, (size_t)l);
    total += l;
    p += 8 + l;
    if (mm >= 0 && p != *pos + 8 + l) break;
    if (mm > 0) break;
    if (mm < 0 && total == l && p - 8 - l == *pos) continue;
    if (mm < 0) continue;
    break;
  }
  *pos = p;
  *rlen = total;
  *owned = acc;
  return acc;
}

int orc_read_assembled(const char *path, int format, int *n, int *nnz, int **ii,
                       int **jj, double **vv) {
  long len = 0;
  unsigned char *buf = slurp(path, &len);
  if (!buf) return -1;
  int N = 0, NNZ = 0, k;
  if (format == 0) {
    char *p = (char *)buf, *e;
    long a = strtol(p, &e, 10); if (e == p) { free(buf); return -2; } p = e;
    long b = strtol(p, &e, 10); if (e == p) { free(buf); return -2; } p = e;
    N = (int)a; NNZ = (int)b;
    int cnt = N > NNZ ? N : NNZ;
    *ii = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *jj = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *vv = (double *)malloc(sizeof(double) * (size_t)(cnt + 1));
    for (k = 0; k < cnt; k++) {
      while (*p == ',' || isspace((unsigned char)*p)) p++;
      long i1 = strtol(p, &e, 10); if (e == p) { free(buf); return -3; } p = e;
      while (*p == ',' || isspace((unsigned char)*p)) p++;
      long j1 = strtol(p, &e, 10); if (e == p) { free(buf); return -3; } p = e;
      while (*p == ',' || isspace((unsigned char)*p)) p++;
      for (char *q = p; *q && !isspace((unsigned char)*q); q++) if (*q == 'd' || *q == 'D') *q = 'e';
      double v = strtod(p, &e); if (e == p) { free(buf); return -3; } p = e;
      (*ii)[k] = (int)i1; (*jj)[k] = (int)j1; (*vv)[k] = v;
    }
  } else if (format == 1) {
    long pos = 0, rl;
    unsigned char *own;
    const unsigned char *d = fort_record(buf, len, &pos, &rl, &own);
    if (!d || rl < 8) { free(buf); return -2; }
    N = (int)le32(d); NNZ = (int)le32(d + 4);
    free(own);
    int cnt = N > NNZ ? N : NNZ;
    d = fort_record(buf, len, &pos, &rl, &own);
    if (!d || rl < 16L * cnt) { free(buf); return -3; }
    *ii = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *jj = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *vv = (double *)malloc(sizeof(double) * (size_t)(cnt + 1));
    for (k = 0; k < cnt; k++) {
      (*ii)[k] = (int)le32(d + 16L * k);
      (*jj)[k] = (int)le32(d + 16L * k + 4);
      (*vv)[k] = led(d + 16L * k + 8);
    }
    free(own);
  } else if (format == 2) {
    if (len < 8) { free(buf); return -2; }
    N = (int)be32(buf); NNZ = (int)be32(buf + 4);
    int cnt = N > NNZ ? N : NNZ;
    if (len < 8 + 16L * cnt) { free(buf); return -3; }
    *ii = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *jj = (int *)malloc(sizeof(int) * (size_t)(cnt + 1));
    *vv = (double *)malloc(sizeof(double) * (size_t)(cnt + 1));
    for (k = 0; k < cnt; k++) {
      (*ii)[k] = (int)be32(buf + 8 + 16L * k);
      (*jj)[k] = (int)be32(buf + 8 + 16L * k + 4);
      (*vv)[k] = bed(buf + 8 + 16L * k + 8);
    }
  } else {
    free(buf);
    return -4;
  }
  free(buf);
  *n = N;
  *nnz = NNZ;
  return 0;
}

int orc_read_vector(const char *path, int format, int n, double *x) {
  long len = 0;
  unsigned char *buf = slurp(path, &len);
  if (!buf) return -1;
  int k;
  if (format == 0) { /* '(i9)' count then '(e23.16)' per line */
    char *p = (char *)buf, *e;
    long m = strtol(p, &e, 10);
    if (e == p || m != n) { free(buf); return -2; }
    p = e;
    for (k = 0; k < n; k++) {
      while (isspace((unsigned char)*p)) p++;
      for (char *q = p; *q && !isspace((unsigned char)*q); q++) if (*q == 'd' || *q == 'D') *q = 'e';
      x[k] = strtod(p, &e);
      if (e == p) { free(buf); return -3; }
      p = e;
    }
  } else if (format == 1) {
    long pos = 0, rl;
    unsigned char *own;
    const unsigned char *d = fort_record(buf, len, &pos, &rl, &own);
    if (!d || rl < 8L * n) { free(buf); return -3; }
    for (k = 0; k < n; k++) x[k] = led(d + 8L * k);
    free(own);
  } else if (format == 2) {
    if (len < 4 || (int)be32(buf) != n || len < 4 + 8L * n) { free(buf); return -2; }
    for (k = 0; k < n; k++) x[k] = bed(buf + 4 + 8L * k);
  } else {
    free(buf);
    return -4;
  }
  free(buf);
  return 0;
}

int orc_write_solution(const char *path, int format, int n, const double *x) {
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  int k;
  if (format == 0) {
    fprintf(f, "%6d\n", n);
    for (k = 0; k < n; k++) fprintf(f, "%21.14E\n", x[k]);
  } else if (format == 1) {
    uint32_t m = (uint32_t)(8 * n);
    fwrite(&m, 4, 1, f);
    for (k = 0; k < n; k++) fwrite(&x[k], 8, 1, f);
    fwrite(&m, 4, 1, f);
  } else if (format == 2) {
    unsigned char b[8];
    uint32_t m = (uint32_t)n;
    b[0] = (unsigned char)(m >> 24); b[1] = (unsigned char)(m >> 16);
    b[2] = (unsigned char)(m >> 8); b[3] = (unsigned char)m;
    fwrite(b, 1, 4, f);
    for (k = 0; k < n; k++) {
      uint64_t u;
      memcpy(&u, &x[k], 8);
      int q;
      for (q = 0; q < 8; q++) b[q] = (unsigned char)(u >> (56 - 8 * q));
      fwrite(b, 1, 8, f);
    }
  } else {
    fclose(f);
    return -4;
  }
  fclose(f);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Elemental input, one process.  Restates Mesh_initFromFile and
 * Mesh_readFileFreelists (src/datatypes/Mesh.F90:293-460), the element loop of
 * ElemMtxs_readAndDistribute (src/datatypes/ElemMtxs/ElemMtxs_distribute.F90:548-575),
 * the one-partition local numbering of Mesh_MapsAndNghbrs (Mesh.F90:1131-1193)
 * and ElemMtxsAssembleContext_addChunk / _extractSpMtx / _extractVect
 * (src/datatypes/ElemMtxs/ElemMtxs_assemble.F90:158-289), with the sorted
 * per-row index map of src/datatypes/IdxMap.f90:108-182. */
typedef struct { int size, cap; int *key, *val; } idxmap_t;

static int idxmap_pos(const idxmap_t *m, int k) { /* first position with key >= k */
  int lo = 0, hi = m->size;
  while (lo < hi) { int mid = (lo + hi) / 2; if (m->key[mid] < k) lo = mid + 1; else hi = mid; }
  return lo;
}
static int idxmap_lookup(const idxmap_t *m, int k) {
  int p = idxmap_pos(m, k);
  return (p < m->size && m->key[p] == k) ? m->val[p] : -1;
}
static void idxmap_insert(idxmap_t *m, int k, int x) {
  int p = idxmap_pos(m, k);
  if (p < m->size && m->key[p] == k) return;
  if (m->size + 1 > m->cap) {
    m->cap = m->size * 4 / 3 + 4;
    m->key = (int *)realloc(m->key, sizeof(int) * (size_t)m->cap);
    m->val = (int *)realloc(m->val, sizeof(int) * (size_t)m->cap);
  }
  memmove(m->key + p + 1, m->key + p, sizeof(int) * (size_t)(m->size - p));
  memmove(m->val + p + 1, m->val + p, sizeof(int) * (size_t)(m->size - p));
  m->key[p] = k;
  m->val[p] = x;
  m->size++;
}

/* out: n local freedoms, 1-based COO (indi = column freedom, indj = row,
 * the reference's flip), rhs.  Returns 0 or a negative error code. */
int orc_read_elemental(const char *info, const char *freel, const char *elemmat, int nblocks,
                       int *n_out, int *nnz_out, int **ii_out, int **jj_out, double **vv_out,
                       double **rhs_out) {
  long len, pos, rl;
  unsigned char *own;
  const unsigned char *r;
  unsigned char *buf = slurp(info, &len);
  if (!buf) return -1;
  pos = 0;
  r = fort_record(buf, len, &pos, &rl, &own);
  if (!r || rl < 20) { free(buf); free(own); return -2; }
  int nell = (int32_t)le32(r), ngf = (int32_t)le32(r + 4), mfrelt = (int32_t)le32(r + 12);
  free(own); free(buf);
  if (nell <= 0 || ngf <= 0 || mfrelt <= 0) return -2;
  /* freedom lists: record = nfrelt, mhead(1:nfrelt) */
  int *nfrelt = (int *)calloc((size_t)nell, sizeof(int));
  int *mhead = (int *)calloc((size_t)nell * (size_t)mfrelt, sizeof(int)); /* mhead(i,e) = [e*mfrelt+i-1] */
  buf = slurp(freel, &len);
  if (!buf) { free(nfrelt); free(mhead); return -3; }
  pos = 0;
  for (int e = 0; e < nell; e++) {
    r = fort_record(buf, len, &pos, &rl, &own);
    if (!r || rl < 4) { free(own); free(buf); free(nfrelt); free(mhead); return -3; }
    int nf = (int32_t)le32(r);
    if (nf < 0 || nf > mfrelt || rl < 4 + 4L * nf) { free(own); free(buf); free(nfrelt); free(mhead); return -3; }
    nfrelt[e] = nf;
    for (int i = 0; i < nf; i++) mhead[(size_t)e * mfrelt + i] = (int32_t)le32(r + 4 + 4 * i);
    free(own);
  }
  free(buf);
  if (nblocks > 1) { /* Mesh.F90:313-319: ngf = maxval(mhead) */
    int mx = 0;
    for (int e = 0; e < nell; e++)
      for (int i = 0; i < nfrelt[e]; i++) if (mhead[(size_t)e * mfrelt + i] > mx) mx = mhead[(size_t)e * mfrelt + i];
    ngf = mx;
  }
  for (int e = 0; e < nell; e++)
    for (int i = 0; i < nfrelt[e]; i++) {
      int g = mhead[(size_t)e * mfrelt + i];
      if (g < 1 || g > ngf) { free(nfrelt); free(mhead); return -4; }
    }
  /* one partition: a freedom is local iff some element has it; local
   * numbers in increasing global order, all inner (inv_perm_map = identity) */
  int *gl = (int *)calloc((size_t)ngf + 1, sizeof(int));
  for (int e = 0; e < nell; e++)
    for (int i = 0; i < nfrelt[e]; i++) gl[mhead[(size_t)e * mfrelt + i]] = 1;
  int nlf = 0;
  for (int g = 1; g <= ngf; g++) if (gl[g]) gl[g] = ++nlf;
  idxmap_t *maps = (idxmap_t *)calloc((size_t)nlf + 1, sizeof(idxmap_t)); /* 1-based rows */
  double *val = NULL, *rhs = (double *)calloc((size_t)nlf + 1, sizeof(double));
  long nval = 0, cap = 0;
  buf = slurp(elemmat, &len);
  if (!buf) { free(gl); free(maps); free(rhs); free(nfrelt); free(mhead); return -5; }
  pos = 0;
  double *elem = (double *)malloc(sizeof(double) * (size_t)mfrelt * (size_t)mfrelt);
  double *erhs = (double *)malloc(sizeof(double) * (size_t)mfrelt);
  int bad = 0;
  for (int e = 0; e < nell && !bad; e++) {
    int nf = nfrelt[e];
    for (int j = 1; j <= nf && !bad; j++) { /* record j: elem(1:nf, j) */
      r = fort_record(buf, len, &pos, &rl, &own);
      if (!r || rl < 8L * nf) bad = 1;
      else for (int k = 1; k <= nf; k++) elem[(size_t)(j - 1) * nf + (k - 1)] = led(r + 8 * (k - 1));
      free(own);
    }
    if (bad) break;
    r = fort_record(buf, len, &pos, &rl, &own);
    if (!r || rl < 8L * nf) { free(own); bad = 1; break; }
    for (int k = 1; k <= nf; k++) erhs[k - 1] = led(r + 8 * (k - 1));
    free(own);
    /* ElemMtxsAssembleContext_addChunk, one element */
    for (int i = 1; i <= nf; i++) {
      int lf = gl[mhead[(size_t)e * mfrelt + i - 1]];
      for (int j = 1; j <= nf; j++) {
        double a = elem[(size_t)(j - 1) * nf + (i - 1)];
        if (a == 0.0) continue;
        int collf = gl[mhead[(size_t)e * mfrelt + j - 1]];
        int idx = idxmap_lookup(&maps[lf], collf);
        if (idx == -1) {
          nval++;
          idx = (int)nval;
          if (cap < nval) {
            long nc = nval * 4 / 3 + 16;
            val = (double *)realloc(val, sizeof(double) * (size_t)(nc + 1));
            for (long q = cap + 1; q <= nc; q++) val[q] = 0.0;
            cap = nc;
          }
          idxmap_insert(&maps[lf], collf, idx);
        }
        val[idx] = val[idx] + a;
      }
      rhs[lf] = rhs[lf] + erhs[i - 1];
    }
  }
  free(buf); free(elem); free(erhs);
  if (bad) {
    for (int i = 1; i <= nlf; i++) { free(maps[i].key); free(maps[i].val); }
    free(maps); free(val); free(rhs); free(gl); free(nfrelt); free(mhead);
    return -5;
  }
  /* _extractSpMtx: rows in order, keys ascending, indi = key, indj = row */
  int *ii = (int *)malloc(sizeof(int) * (size_t)(nval + 1));
  int *jj = (int *)malloc(sizeof(int) * (size_t)(nval + 1));
  double *vv = (double *)malloc(sizeof(double) * (size_t)(nval + 1));
  long bbe = 0;
  for (int i = 1; i <= nlf; i++)
    for (int k = 0; k < maps[i].size; k++) {
      int jkey = maps[i].key[k];
      vv[bbe] = val[idxmap_lookup(&maps[i], jkey)];
      ii[bbe] = jkey;
      jj[bbe] = i;
      bbe++;
    }
  double *b = (double *)malloc(sizeof(double) * (size_t)(nlf + 1));
  for (int i = 0; i < nlf; i++) b[i] = rhs[i + 1];
  for (int i = 1; i <= nlf; i++) { free(maps[i].key); free(maps[i].val); }
  free(maps); free(val); free(rhs); free(gl); free(nfrelt); free(mhead);
  *n_out = nlf;
  *nnz_out = (int)nval;
  *ii_out = ii;
  *jj_out = jj;
  *vv_out = vv;
  *rhs_out = b;
  return 0;
}

void orc_free_buffers(void *a, void *b, void *c, void *d) { free(a); free(b); free(c); free(d); }

static void geom_mesh_free(geom_mesh *G) {
  free(G->coords); free(G->freemap); free(G->nfrelt); free(G->mhead); free(G->lg_fmap);
  memset(G, 0, sizeof *G);
}

/* Mesh_readFromFile for doug_geom (Mesh.F90:293-552): info (nell, ngf,
 * nsd, mfrelt, nnode), the freedom lists, coords(nsd, nnode) in one record
 * and freemap(ngf) in one record; local freedoms = the used freedoms in
 * increasing order (one process).  Returns 0 or a negative error code. */
static int read_geom_mesh(const char *info, const char *freel, const char *coords, const char *freemap,
                          int nblocks, geom_mesh *G) {
  long len, pos, rl;
  unsigned char *own;
  const unsigned char *r;
  unsigned char *buf = slurp(info, &len);
  if (!buf) return -1;
  pos = 0;
  r = fort_record(buf, len, &pos, &rl, &own);
  if (!r || rl < 20) { free(buf); free(own); return -2; }
  G->nell = (int32_t)le32(r); G->ngf = (int32_t)le32(r + 4); G->nsd = (int32_t)le32(r + 8);
  G->mfrelt = (int32_t)le32(r + 12); G->nnode = (int32_t)le32(r + 16);
  free(own); free(buf);
  if (G->nell <= 0 || G->ngf <= 0 || G->nsd <= 0 || G->nsd > 3 || G->mfrelt <= 0 || G->nnode <= 0) return -2;
  G->nfrelt = (int *)xcalloc((size_t)G->nell + 1, sizeof(int));
  G->mhead = (int *)xcalloc((size_t)G->nell * G->mfrelt, sizeof(int));
  buf = slurp(freel, &len);
  if (!buf) return -3;
  pos = 0;
  for (int e = 1; e <= G->nell; e++) {
    r = fort_record(buf, len, &pos, &rl, &own);
    if (!r || rl < 4) { free(own); free(buf); return -3; }
    int nf = (int32_t)le32(r);
    if (nf < 0 || nf > G->mfrelt || rl < 4 + 4L * nf) { free(own); free(buf); return -3; }
    G->nfrelt[e] = nf;
    for (int i = 0; i < nf; i++) G->mhead[(size_t)(e - 1) * G->mfrelt + i] = (int32_t)le32(r + 4 + 4 * i);
    free(own);
  }
  free(buf);
  if (nblocks > 1) {
    int mx = 0;
    for (int e = 1; e <= G->nell; e++)
      for (int i = 0; i < G->nfrelt[e]; i++) if (G->mhead[(size_t)(e - 1) * G->mfrelt + i] > mx) mx = G->mhead[(size_t)(e - 1) * G->mfrelt + i];
    G->ngf = mx;
  }
  buf = slurp(coords, &len);
  if (!buf) return -4;
  pos = 0;
  r = fort_record(buf, len, &pos, &rl, &own);
  if (!r || rl < 8L * G->nsd * G->nnode) { free(own); free(buf); return -4; }
  G->coords = (double *)xcalloc((size_t)G->nsd * G->nnode, sizeof(double));
  for (long q = 0; q < (long)G->nsd * G->nnode; q++) G->coords[q] = led(r + 8 * q);
  free(own); free(buf);
  buf = slurp(freemap, &len);
  if (!buf) return -5;
  pos = 0;
  r = fort_record(buf, len, &pos, &rl, &own);
  if (!r || rl < 4L * G->ngf) { free(own); free(buf); return -5; }
  G->freemap = (int *)xcalloc((size_t)G->ngf + 1, sizeof(int));
  for (int f = 1; f <= G->ngf; f++) {
    G->freemap[f] = (int32_t)le32(r + 4 * (f - 1));
    if (G->freemap[f] < 1 || G->freemap[f] > G->nnode) { free(own); free(buf); return -6; }
  }
  free(own); free(buf);
  char *usedf = (char *)xcalloc((size_t)G->ngf + 1, 1);
  for (int e = 1; e <= G->nell; e++)
    for (int i = 0; i < G->nfrelt[e]; i++) {
      int g = G->mhead[(size_t)(e - 1) * G->mfrelt + i];
      if (g < 1 || g > G->ngf) { free(usedf); return -7; }
      usedf[g] = 1;
    }
  G->lg_fmap = (int *)xcalloc((size_t)G->ngf + 1, sizeof(int));
  G->nlf = 0;
  for (int g = 1; g <= G->ngf; g++) if (usedf[g]) G->lg_fmap[++G->nlf] = g;
  free(usedf);
  return 0;
}

static int run_ctl_common(const char *ctl_path, const char *overrides, const int *part, int nparts,
                          orc_result **out);
int orc_run_ctl(const char *ctl_path, const char *overrides, orc_result **out) {
  return run_ctl_common(ctl_path, overrides, NULL, 0, out);
}
int orc_run_ctl_part(const char *ctl_path, const char *overrides, const int *part, int nparts,
                     orc_result **out) {
  return run_ctl_common(ctl_path, overrides, part, nparts, out);
}
static int run_ctl_common(const char *ctl_path, const char *overrides, const int *part, int nparts,
                          orc_result **out) {
  *out = NULL;
  long len = 0;
  unsigned char *txt = slurp(ctl_path, &len);
  if (!txt) {
    orc_result *r = (orc_result *)calloc(1, sizeof(orc_result));
    r->status = -1;
    snprintf(r->errmsg, sizeof r->errmsg, "Unable to open DOUG control file: %s", ctl_path);
    *out = r;
    return -1;
  }
  size_t ol = overrides ? strlen(overrides) : 0;
  char *all = (char *)malloc(ol + (size_t)len + 2);
  memcpy(all, overrides ? overrides : "", ol);
  all[ol] = '\n';
  memcpy(all + ol + 1, txt, (size_t)len);
  all[ol + 1 + len] = 0;
  free(txt);
  /* resolve input files relative to the control file's directory */
  char dir[1024];
  snprintf(dir, sizeof dir, "%s", ctl_path);
  char *slash = strrchr(dir, '/');
  if (slash) *slash = 0; else snprintf(dir, sizeof dir, ".");
  ctl_t c;
  int rc;
  orc_result *r = NULL;
  if (setjmp(g_jmp)) {
    r = (orc_result *)calloc(1, sizeof(orc_result));
    r->status = -1;
    snprintf(r->errmsg, sizeof r->errmsg, "%s", g_err);
    *out = r;
    free(all);
    return -1;
  }
  ctl_defaults(&c);
  ctl_parse_text(&c, all);
  if (c.input_type == 1) { /* elemental input (Distribution.F90:62-64) */
    char ip[1400], fp[1400], ep[1400];
#define ORC_PATH(dst, name) \
    if (name[0] == '/') snprintf(dst, sizeof dst, "%s", name); else snprintf(dst, sizeof dst, "%s/%s", dir, name);
    ORC_PATH(ip, c.info_file) ORC_PATH(fp, c.freedom_lists_file) ORC_PATH(ep, c.elemmat_rhs_file)
#undef ORC_PATH
    int n, nnz, *ii, *jj;
    double *vv, *rhs;
    rc = orc_read_elemental(ip, fp, ep, c.number_of_blocks, &n, &nnz, &ii, &jj, &vv, &rhs);
    if (rc) orc_abort("Unable to read elemental input (%d)", rc);
    geom_mesh G;
    memset(&G, 0, sizeof G);
    int have_geom = 0;
    if (c.executable == 1 && c.coords_file[0] && c.freemap_file[0]) {
      char cp[1400], mp[1400];
#define ORC_PATH(dst, name) \
      if (name[0] == '/') snprintf(dst, sizeof dst, "%s", name); else snprintf(dst, sizeof dst, "%s/%s", dir, name);
      ORC_PATH(cp, c.coords_file) ORC_PATH(mp, c.freemap_file)
#undef ORC_PATH
      rc = read_geom_mesh(ip, fp, cp, mp, c.number_of_blocks, &G);
      if (rc) orc_abort("Unable to read the node coordinates / freemap (%d)", rc);
      have_geom = 1;
    }
    rc = run_common(n, nnz, ii, jj, vv, rhs, all, part, nparts, 1, have_geom ? &G : NULL, &r);
    geom_mesh_free(&G);
    free(ii); free(jj); free(vv); free(rhs); free(all);
    *out = r;
    return rc;
  }
  if (c.input_type == 3) { /* Distribution_struct_NewInit (Distribution_struct.F90:36-147), one process */
    int g = c.grid_size < 1 ? 100 : c.grid_size; /* Distribution.F90:69 */
    int n = g * g, cap = 5 * n, nnz = 0;
    int *ii = (int *)malloc(sizeof(int) * (size_t)cap), *jj = (int *)malloc(sizeof(int) * (size_t)cap);
    double *vv = (double *)malloc(sizeof(double) * (size_t)cap), *rhs = (double *)malloc(sizeof(double) * (size_t)n);
    for (int ri = 1; ri <= g; ri++)
      for (int ci = 1; ci <= g; ci++) {
        int mri = (ri - 1) * g + ci;
        ii[nnz] = mri; jj[nnz] = mri; vv[nnz++] = 4;             /* diagonal */
        if (ci > 1) { ii[nnz] = mri; jj[nnz] = mri - 1; vv[nnz++] = -1; } /* left */
        if (ci < g) { ii[nnz] = mri; jj[nnz] = mri + 1; vv[nnz++] = -1; } /* right */
        if (ri > 1) { ii[nnz] = mri; jj[nnz] = mri - g; vv[nnz++] = -1; } /* up */
        if (ri < g) { ii[nnz] = mri; jj[nnz] = mri + g; vv[nnz++] = -1; } /* down */
      }
    for (int i = 0; i < n; i++) rhs[i] = -1;
    rc = orc_run_coo(n, nnz, ii, jj, vv, rhs, all, part, nparts, &r);
    free(ii); free(jj); free(vv); free(rhs); free(all);
    *out = r;
    return rc;
  }
  if (c.input_type != 2) orc_abort("input_type %d not supported by the oracle", c.input_type);
  char mpath[1400], rpath[1400];
  if (c.assembled_mtx_file[0] == '/') snprintf(mpath, sizeof mpath, "%s", c.assembled_mtx_file);
  else snprintf(mpath, sizeof mpath, "%s/%s", dir, c.assembled_mtx_file);
  int n, nnz, *ii, *jj;
  double *vv;
  rc = orc_read_assembled(mpath, c.assembled_mtx_format < 0 ? 0 : c.assembled_mtx_format,
                          &n, &nnz, &ii, &jj, &vv);
  if (rc) orc_abort("Unable to read assembled file: %s (%d)", mpath, rc);
  int nn = n > nnz ? nnz : n;
  double *rhs = NULL;
  if (c.assembled_rhs_file[0]) {
    if (c.assembled_rhs_file[0] == '/') snprintf(rpath, sizeof rpath, "%s", c.assembled_rhs_file);
    else snprintf(rpath, sizeof rpath, "%s/%s", dir, c.assembled_rhs_file);
    rhs = (double *)malloc(sizeof(double) * (size_t)nn);
    rc = orc_read_vector(rpath, c.assembled_rhs_format < 0 ? 1 : c.assembled_rhs_format, nn, rhs);
    if (rc) orc_abort("Unable to read rhs file: %s (%d)", rpath, rc);
  }
  int nz2 = n > nnz ? n : nnz;
  rc = orc_run_coo(nn, nz2, ii, jj, vv, rhs, all, part, nparts, &r);
  free(ii); free(jj); free(vv); free(rhs); free(all);
  *out = r;
  return rc;
}
