/*
 * spchol.c -- exact sparse Cholesky of the oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Nested dissection (level-set separators) -> elimination tree -> postorder
 * -> column counts -> fundamental supernodes -> multifrontal numeric
 * factorisation with blocked dense kernels -> supernodal triangular solves.
 * The method is the published one named in spchol.h; this is a restatement
 * for the oracle's exact subdomain and coarse solves, standing in for the
 * reference's UMFPACK (src/solvers/Fact.F90:102-159, 246-281).
 */
#include "spchol.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct spchol {
  int n;
  int *perm;     /* new -> old */
  int nsuper;
  int *sfirst;   /* nsuper+1: supernode s owns columns [sfirst[s], sfirst[s+1]) */
  long *rptr;    /* nsuper+1: front row lists in rows[] */
  int *rows;     /* per supernode its front rows (new numbering), its own columns first */
  long *lptr;    /* nsuper+1: per supernode an m x k column-major block in L */
  double *L;
  double flops;
  int maxm;      /* largest front */
};

#define ND_LEAF 48
#define NB 64

static void *zalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* ------------------------------------------------------------------ */
/* nested dissection by breadth-first level-set separators              */
/* ------------------------------------------------------------------ */
typedef struct { int off, cnt, out; } ndtask;

typedef struct {
  const int *adjp, *adj;
  int *mark, *vis, *level, *queue;
  int vstamp;
} ndctx;

/* BFS from root over the vertices marked `tag`; returns the number reached,
 * fills queue[0..reached) in BFS order and level[], *nlev and *last. */
static int nd_bfs(ndctx *c, int root, int tag, int *nlev, int *last) {
  int h = 0, t = 0;
  c->vstamp++;
  c->queue[t++] = root;
  c->vis[root] = c->vstamp;
  c->level[root] = 0;
  int maxl = 0;
  while (h < t) {
    int v = c->queue[h++];
    int lv = c->level[v];
    if (lv > maxl) maxl = lv;
    for (int k = c->adjp[v]; k < c->adjp[v + 1]; k++) {
      int w = c->adj[k];
      if (c->mark[w] == tag && c->vis[w] != c->vstamp) {
        c->vis[w] = c->vstamp;
        c->level[w] = lv + 1;
        c->queue[t++] = w;
      }
    }
  }
  *nlev = maxl + 1;
  *last = c->queue[t - 1];
  return t;
}

static int nd_order(int n, const int *adjp, const int *adj, int *order) {
  ndctx c;
  c.adjp = adjp; c.adj = adj;
  c.mark = (int *)zalloc((size_t)n, sizeof(int));
  c.vis = (int *)zalloc((size_t)n, sizeof(int));
  c.level = (int *)zalloc((size_t)n, sizeof(int));
  c.queue = (int *)zalloc((size_t)n, sizeof(int));
  c.vstamp = 0;
  int *verts = (int *)zalloc((size_t)n, sizeof(int));
  int *tmp = (int *)zalloc((size_t)n, sizeof(int));
  int *lsz = (int *)zalloc((size_t)n + 1, sizeof(int));
  int cap = 64, top = 0, tag = 0;
  ndtask *st = (ndtask *)malloc(sizeof(ndtask) * (size_t)cap);
  if (!c.mark || !c.vis || !c.level || !c.queue || !verts || !tmp || !lsz || !st) {
    free(c.mark); free(c.vis); free(c.level); free(c.queue); free(verts); free(tmp); free(lsz); free(st);
    return -1;
  }
  for (int i = 0; i < n; i++) verts[i] = i;
  st[top++] = (ndtask){0, n, 0};
  while (top > 0) {
    ndtask T = st[--top];
    int *seg = verts + T.off;
    if (T.cnt <= ND_LEAF) {
      for (int t = 0; t < T.cnt; t++) order[T.out + t] = seg[t];
      continue;
    }
    tag++;
    for (int t = 0; t < T.cnt; t++) c.mark[seg[t]] = tag;
    int nlev, last;
    int reached = nd_bfs(&c, seg[0], tag, &nlev, &last);
    if (reached < T.cnt) { /* disconnected: the reached component first, then the rest */
      int stamp = c.vstamp, a = 0, b = reached;
      for (int t = 0; t < reached; t++) tmp[a++] = c.queue[t];
      for (int t = 0; t < T.cnt; t++)
        if (c.vis[seg[t]] != stamp) tmp[b++] = seg[t];
      memcpy(seg, tmp, sizeof(int) * (size_t)T.cnt);
      if (top + 2 > cap) { cap *= 2; st = (ndtask *)realloc(st, sizeof(ndtask) * (size_t)cap); }
      st[top++] = (ndtask){T.off + reached, T.cnt - reached, T.out + reached};
      st[top++] = (ndtask){T.off, reached, T.out};
      continue;
    }
    /* pseudo-peripheral root: restart from the last vertex while the
     * eccentricity grows (at most three sweeps) */
    for (int sweep = 0; sweep < 3; sweep++) {
      int nl2, last2;
      int root = last;
      nd_bfs(&c, root, tag, &nl2, &last2);
      if (nl2 <= nlev && sweep > 0) { nlev = nl2; last = last2; break; }
      nlev = nl2; last = last2;
    }
    if (nlev < 3) {
      for (int t = 0; t < T.cnt; t++) order[T.out + t] = c.queue[t];
      continue;
    }
    for (int l = 0; l < nlev; l++) lsz[l] = 0;
    for (int t = 0; t < T.cnt; t++) lsz[c.level[c.queue[t]]]++;
    /* the smallest level with at least a quarter of the vertices on each side */
    int best = -1, before = 0;
    for (int l = 0; l < nlev; l++) {
      int after = T.cnt - before - lsz[l];
      if (l >= 1 && l <= nlev - 2 && 4 * before >= T.cnt && 4 * after >= T.cnt)
        if (best < 0 || lsz[l] < lsz[best]) best = l;
      before += lsz[l];
    }
    if (best < 0) {
      before = 0;
      for (int l = 0; l < nlev; l++) {
        if (2 * (before + lsz[l]) > T.cnt) { best = l; break; }
        before += lsz[l];
      }
      if (best < 1) best = 1;
      if (best > nlev - 2) best = nlev - 2;
    }
    int na = 0, nb = 0, ns = 0;
    for (int t = 0; t < T.cnt; t++) {
      int l = c.level[c.queue[t]];
      if (l < best) na++;
      else if (l > best) nb++;
      else ns++;
    }
    int pa = 0, pb = na, ps = na + nb;
    for (int t = 0; t < T.cnt; t++) {
      int v = c.queue[t], l = c.level[v];
      if (l < best) tmp[pa++] = v;
      else if (l > best) tmp[pb++] = v;
      else tmp[ps++] = v;
    }
    memcpy(seg, tmp, sizeof(int) * (size_t)T.cnt);
    for (int t = 0; t < ns; t++) order[T.out + na + nb + t] = seg[na + nb + t];
    if (top + 2 > cap) { cap *= 2; st = (ndtask *)realloc(st, sizeof(ndtask) * (size_t)cap); }
    if (nb > 0) st[top++] = (ndtask){T.off + na, nb, T.out + na};
    if (na > 0) st[top++] = (ndtask){T.off, na, T.out};
  }
  free(c.mark); free(c.vis); free(c.level); free(c.queue); free(verts); free(tmp); free(lsz); free(st);
  return 0;
}

/* ------------------------------------------------------------------ */
/* dense kernels on a front (column-major, leading dimension m)          */
/* ------------------------------------------------------------------ */

/* C[i,c] -= sum_t P[t][i] P[t][c] for 0 <= c <= i < R; P is t-major with
 * row stride RP (a multiple of 8, rows R..RP-1 zero). */
static void syrk_lower(double *C, long ldc, int R, const double *P, long RP, int K) {
  for (int cb = 0; cb < R; cb += 4) {
    for (int ib = cb & ~7; ib < R; ib += 8) {
      double c0[8] = {0}, c1[8] = {0}, c2[8] = {0}, c3[8] = {0};
      for (int t = 0; t < K; t++) {
        const double *pt = P + (size_t)t * RP;
        const double b0 = pt[cb], b1 = pt[cb + 1], b2 = pt[cb + 2], b3 = pt[cb + 3];
        const double *a = pt + ib;
        for (int r = 0; r < 8; r++) {
          c0[r] += a[r] * b0;
          c1[r] += a[r] * b1;
          c2[r] += a[r] * b2;
          c3[r] += a[r] * b3;
        }
      }
      const double *acc[4] = {c0, c1, c2, c3};
      for (int q = 0; q < 4; q++) {
        int col = cb + q;
        if (col >= R) break;
        double *cc = C + (size_t)col * ldc;
        int r0 = col > ib ? col - ib : 0;
        int r1 = R - ib < 8 ? R - ib : 8;
        for (int r = r0; r < r1; r++) cc[ib + r] -= acc[q][r];
      }
    }
  }
}

/* Cholesky of the k pivot columns of an m x m front; the trailing
 * (m-k) x (m-k) block receives the update.  pack holds NB * round8(m). */
static int partial_chol(double *F, int m, int k, double *pack) {
  for (int p0 = 0; p0 < k; p0 += NB) {
    int pb = k - p0 < NB ? k - p0 : NB;
    for (int j = p0; j < p0 + pb; j++) {
      double *cj = F + (size_t)j * m;
      double d = cj[j];
      if (!(d > 0.0)) return -1;
      d = sqrt(d);
      cj[j] = d;
      for (int i = j + 1; i < m; i++) cj[i] /= d;
      for (int jj = j + 1; jj < p0 + pb; jj++) {
        double *cjj = F + (size_t)jj * m;
        const double f = cj[jj];
        for (int i = jj; i < m; i++) cjj[i] -= cj[i] * f;
      }
    }
    int r0 = p0 + pb, R = m - r0;
    if (R <= 0) continue;
    long RP = (R + 7) & ~7;
    for (int t = 0; t < pb; t++) {
      const double *src = F + (size_t)(p0 + t) * m + r0;
      double *dst = pack + (size_t)t * RP;
      memcpy(dst, src, sizeof(double) * (size_t)R);
      for (long i = R; i < RP; i++) dst[i] = 0.0;
    }
    syrk_lower(F + (size_t)r0 * m + r0, m, R, pack, RP, pb);
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* symbolic + numeric factorisation                                     */
/* ------------------------------------------------------------------ */
spchol *spchol_factor(int n, long nnz, const int *ii, const int *jj, const double *vv,
                      char *err, int errsz) {
  spchol *f = (spchol *)calloc(1, sizeof(spchol));
  int *deg = NULL, *adjp = NULL, *adj = NULL, *fillc = NULL, *order = NULL, *iperm = NULL;
  int *lp = NULL, *li = NULL, *parent = NULL, *anc = NULL, *cnt = NULL, *mark = NULL;
  int *head = NULL, *next = NULL, *post = NULL, *stack = NULL, *map = NULL, *snode = NULL;
  int *nchild = NULL, *chead = NULL, *cnext = NULL, *rbuf = NULL;
  long *cp = NULL;
  double *cv = NULL, *pack = NULL;
  double **front = NULL;
  if (!f) goto oom;
  f->n = n;
  if (n <= 0) {
    f->perm = (int *)zalloc(1, sizeof(int));
    f->sfirst = (int *)zalloc(1, sizeof(int));
    f->rptr = (long *)zalloc(1, sizeof(long));
    f->lptr = (long *)zalloc(1, sizeof(long));
    f->rows = (int *)zalloc(1, sizeof(int));
    f->L = (double *)zalloc(1, sizeof(double));
    return f;
  }
  /* symmetric adjacency without the diagonal, deduplicated */
  deg = (int *)zalloc((size_t)n + 1, sizeof(int));
  adjp = (int *)zalloc((size_t)n + 1, sizeof(int));
  if (!deg || !adjp) goto oom;
  for (long k = 0; k < nnz; k++)
    if (ii[k] != jj[k]) { deg[ii[k]]++; deg[jj[k]]++; }
  for (int i = 0; i < n; i++) adjp[i + 1] = adjp[i] + deg[i];
  adj = (int *)zalloc((size_t)adjp[n] + 1, sizeof(int));
  fillc = (int *)zalloc((size_t)n, sizeof(int));
  mark = (int *)zalloc((size_t)n, sizeof(int));
  if (!adj || !fillc || !mark) goto oom;
  for (long k = 0; k < nnz; k++)
    if (ii[k] != jj[k]) {
      adj[adjp[ii[k]] + fillc[ii[k]]++] = jj[k];
      adj[adjp[jj[k]] + fillc[jj[k]]++] = ii[k];
    }
  for (int i = 0; i < n; i++) mark[i] = -1;
  {
    int w = 0;
    for (int i = 0; i < n; i++) {
      int s0 = adjp[i], e0 = adjp[i] + fillc[i];
      adjp[i] = w;
      for (int k = s0; k < e0; k++)
        if (mark[adj[k]] != i) { mark[adj[k]] = i; adj[w++] = adj[k]; }
    }
    adjp[n] = w;
  }
  order = (int *)zalloc((size_t)n, sizeof(int));
  iperm = (int *)zalloc((size_t)n, sizeof(int));
  if (!order || !iperm) goto oom;
  if (nd_order(n, adjp, adj, order)) goto oom;
  for (int i = 0; i < n; i++) iperm[order[i]] = i;

  /* lower-triangular rows of the permuted pattern (row i: columns j < i) */
  lp = (int *)zalloc((size_t)n + 1, sizeof(int));
  if (!lp) goto oom;
  for (int v = 0; v < n; v++)
    for (int k = adjp[v]; k < adjp[v + 1]; k++)
      if (iperm[adj[k]] < iperm[v]) lp[iperm[v] + 1]++;
  for (int i = 0; i < n; i++) lp[i + 1] += lp[i];
  li = (int *)zalloc((size_t)lp[n] + 1, sizeof(int));
  parent = (int *)zalloc((size_t)n, sizeof(int));
  anc = (int *)zalloc((size_t)n, sizeof(int));
  if (!li || !parent || !anc) goto oom;
  for (int i = 0; i < n; i++) fillc[i] = lp[i];
  for (int v = 0; v < n; v++)
    for (int k = adjp[v]; k < adjp[v + 1]; k++)
      if (iperm[adj[k]] < iperm[v]) li[fillc[iperm[v]]++] = iperm[adj[k]];
  /* elimination tree (Liu) */
  for (int i = 0; i < n; i++) {
    parent[i] = -1; anc[i] = -1;
    for (int k = lp[i]; k < lp[i + 1]; k++) {
      int j = li[k];
      while (j != -1 && j < i) {
        int nx = anc[j];
        anc[j] = i;
        if (nx == -1) { parent[j] = i; break; }
        j = nx;
      }
    }
  }
  /* postorder */
  head = (int *)zalloc((size_t)n, sizeof(int));
  next = (int *)zalloc((size_t)n, sizeof(int));
  post = (int *)zalloc((size_t)n, sizeof(int));
  stack = (int *)zalloc((size_t)n, sizeof(int));
  if (!head || !next || !post || !stack) goto oom;
  for (int i = 0; i < n; i++) head[i] = -1;
  for (int j = n - 1; j >= 0; j--)
    if (parent[j] != -1) { next[j] = head[parent[j]]; head[parent[j]] = j; }
  {
    int k = 0;
    for (int r = 0; r < n; r++) {
      if (parent[r] != -1) continue;
      int top = 0;
      stack[top++] = r;
      while (top > 0) {
        int p = stack[top - 1];
        int ch = head[p];
        if (ch == -1) { top--; post[k++] = p; }
        else { head[p] = next[ch]; stack[top++] = ch; }
      }
    }
  }
  /* compose: new order = ND order taken in postorder; rebuild rows + etree */
  f->perm = (int *)zalloc((size_t)n, sizeof(int));
  if (!f->perm) goto oom;
  for (int k = 0; k < n; k++) f->perm[k] = order[post[k]];
  for (int k = 0; k < n; k++) iperm[f->perm[k]] = k;
  memset(lp, 0, sizeof(int) * ((size_t)n + 1));
  for (int v = 0; v < n; v++)
    for (int k = adjp[v]; k < adjp[v + 1]; k++)
      if (iperm[adj[k]] < iperm[v]) lp[iperm[v] + 1]++;
  for (int i = 0; i < n; i++) lp[i + 1] += lp[i];
  for (int i = 0; i < n; i++) fillc[i] = lp[i];
  for (int v = 0; v < n; v++)
    for (int k = adjp[v]; k < adjp[v + 1]; k++)
      if (iperm[adj[k]] < iperm[v]) li[fillc[iperm[v]]++] = iperm[adj[k]];
  for (int i = 0; i < n; i++) {
    parent[i] = -1; anc[i] = -1;
    for (int k = lp[i]; k < lp[i + 1]; k++) {
      int j = li[k];
      while (j != -1 && j < i) {
        int nx = anc[j];
        anc[j] = i;
        if (nx == -1) { parent[j] = i; break; }
        j = nx;
      }
    }
  }
  /* column counts by row subtrees */
  cnt = (int *)zalloc((size_t)n, sizeof(int));
  if (!cnt) goto oom;
  for (int i = 0; i < n; i++) mark[i] = -1;
  for (int i = 0; i < n; i++) {
    cnt[i]++; /* diagonal */
    mark[i] = i;
    for (int k = lp[i]; k < lp[i + 1]; k++) {
      int j = li[k];
      while (mark[j] != i) { cnt[j]++; mark[j] = i; j = parent[j]; }
    }
  }
  /* fundamental supernodes */
  nchild = (int *)zalloc((size_t)n, sizeof(int));
  snode = (int *)zalloc((size_t)n, sizeof(int));
  if (!nchild || !snode) goto oom;
  for (int j = 0; j < n; j++) if (parent[j] != -1) nchild[parent[j]]++;
  f->sfirst = (int *)zalloc((size_t)n + 1, sizeof(int));
  if (!f->sfirst) goto oom;
  {
    int ns = 0;
    for (int j = 0; j < n; j++) {
      int merge = j > 0 && parent[j - 1] == j && cnt[j - 1] == cnt[j] + 1 && nchild[j] == 1;
      if (!merge) f->sfirst[ns++] = j;
      snode[j] = ns - 1;
    }
    f->sfirst[ns] = n;
    f->nsuper = ns;
  }
  int ns = f->nsuper;
  /* front row lists: own columns, then A's rows below and the children's
   * update rows, ascending */
  f->rptr = (long *)zalloc((size_t)ns + 1, sizeof(long));
  f->lptr = (long *)zalloc((size_t)ns + 1, sizeof(long));
  if (!f->rptr || !f->lptr) goto oom;
  for (int s = 0; s < ns; s++) {
    int j0 = f->sfirst[s], k = f->sfirst[s + 1] - j0, m = cnt[j0];
    f->rptr[s + 1] = f->rptr[s] + m;
    f->lptr[s + 1] = f->lptr[s] + (long)m * k;
    f->flops += (double)k * k * k / 3.0 + (double)(m - k) * k * k + (double)(m - k) * (m - k) * k;
  }
  f->rows = (int *)zalloc((size_t)f->rptr[ns] + 1, sizeof(int));
  /* the lower CSC of the permuted matrix with values, for assembly */
  cp = (long *)zalloc((size_t)n + 1, sizeof(long));
  if (!f->rows || !cp) goto oom;
  for (long k = 0; k < nnz; k++) {
    int r = iperm[ii[k]], c = iperm[jj[k]];
    if (r >= c) cp[c + 1]++;
  }
  for (int j = 0; j < n; j++) cp[j + 1] += cp[j];
  rbuf = (int *)zalloc((size_t)cp[n] + 1, sizeof(int));
  cv = (double *)zalloc((size_t)cp[n] + 1, sizeof(double));
  if (!rbuf || !cv) goto oom;
  {
    long *pos = (long *)zalloc((size_t)n, sizeof(long));
    if (!pos) goto oom;
    for (int j = 0; j < n; j++) pos[j] = cp[j];
    for (long k = 0; k < nnz; k++) {
      int r = iperm[ii[k]], c = iperm[jj[k]];
      if (r >= c) { rbuf[pos[c]] = r; cv[pos[c]] = vv[k]; pos[c]++; }
    }
    free(pos);
  }
  chead = (int *)zalloc((size_t)ns, sizeof(int));
  cnext = (int *)zalloc((size_t)ns, sizeof(int));
  if (!chead || !cnext) goto oom;
  for (int s = 0; s < ns; s++) chead[s] = -1;
  for (int s = ns - 1; s >= 0; s--) {
    int last = f->sfirst[s + 1] - 1;
    int p = parent[last];
    if (p != -1) { int ps = snode[p]; cnext[s] = chead[ps]; chead[ps] = s; }
  }
  for (int i = 0; i < n; i++) mark[i] = -1;
  for (int s = 0; s < ns; s++) {
    int j0 = f->sfirst[s], j1 = f->sfirst[s + 1], k = j1 - j0, m = cnt[j0];
    int *rw = f->rows + f->rptr[s];
    int nr = 0;
    for (int j = j0; j < j1; j++) { rw[nr++] = j; mark[j] = s; }
    for (int j = j0; j < j1; j++)
      for (long q = cp[j]; q < cp[j + 1]; q++) {
        int r = rbuf[q];
        if (mark[r] != s) { mark[r] = s; rw[nr++] = r; }
      }
    for (int ch = chead[s]; ch != -1; ch = cnext[ch]) {
      const int *cr = f->rows + f->rptr[ch];
      int ck = f->sfirst[ch + 1] - f->sfirst[ch], cm = (int)(f->rptr[ch + 1] - f->rptr[ch]);
      for (int a = ck; a < cm; a++)
        if (mark[cr[a]] != s) { mark[cr[a]] = s; rw[nr++] = cr[a]; }
    }
    if (nr != m) { snprintf(err, (size_t)errsz, "spchol: front %d has %d rows, column count %d", s, nr, m); goto fail; }
    /* insertion sort of the rows below the supernode (short lists) */
    for (int a = k + 1; a < m; a++) {
      int x = rw[a], b = a - 1;
      while (b >= k && rw[b] > x) { rw[b + 1] = rw[b]; b--; }
      rw[b + 1] = x;
    }
  }
  /* numeric: multifrontal in postorder */
  f->L = (double *)malloc(sizeof(double) * ((size_t)f->lptr[ns] + 1));
  front = (double **)zalloc((size_t)ns, sizeof(double *));
  map = (int *)zalloc((size_t)n, sizeof(int));
  int maxm = 1;
  for (int s = 0; s < ns; s++) {
    int m = (int)(f->rptr[s + 1] - f->rptr[s]);
    if (m > maxm) maxm = m;
  }
  f->maxm = maxm;
  pack = (double *)malloc(sizeof(double) * (size_t)NB * (size_t)((maxm + 7) & ~7));
  if (!f->L || !front || !map || !pack) goto oom;
  for (int s = 0; s < ns; s++) {
    int j0 = f->sfirst[s], j1 = f->sfirst[s + 1], k = j1 - j0;
    int m = (int)(f->rptr[s + 1] - f->rptr[s]);
    const int *rw = f->rows + f->rptr[s];
    double *F = (double *)calloc((size_t)m * m, sizeof(double));
    if (!F) goto oom;
    for (int a = 0; a < m; a++) map[rw[a]] = a;
    for (int j = j0; j < j1; j++) {
      double *col = F + (size_t)(j - j0) * m;
      for (long q = cp[j]; q < cp[j + 1]; q++) col[map[rbuf[q]]] += cv[q];
    }
    for (int ch = chead[s]; ch != -1; ch = cnext[ch]) {
      const int *cr = f->rows + f->rptr[ch];
      int ck = f->sfirst[ch + 1] - f->sfirst[ch], cm = (int)(f->rptr[ch + 1] - f->rptr[ch]);
      double *U = front[ch];
      for (int b = ck; b < cm; b++) {
        double *dst = F + (size_t)map[cr[b]] * m;
        const double *src = U + (size_t)b * cm;
        for (int a = b; a < cm; a++) dst[map[cr[a]]] += src[a];
      }
      free(U);
      front[ch] = NULL;
    }
    if (partial_chol(F, m, k, pack)) {
      snprintf(err, (size_t)errsz, "matrix not positive definite (pivot in columns %d..%d)", j0, j1 - 1);
      free(F);
      goto fail;
    }
    memcpy(f->L + f->lptr[s], F, sizeof(double) * (size_t)m * k);
    if (m > k) front[s] = F;
    else free(F);
  }
  goto done;
oom:
  snprintf(err, (size_t)errsz, "spchol: out of memory (n = %d)", n);
fail:
  if (front) for (int s = 0; s < f->nsuper; s++) free(front[s]);
  spchol_free(f);
  f = NULL;
done:
  free(deg); free(adjp); free(adj); free(fillc); free(order); free(iperm); free(lp); free(li);
  free(parent); free(anc); free(cnt); free(mark); free(head); free(next); free(post); free(stack);
  free(map); free(snode); free(nchild); free(chead); free(cnext); free(rbuf); free(cp); free(cv);
  free(pack); free(front);
  return f;
}

void spchol_solve(const spchol *f, const double *b, double *x, double *w) {
  int n = f->n;
  double *g = w + n; /* gathered rows below a supernode */
  for (int i = 0; i < n; i++) w[i] = b[f->perm[i]];
  for (int s = 0; s < f->nsuper; s++) {
    int j0 = f->sfirst[s], k = f->sfirst[s + 1] - j0;
    int m = (int)(f->rptr[s + 1] - f->rptr[s]), mb = m - k;
    const int *rw = f->rows + f->rptr[s] + k;
    const double *Ls = f->L + f->lptr[s];
    double *y = w + j0;
    for (int a = 0; a < mb; a++) g[a] = 0.0;
    for (int t = 0; t < k; t++) {
      const double *c = Ls + (size_t)t * m;
      const double v = y[t] / c[t];
      y[t] = v;
      for (int a = t + 1; a < k; a++) y[a] -= c[a] * v;
      const double *cb = c + k;
      for (int a = 0; a < mb; a++) g[a] += cb[a] * v;
    }
    for (int a = 0; a < mb; a++) w[rw[a]] -= g[a];
  }
  for (int s = f->nsuper - 1; s >= 0; s--) {
    int j0 = f->sfirst[s], k = f->sfirst[s + 1] - j0;
    int m = (int)(f->rptr[s + 1] - f->rptr[s]), mb = m - k;
    const int *rw = f->rows + f->rptr[s] + k;
    const double *Ls = f->L + f->lptr[s];
    double *y = w + j0;
    for (int a = 0; a < mb; a++) g[a] = w[rw[a]];
    for (int t = k - 1; t >= 0; t--) {
      const double *c = Ls + (size_t)t * m;
      const double *cb = c + k;
      double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
      int a = 0;
      for (; a + 4 <= mb; a += 4) {
        v0 += cb[a] * g[a]; v1 += cb[a + 1] * g[a + 1];
        v2 += cb[a + 2] * g[a + 2]; v3 += cb[a + 3] * g[a + 3];
      }
      for (; a < mb; a++) v0 += cb[a] * g[a];
      double v = y[t] - ((v0 + v1) + (v2 + v3));
      for (a = t + 1; a < k; a++) v -= c[a] * y[a];
      y[t] = v / c[t];
    }
  }
  for (int i = 0; i < n; i++) x[f->perm[i]] = w[i];
}

void spchol_free(spchol *f) {
  if (!f) return;
  free(f->perm); free(f->sfirst); free(f->rptr); free(f->rows); free(f->lptr); free(f->L);
  free(f);
}

long spchol_work_size(const spchol *f) { return (long)f->n + f->maxm + 1; }
long spchol_nnz(const spchol *f) { return f ? f->lptr[f->nsuper] : 0; }
double spchol_flops(const spchol *f) { return f ? f->flops : 0.0; }
