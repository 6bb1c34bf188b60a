// Nested-dissection ordering and multifrontal symbolic factorisation on the
// host.  The numeric work happens on the GPU (mf_kernels.cu).
#include "mf_symbolic.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <stdexcept>
#include <thread>

namespace dg {
namespace {

struct Graph {  // symmetric adjacency without self loops
  int n = 0;
  std::vector<int64_t> ptr;
  std::vector<int> adj;
};

// One matrix' symbolic result before it is placed into the batch.
struct Local {
  int n = 0;
  std::vector<int> perm;      // new -> local
  std::vector<int> iperm;     // local -> new
  // fronts in creation (post) order
  std::vector<int> p0, k, parent, level;
  std::vector<std::vector<int>> children;
  std::vector<std::vector<int>> rows;  // pivots then update rows (new numbering)
  // lower-triangle entries: (new row, new col, source index)
  std::vector<int> er, ec;
  std::vector<int64_t> es;
};

class Dissector {
 public:
  Dissector(const Graph &g, int leaf, Local &L) : g_(g), leaf_(leaf), L_(L) {
    mark_.assign((size_t)g.n, 0);
    lev_.assign((size_t)g.n, -1);
  }

  void run() {
    std::vector<int> all((size_t)g_.n);
    for (int i = 0; i < g_.n; i++) all[(size_t)i] = i;
    std::vector<int> roots;
    dissect(all, roots);
  }

 private:
  // BFS restricted to the set stamped with `stamp`; returns visit order and
  // fills lev_ for visited nodes.
  void bfs(int s, int stamp, std::vector<int> &order, int &nlev) {
    order.clear();
    order.push_back(s);
    lev_[(size_t)s] = 0;
    mark_[(size_t)s] = -stamp;
    nlev = 1;
    for (size_t h = 0; h < order.size(); h++) {
      int v = order[h];
      for (int64_t e = g_.ptr[(size_t)v]; e < g_.ptr[(size_t)v + 1]; e++) {
        int w = g_.adj[(size_t)e];
        if (mark_[(size_t)w] == stamp) {
          mark_[(size_t)w] = -stamp;
          lev_[(size_t)w] = lev_[(size_t)v] + 1;
          nlev = std::max(nlev, lev_[(size_t)w] + 1);
          order.push_back(w);
        }
      }
    }
    for (int v : order) mark_[(size_t)v] = stamp;  // restore membership
  }

  int new_front(const std::vector<int> &piv) {
    int f = (int)L_.p0.size();
    L_.p0.push_back((int)L_.perm.size());
    L_.k.push_back((int)piv.size());
    L_.parent.push_back(-1);
    L_.level.push_back(0);
    L_.children.emplace_back();
    for (int v : piv) L_.perm.push_back(v);
    return f;
  }

  void dissect(std::vector<int> &nodes, std::vector<int> &roots) {
    roots.clear();
    if (nodes.empty()) return;
    int stamp = ++stamp_;
    for (int v : nodes) mark_[(size_t)v] = stamp;
    // connected components
    std::vector<int> order;
    std::vector<std::vector<int>> comps;
    {
      int cstamp = ++stamp_;
      (void)cstamp;
      std::vector<char> seen;
      for (int v : nodes) {
        if (mark_[(size_t)v] != stamp) continue;  // already taken by a component
        int nl;
        bfs(v, stamp, order, nl);
        for (int w : order) mark_[(size_t)w] = 0;  // remove from the pending set
        comps.push_back(order);
      }
    }
    if (comps.size() > 1) {
      // components larger than a leaf are dissected on their own; the small
      // ones are packed together into leaf fronts (one dense front may hold
      // several disconnected pieces), which keeps tiny fronts with large
      // boundaries out of the tree
      std::vector<int> pack;
      auto flush = [&]() {
        if (!pack.empty()) { roots.push_back(new_front(pack)); pack.clear(); }
      };
      for (auto &c : comps) {
        if ((int)c.size() > leaf_) {
          std::vector<int> r;
          dissect(c, r);
          roots.insert(roots.end(), r.begin(), r.end());
        } else {
          if ((int)(pack.size() + c.size()) > leaf_) flush();
          pack.insert(pack.end(), c.begin(), c.end());
        }
      }
      flush();
      return;
    }
    std::vector<int> &S = comps[0];
    int N = (int)S.size();
    if (N <= leaf_) {
      roots.push_back(new_front(S));
      return;
    }
    stamp = ++stamp_;
    for (int v : S) mark_[(size_t)v] = stamp;
    // pseudo-peripheral start: two sweeps
    int nl = 0;
    bfs(S[0], stamp, order, nl);
    int s = order.back();
    bfs(s, stamp, order, nl);
    s = order.back();
    bfs(s, stamp, order, nl);
    if (nl < 3) {
      for (int v : S) mark_[(size_t)v] = 0;
      roots.push_back(new_front(S));
      return;
    }
    std::vector<int> cnt((size_t)nl, 0);
    for (int v : order) cnt[(size_t)lev_[(size_t)v]]++;
    // separator: a level near the middle with few nodes
    int best = -1;
    int64_t before = 0;
    double bestscore = 1e300;
    for (int l = 0; l < nl; l++) {
      int64_t after = N - before - cnt[(size_t)l];
      if (l > 0 && l < nl - 1) {
        double bal = std::fabs((double)before - (double)after) / (double)N;
        if (before >= (int64_t)(0.25 * N) && after >= (int64_t)(0.25 * N)) {
          double score = (double)cnt[(size_t)l] * (1.0 + bal);
          if (score < bestscore) { bestscore = score; best = l; }
        }
      }
      before += cnt[(size_t)l];
    }
    if (best < 0) {  // fall back to the median level
      before = 0;
      for (int l = 0; l < nl; l++) {
        if (before + cnt[(size_t)l] >= N / 2) { best = std::min(std::max(l, 1), nl - 2); break; }
        before += cnt[(size_t)l];
      }
    }
    std::vector<int> A, B, Sep;
    for (int v : order) {
      int l = lev_[(size_t)v];
      if (l < best) A.push_back(v);
      else if (l > best) B.push_back(v);
      else Sep.push_back(v);
    }
    for (int v : S) mark_[(size_t)v] = 0;
    std::vector<int> ra, rb;
    dissect(A, ra);
    dissect(B, rb);
    int f = new_front(Sep);
    for (int c : ra) { L_.children[(size_t)f].push_back(c); L_.parent[(size_t)c] = f; }
    for (int c : rb) { L_.children[(size_t)f].push_back(c); L_.parent[(size_t)c] = f; }
    roots.push_back(f);
  }

  const Graph &g_;
  int leaf_;
  Local &L_;
  std::vector<int> mark_, lev_;
  int stamp_ = 0;
};

// Front row structure: pivots, then the later-numbered rows adjacent to the
// front's subtree (the multifrontal update rows).
void finish_local(const Graph &g, Local &L) {
  int n = g.n;
  L.iperm.assign((size_t)n, 0);
  for (int i = 0; i < n; i++) L.iperm[(size_t)L.perm[(size_t)i]] = i;
  int nf = (int)L.p0.size();
  L.rows.assign((size_t)nf, {});
  std::vector<int> stamp((size_t)n, -1);
  for (int f = 0; f < nf; f++) {  // creation order is a post-order
    int p0 = L.p0[(size_t)f], k = L.k[(size_t)f], last = p0 + k - 1;
    std::vector<int> U;
    for (int q = 0; q < k; q++) {
      int v = L.perm[(size_t)(p0 + q)];
      for (int64_t e = g.ptr[(size_t)v]; e < g.ptr[(size_t)v + 1]; e++) {
        int w = L.iperm[(size_t)g.adj[(size_t)e]];
        if (w > last && stamp[(size_t)w] != f) { stamp[(size_t)w] = f; U.push_back(w); }
      }
    }
    int lev = 0;
    for (int c : L.children[(size_t)f]) {
      const std::vector<int> &rc = L.rows[(size_t)c];
      for (size_t q = (size_t)L.k[(size_t)c]; q < rc.size(); q++) {
        int w = rc[q];
        if (w > last && stamp[(size_t)w] != f) { stamp[(size_t)w] = f; U.push_back(w); }
      }
      lev = std::max(lev, L.level[(size_t)c] + 1);
    }
    L.level[(size_t)f] = L.children[(size_t)f].empty() ? 0 : lev;
    std::sort(U.begin(), U.end());
    std::vector<int> &R = L.rows[(size_t)f];
    R.reserve((size_t)k + U.size());
    for (int q = 0; q < k; q++) R.push_back(p0 + q);
    R.insert(R.end(), U.begin(), U.end());
  }
}

Graph graph_of_local(int n, const std::vector<int> &er, const std::vector<int> &ec) {
  Graph g;
  g.n = n;
  std::vector<int64_t> deg((size_t)n + 1, 0);
  for (size_t q = 0; q < er.size(); q++)
    if (er[q] != ec[q]) { deg[(size_t)er[q] + 1]++; deg[(size_t)ec[q] + 1]++; }
  for (int i = 0; i < n; i++) deg[(size_t)i + 1] += deg[(size_t)i];
  g.ptr = deg;
  std::vector<int> adj((size_t)deg[(size_t)n]);
  std::vector<int64_t> fill(deg.begin(), deg.end() - 1);
  for (size_t q = 0; q < er.size(); q++)
    if (er[q] != ec[q]) {
      adj[(size_t)fill[(size_t)er[q]]++] = ec[q];
      adj[(size_t)fill[(size_t)ec[q]]++] = er[q];
    }
  // dedupe
  g.ptr.assign((size_t)n + 1, 0);
  std::vector<int> mark((size_t)n, -1);
  g.adj.clear();
  g.adj.reserve(adj.size());
  for (int i = 0; i < n; i++) {
    for (int64_t e = deg[(size_t)i]; e < deg[(size_t)i + 1]; e++) {
      int w = adj[(size_t)e];
      if (mark[(size_t)w] != i) { mark[(size_t)w] = i; g.adj.push_back(w); }
    }
    g.ptr[(size_t)i + 1] = (int64_t)g.adj.size();
  }
  return g;
}

// Local symbolic analysis for one matrix given its entries (local ids).
void analyse(int n, const std::vector<int> &lr, const std::vector<int> &lc,
             const std::vector<int64_t> &src, int leaf, Local &L) {
  Graph g = graph_of_local(n, lr, lc);
  L = Local();
  L.n = n;
  Dissector d(g, leaf, L);
  d.run();
  finish_local(g, L);
  // keep entries of the lower triangle in the new numbering
  for (size_t q = 0; q < lr.size(); q++) {
    int a = L.iperm[(size_t)lr[q]], b = L.iperm[(size_t)lc[q]];
    if (a >= b) { L.er.push_back(a); L.ec.push_back(b); L.es.push_back(src[q]); }
  }
}

void append(const Local &L, const std::vector<int> &gid_of_local, MfBatch &B) {
  int base_front = B.nfronts;
  int64_t xoff = B.xlen;
  B.xoff.push_back(xoff);
  for (int i = 0; i < L.n; i++) B.gidx.push_back(gid_of_local[(size_t)L.perm[(size_t)i]]);
  B.xlen += L.n;
  int nf = (int)L.p0.size();
  // owner front of each pivot
  std::vector<int> owner((size_t)L.n, -1);
  for (int f = 0; f < nf; f++)
    for (int q = 0; q < L.k[(size_t)f]; q++) owner[(size_t)(L.p0[(size_t)f] + q)] = f;
  std::vector<int64_t> foff((size_t)nf);
  for (int f = 0; f < nf; f++) {
    int m = (int)L.rows[(size_t)f].size(), k = L.k[(size_t)f];
    foff[(size_t)f] = B.arena;
    B.f_off.push_back(B.arena);
    B.arena += ((int64_t)m * m + 3) & ~(int64_t)3;  // 16-byte aligned fronts (cp.async staging)
    B.f_m.push_back(m);
    B.f_k.push_back(k);
    B.f_rows.push_back((int64_t)B.rows.size());
    B.rows.insert(B.rows.end(), L.rows[(size_t)f].begin(), L.rows[(size_t)f].end());
    B.f_xoff.push_back(xoff);
    B.f_p0.push_back(L.p0[(size_t)f]);
    B.f_uoff.push_back(B.ulen);
    B.ulen += m - k;
    B.f_woff.push_back(B.wlen);
    B.wlen += m;
    B.f_parent.push_back(L.parent[(size_t)f] < 0 ? -1 : L.parent[(size_t)f] + base_front);
    B.f_level.push_back(L.level[(size_t)f]);
    B.factor_nnz += (int64_t)m * k - (int64_t)k * (k - 1) / 2;
    double r = m - k;
    B.factor_flops += (double)k * k * k / 3.0 + r * k * k + r * r * k;
    B.max_m = std::max(B.max_m, m);
  }
  for (int f = 0; f < nf; f++) {
    B.f_child_ptr.push_back((int)B.f_children.size());
    for (int c : L.children[(size_t)f]) B.f_children.push_back(c + base_front);
  }
  // relmaps: child update rows -> positions in the parent's row list
  for (int f = 0; f < nf; f++) {
    B.f_relmap.push_back((int64_t)B.relmap.size());
    int p = L.parent[(size_t)f];
    const std::vector<int> &rc = L.rows[(size_t)f];
    int k = L.k[(size_t)f];
    if (p < 0) {
      if ((int)rc.size() != k) throw std::runtime_error("root front with update rows");
      continue;
    }
    const std::vector<int> &rp = L.rows[(size_t)p];
    for (size_t q = (size_t)k; q < rc.size(); q++) {
      auto it = std::lower_bound(rp.begin(), rp.end(), rc[q]);
      if (it == rp.end() || *it != rc[q]) throw std::runtime_error("update row missing in parent");
      B.relmap.push_back((int)(it - rp.begin()));
    }
  }
  // assembly entries, grouped by target (duplicates summed in entry order)
  std::vector<std::pair<int64_t, int64_t>> te;  // (target, source)
  te.reserve(L.er.size());
  for (size_t q = 0; q < L.er.size(); q++) {
    int a = L.er[q], b = L.ec[q];
    int f = owner[(size_t)b];
    const std::vector<int> &R = L.rows[(size_t)f];
    auto it = std::lower_bound(R.begin(), R.end(), a);
    if (it == R.end() || *it != a) throw std::runtime_error("entry row not in its front");
    int64_t row = it - R.begin();
    int64_t col = b - L.p0[(size_t)f];
    int64_t m = (int64_t)R.size();
    te.emplace_back(foff[(size_t)f] + col * m + row, L.es[q]);
  }
  std::stable_sort(te.begin(), te.end(),
                   [](const std::pair<int64_t, int64_t> &x, const std::pair<int64_t, int64_t> &y) {
                     return x.first < y.first;
                   });
  // per-front entry ranges (entries are sorted by target, fronts by offset)
  {
    size_t e = 0;
    int64_t ent = (int64_t)B.asm_tgt.size();
    for (int ff = 0; ff < nf; ff++) {
      B.f_asm.push_back(ent);
      int64_t end = foff[(size_t)ff] + (int64_t)L.rows[(size_t)ff].size() * L.rows[(size_t)ff].size();
      while (e < te.size() && te[e].first < end) {
        int64_t t = te[e].first;
        B.asm_tgt.push_back(t);
        B.asm_sp.push_back((int64_t)B.asm_src.size());
        while (e < te.size() && te[e].first == t) { B.asm_src.push_back(te[e].second); e++; }
        ent++;
      }
    }
  }
  B.nmat++;
  B.nfronts += nf;
}

// Appends batch P (built by append from an empty batch) to B: the result is
// what appending P's matrices to B directly gives (offsets shifted by B's
// sizes; the flop count is summed per piece).
void merge(const MfBatch &P, MfBatch &B) {
  const int base_front = B.nfronts;
  const int64_t arena = B.arena, xlen = B.xlen, ulen = B.ulen, wlen = B.wlen;
  const int64_t nrows = (int64_t)B.rows.size(), nrel = (int64_t)B.relmap.size();
  const int64_t nasm = (int64_t)B.asm_tgt.size(), nsrc = (int64_t)B.asm_src.size();
  const int nchild = (int)B.f_children.size();
  for (int64_t v : P.xoff) B.xoff.push_back(v + xlen);
  B.gidx.insert(B.gidx.end(), P.gidx.begin(), P.gidx.end());
  for (int64_t v : P.f_off) B.f_off.push_back(v + arena);
  B.f_m.insert(B.f_m.end(), P.f_m.begin(), P.f_m.end());
  B.f_k.insert(B.f_k.end(), P.f_k.begin(), P.f_k.end());
  for (int64_t v : P.f_rows) B.f_rows.push_back(v + nrows);
  for (int64_t v : P.f_xoff) B.f_xoff.push_back(v + xlen);
  B.f_p0.insert(B.f_p0.end(), P.f_p0.begin(), P.f_p0.end());
  for (int64_t v : P.f_uoff) B.f_uoff.push_back(v + ulen);
  for (int64_t v : P.f_woff) B.f_woff.push_back(v + wlen);
  for (int v : P.f_child_ptr) B.f_child_ptr.push_back(v + nchild);
  for (int v : P.f_children) B.f_children.push_back(v + base_front);
  for (int64_t v : P.f_relmap) B.f_relmap.push_back(v + nrel);
  for (int64_t v : P.f_asm) B.f_asm.push_back(v + nasm);
  for (int v : P.f_parent) B.f_parent.push_back(v < 0 ? -1 : v + base_front);
  B.f_level.insert(B.f_level.end(), P.f_level.begin(), P.f_level.end());
  B.rows.insert(B.rows.end(), P.rows.begin(), P.rows.end());
  B.relmap.insert(B.relmap.end(), P.relmap.begin(), P.relmap.end());
  for (int64_t v : P.asm_tgt) B.asm_tgt.push_back(v + arena);
  for (int64_t v : P.asm_sp) B.asm_sp.push_back(v + nsrc);
  B.asm_src.insert(B.asm_src.end(), P.asm_src.begin(), P.asm_src.end());
  B.nmat += P.nmat;
  B.nfronts += P.nfronts;
  B.arena += P.arena;
  B.xlen += P.xlen;
  B.ulen += P.ulen;
  B.wlen += P.wlen;
  B.factor_nnz += P.factor_nnz;
  B.factor_flops += P.factor_flops;
  B.max_m = std::max(B.max_m, P.max_m);
}

void finalize(MfBatch &B) {
  B.xoff.push_back(B.xlen);
  B.arena += 16;  // slack: staging copies round the last front up to 16 bytes
  B.f_child_ptr.push_back((int)B.f_children.size());
  B.f_asm.push_back((int64_t)B.asm_tgt.size());
  B.asm_sp.push_back((int64_t)B.asm_src.size());
  int L = 0;
  for (int lv : B.f_level) L = std::max(L, lv + 1);
  B.nlevels = L;
  B.lvl_ptr.assign((size_t)L + 1, 0);
  for (int lv : B.f_level) B.lvl_ptr[(size_t)lv + 1]++;
  for (int l = 0; l < L; l++) B.lvl_ptr[(size_t)l + 1] += B.lvl_ptr[(size_t)l];
  B.lvl_fronts.assign((size_t)B.nfronts, 0);
  std::vector<int> fill(B.lvl_ptr.begin(), B.lvl_ptr.end() - 1);
  for (int f = 0; f < B.nfronts; f++) B.lvl_fronts[(size_t)fill[(size_t)B.f_level[(size_t)f]]++] = f;
  // largest fronts first inside a level, so that long blocks start early
  for (int l = 0; l < L; l++)
    std::stable_sort(B.lvl_fronts.begin() + B.lvl_ptr[(size_t)l], B.lvl_fronts.begin() + B.lvl_ptr[(size_t)l + 1],
                     [&](int a, int b) { return B.f_m[(size_t)a] > B.f_m[(size_t)b]; });
  B.lvl_max_m.assign((size_t)L, 0);
  for (int l = 0; l < L; l++)
    for (int q = B.lvl_ptr[(size_t)l]; q < B.lvl_ptr[(size_t)l + 1]; q++)
      B.lvl_max_m[(size_t)l] = std::max(B.lvl_max_m[(size_t)l], B.f_m[(size_t)B.lvl_fronts[(size_t)q]]);
}

template <class F>
void parallel_for(int n, F fn) {
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
  if (n < 2 || nt < 2) {
    for (int i = 0; i < n; i++) fn(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&] {
      for (;;) {
        int i = next.fetch_add(1);
        if (i >= n) break;
        fn(i);
      }
    });
  for (auto &t : th) t.join();
}

}  // namespace

void mf_build_subdomains(const Csr &A, const std::vector<int64_t> &sd_ptr,
                         const std::vector<int> &sd_nodes, const MfOptions &opt, MfBatch &out) {
  out = MfBatch();
  int nsd = (int)sd_ptr.size() - 1;
  // every subdomain is analysed and laid out as its own batch on a host
  // thread; the pieces are then joined in subdomain order
  std::vector<MfBatch> pieces((size_t)nsd);
  parallel_for(nsd, [&](int s) {
    int64_t b0 = sd_ptr[(size_t)s], m = sd_ptr[(size_t)s + 1] - b0;
    std::vector<int> gid((size_t)m);
    // local position of each global node (sorted lookup keeps memory per subdomain small)
    std::vector<std::pair<int, int>> lut((size_t)m);
    for (int64_t t = 0; t < m; t++) {
      gid[(size_t)t] = sd_nodes[(size_t)(b0 + t)] - 1;
      lut[(size_t)t] = {gid[(size_t)t], (int)t};
    }
    std::sort(lut.begin(), lut.end());
    auto loc = [&](int g) -> int {
      auto it = std::lower_bound(lut.begin(), lut.end(), std::make_pair(g, -1));
      if (it != lut.end() && it->first == g) return it->second;
      return -1;
    };
    std::vector<int> lr, lc;
    std::vector<int64_t> src;
    for (int64_t t = 0; t < m; t++) {
      int g = gid[(size_t)t];
      for (int64_t e = A.ptr[(size_t)g]; e < A.ptr[(size_t)g + 1]; e++) {
        int h = loc(A.col[(size_t)e]);
        if (h >= 0) { lr.push_back((int)t); lc.push_back(h); src.push_back(e); }
      }
    }
    Local L;
    analyse((int)m, lr, lc, src, opt.leaf, L);
    append(L, gid, pieces[(size_t)s]);
  });
  // reserve the batch arrays once (they are large for big subdomains)
  {
    size_t nf = 0, nr = 0, ne = 0, nsrc = 0, nx = 0;
    for (const MfBatch &P : pieces) {
      nf += (size_t)P.nfronts;
      nr += P.rows.size();
      ne += P.asm_tgt.size();
      nsrc += P.asm_src.size();
      nx += P.gidx.size();
    }
    out.f_off.reserve(nf); out.f_m.reserve(nf); out.f_k.reserve(nf); out.f_rows.reserve(nf);
    out.f_xoff.reserve(nf); out.f_p0.reserve(nf); out.f_uoff.reserve(nf); out.f_woff.reserve(nf);
    out.f_parent.reserve(nf); out.f_level.reserve(nf); out.f_relmap.reserve(nf); out.f_asm.reserve(nf + 1);
    out.f_child_ptr.reserve(nf + 1); out.f_children.reserve(nf);
    out.rows.reserve(nr); out.relmap.reserve(nr);
    out.asm_tgt.reserve(ne); out.asm_sp.reserve(ne + 1); out.asm_src.reserve(nsrc);
    out.gidx.reserve(nx);
  }
  for (int s = 0; s < nsd; s++) {
    merge(pieces[(size_t)s], out);
    MfBatch().rows.swap(pieces[(size_t)s].rows);  // release as we go
  }
  finalize(out);
}

void mf_build_single(const Csr &M, const MfOptions &opt, MfBatch &out) {
  out = MfBatch();
  int n = M.nrows;
  std::vector<int> lr, lc, gid((size_t)n);
  std::vector<int64_t> src;
  for (int i = 0; i < n; i++) {
    gid[(size_t)i] = i;
    for (int64_t e = M.ptr[(size_t)i]; e < M.ptr[(size_t)i + 1]; e++) {
      lr.push_back(i); lc.push_back(M.col[(size_t)e]); src.push_back(e);
    }
  }
  Local L;
  analyse(n, lr, lc, src, opt.leaf, L);
  append(L, gid, out);
  finalize(out);
}

}  // namespace dg
