// GB300 solve path: device data, numeric factorisation and the PCG loop,
// behind the C ABI of include/doug_gpu.h.
//
// Layout in HBM (one handle):
//   fine matrix A           CSR (int64 row pointers, int32 columns, FP64 values)
//   PCG vectors             x, r, p, q, z, z_old, b  (FP64, n each)
//   subdomain batch         front arena (T), local vectors xl (T), update and
//                           work vectors (T); T = double (plain) or float (mixed)
//   coarse batch            same structures in FP64 for the coarse matrix
//   transfer                R (nagr x n) and P = R^T (n x nagr) in CSR
//   reductions              kRedBlocks partials per dot product + 8 scalars
// Nothing is allocated after dg_setup; a solve only launches kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/doug_gpu.h"
#include "dg_kernels.cuh"
#include "host/mf_symbolic.hpp"
#include "host/setup.hpp"

namespace dg {

struct CudaError {
  cudaError_t e;
  const char *what;
};
#define CK(call)                                                     \
  do {                                                               \
    cudaError_t _e = (call);                                         \
    if (_e != cudaSuccess) throw CudaError{_e, #call};               \
  } while (0)

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { if (p) cudaFree(p); }
  void alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
  }
  void upload(const std::vector<T> &v) {
    alloc(v.size());
    if (!v.empty()) CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  }
};

static double wall() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// one multifrontal batch on the device, factor precision T
// fronts of at most panel_rows rows whose panel and E fit in kPanelSmem
// bytes are factored by one CTA each; the others by the multi-CTA pipeline
constexpr size_t kPanelSmem = 96 * 1024;
constexpr int kSuperPanel = 128;      // default columns of L per trailing update of a large front
// tunable batch parameters (control words panel_rows, fwd_task_kb, lean_task_kb)
struct MfTune {
  int panel_rows = 512;                  // fronts of at most this many rows may use mf_factor_panel
  int64_t fwd_task_bytes = 96 * 1024;    // E bytes per forward task of a large front
  int64_t lean_task_bytes = 80 * 1024;   // levels with smaller average tasks use 128-thread CTAs
  int small_min_fronts = 1500;           // levels with fewer small fronts solve them CTA-per-task
  int schedule = 0;                      // solves: 0 one launch per level, 1 dependency-driven queue
  int pdl = 0;                           // 1: level launches with programmatic dependent launch
  int factor_overlap = 1;                // 1: a level's one-CTA fronts beside its large-front steps
  int tiny_rows = 64;                    // panel fronts of at most this many rows: tiny_threads per CTA
  int tiny_threads = 64;
  int tensor_update = 1;                 // FP32 super-panel updates: 1 tcgen05 (TMEM), 0 mma.sync
  int super_panel = kSuperPanel;         // columns of L per trailing update of a large front (multiple of 32)
  long long queue_wait_cycles = kQueueWaitCycles;  // solve_schedule 1: limit of one dependency wait
  int queue_skip_publish = -1;           // solve_schedule 1: forward entry whose done flag is withheld (tests)
};

// Launch k with programmatic stream serialisation when pdl is set: its CTAs
// may start while the previous kernel of the stream drains (the kernels call
// pdl_enter before reading anything); otherwise an ordinary launch.
template <typename... P, typename... A>
void launch_level(bool pdl, void (*k)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args) {
  if (!pdl) {
    k<<<grid, block, smem, s>>>(args...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelEx(&cfg, k, args...));
}

template <typename T>
struct MfDevice {
  DBuf<int64_t> f_off, f_rows, f_xoff, f_uoff, f_woff, f_relmap, f_asm, asm_tgt, asm_sp, asm_src, e_off;
  DBuf<ChildEdge> ch_edge;
  DBuf<int> f_m, f_k, f_p0, f_child_ptr, f_children, rows, relmap, lvl_fronts, gidx;
  DBuf<int> pan_fronts, diag_fronts, solve_small;
  int tiny_threads = 64;
  int tensor_update = 1;   // FP32 super-panel updates: 1 tcgen05 + TMEM, 0 mma.sync
  long long q_wait_cycles = kQueueWaitCycles;  // queue schedule: limit of one dependency wait
  int q_skip_publish = -1;  // queue schedule: forward list entry whose done flag is withheld (tests)
  // dependency-driven schedule of the solves (solve_schedule 1)
  bool queue = false;
  bool pdl = false;
  // factor_overlap: a side stream for the one-CTA fronts of a level while
  // the calling stream runs the level's large-front steps (the fronts of a
  // level have disjoint arena regions and their children are finished)
  bool overlap = false;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  MfDevice() = default;
  MfDevice(const MfDevice &) = delete;
  MfDevice &operator=(const MfDevice &) = delete;
  ~MfDevice() {
    if (aux) cudaStreamDestroy(aux);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
  }
  DBuf<int4> qf_tasks, qb_tasks;
  DBuf<int> qf_dep_ptr, qf_dep, qb_dep_ptr, qb_dep, q_small_off, q_counter, q_done;
  DBuf<SmallBuckets> q_sb;
  int qf_n = 0, qb_n = 0, q_grid = 0, q_k = 0;
  size_t q_smem = 0;
  DBuf<int2> asm_tasks, upd_tasks, panel_tasks, esc_tasks, etile_tasks, fwd_tasks, bwd_tasks;
  DBuf<TaskFront> fwd_tmeta, bwd_tmeta;  // each solve task's front (m, k, E offset)
  DBuf<T> arena, E, xl, yl, u;
  int64_t e_len = 0;
  // per level: small-front range, assembly-task range, steps
  // a panel step (diag, panel + E rows, update inside the super-panel + E
  // update; kw = kNB) or a super-panel's trailing update (kw = kSuperPanel,
  // no diag / panel); cend_base > 0 limits the update to columns < cend_base
  struct Step {
    int j0, diag_off, diag_cnt, panel_off, panel_cnt, esc_off, esc_cnt;
    int upd_off, upd_cnt, etile_off, etile_cnt;
    int kw, cend_base;
    bool big;                     // trailing update in 128 x 128 tiles (FP32)
  };
  struct Level {
    int pan_off, pan_cnt, asm_off, asm_cnt, pan_maxm;
    int tiny_off, tiny_cnt;        // panel fronts of at most tune.tiny_rows rows: narrow CTAs
    size_t tiny_smem;
    size_t pan_smem;
    std::vector<Step> steps;
  };
  std::vector<Level> levels;
  // per level: solve work lists
  struct SolveLevel {
    int small_off, small_cta;     // small fronts of the level (three buckets)
    SmallBuckets sb;
    int fwd_off, fwd_cnt, bwd_off, bwd_cnt;
    size_t fwd_smem, bwd_smem;
    bool fwd_lean, bwd_lean;      // 128-thread CTAs for levels of small tasks
  };
  std::vector<SolveLevel> slevels;
  int nlevels = 0, nfronts = 0;
  int64_t xlen = 0;
  MfView view{};

  void upload(const MfBatch &B, const MfTune &tune) {
    f_off.upload(B.f_off); f_rows.upload(B.f_rows); f_xoff.upload(B.f_xoff);
    f_uoff.upload(B.f_uoff); f_woff.upload(B.f_woff); f_relmap.upload(B.f_relmap);
    f_asm.upload(B.f_asm); asm_tgt.upload(B.asm_tgt); asm_sp.upload(B.asm_sp);
    asm_src.upload(B.asm_src);
    f_m.upload(B.f_m); f_k.upload(B.f_k); f_p0.upload(B.f_p0);
    f_child_ptr.upload(B.f_child_ptr); f_children.upload(B.f_children);
    {
      std::vector<ChildEdge> ce(B.f_children.size());
      for (size_t ci = 0; ci < B.f_children.size(); ci++) {
        const int c = B.f_children[ci];
        ce[ci] = ChildEdge{B.f_relmap[(size_t)c], B.f_uoff[(size_t)c], B.f_m[(size_t)c] - B.f_k[(size_t)c], 0};
      }
      ch_edge.upload(ce);
    }
    rows.upload(B.rows); relmap.upload(B.relmap); lvl_fronts.upload(B.lvl_fronts);
    gidx.upload(B.gidx);
    nlevels = B.nlevels;
    nfronts = B.nfronts;
    xlen = B.xlen;
    // elimination matrices: m x k per front, ld = round4(m); the padding rows
    // are zero once and never written again
    std::vector<int64_t> eo((size_t)nfronts);
    e_len = 0;
    for (int f = 0; f < nfronts; f++) {
      eo[(size_t)f] = e_len;
      e_len += (int64_t)round4(B.f_m[(size_t)f]) * B.f_k[(size_t)f];
    }
    e_off.upload(eo);
    E.alloc((size_t)std::max<int64_t>(e_len, 4));
    CK(cudaMemset(E.p, 0, (size_t)std::max<int64_t>(e_len, 4) * sizeof(T)));
    arena.alloc((size_t)B.arena);
    xl.alloc((size_t)B.xlen);
    yl.alloc((size_t)B.xlen);
    u.alloc((size_t)std::max<int64_t>(B.ulen, 1));
    ulen = B.ulen;
    mk = 0;
    view = MfView{f_off.p, f_m.p, f_k.p, f_rows.p, f_xoff.p, f_p0.p, f_uoff.p, f_woff.p,
                  f_child_ptr.p, f_children.p, f_relmap.p, f_asm.p, rows.p, relmap.p,
                  asm_tgt.p, asm_sp.p, asm_src.p, e_off.p, ch_edge.p};
    int dev = 0, optin = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // work lists of the factorisation
    std::vector<int> pn, df;
    std::vector<int2> at, ut, pf, es, et;
    levels.assign((size_t)nlevels, Level());
    for (int l = 0; l < nlevels; l++) {
      Level &L = levels[(size_t)l];
      L.pan_smem = 0;
      L.pan_maxm = 0;
      L.tiny_smem = 0;
      L.asm_off = (int)at.size();
      std::vector<int> large, tiny, pan;
      for (int q = B.lvl_ptr[(size_t)l]; q < B.lvl_ptr[(size_t)l + 1]; q++) {
        int f = B.lvl_fronts[(size_t)q];
        int m = B.f_m[(size_t)f], k = B.f_k[(size_t)f];
        const size_t smem = pan_smem<T>(m, k);
        if (m <= tune.tiny_rows) {
          tiny.push_back(f);
          L.tiny_smem = std::max(L.tiny_smem, smem);
        } else if (m <= tune.panel_rows && smem <= kPanelSmem) {
          pan.push_back(f);
          L.pan_smem = std::max(L.pan_smem, smem);
          L.pan_maxm = std::max(L.pan_maxm, m);
        } else {
          large.push_back(f);
        }
      }
      L.tiny_off = (int)pn.size();
      pn.insert(pn.end(), tiny.begin(), tiny.end());
      L.tiny_cnt = (int)tiny.size();
      L.pan_off = (int)pn.size();
      pn.insert(pn.end(), pan.begin(), pan.end());
      L.pan_cnt = (int)pan.size();
      int kmax = 0;
      for (int f : large) {
        int m = B.f_m[(size_t)f];
        for (int c0 = 0; c0 < m; c0 += kAsmCols) at.push_back(make_int2(f, c0));
        kmax = std::max(kmax, B.f_k[(size_t)f]);
      }
      L.asm_cnt = (int)at.size() - L.asm_off;
      // right-looking by super-panels of kSuperPanel columns: each 32-column
      // panel updates only the rest of its super-panel; the trailing matrix
      // receives one update with up to kSuperPanel columns of L per super-panel
      const int SP = tune.super_panel;
      for (int S0 = 0; S0 < kmax; S0 += SP) {
        for (int j0 = S0; j0 < std::min(S0 + SP, kmax); j0 += kNB) {
          Step st{j0, (int)df.size(), 0, (int)pf.size(), 0, (int)es.size(), 0,
                  (int)ut.size(), 0, (int)et.size(), 0, kNB, S0 + SP, false};
          for (int f : large) {
            int m = B.f_m[(size_t)f], k = B.f_k[(size_t)f];
            if (j0 >= k) continue;
            // the diagonal block is factored by the kernel that finishes it,
            // except after the mma.sync trailing update (tensor_update 0)
            if (j0 > 0 && j0 == S0 && sizeof(T) == 4 && tune.tensor_update != 1) df.push_back(f);
            const int c0 = j0 + std::min(kNB, k - j0);
            for (int r0 = c0; r0 < m; r0 += kPanelRows) pf.push_back(make_int2(f, r0));
            for (int e0 = 0; e0 < c0; e0 += EscCols<T>::N) es.push_back(make_int2(f, e0));
            const int nt = (m - c0 + kTile - 1) / kTile;
            const int cend = std::min(S0 + SP, k);
            const int ntc = cend > c0 ? (cend - c0 + kTile - 1) / kTile : 0;
            for (int tj = 0; tj < ntc; tj++)
              for (int ti = tj; ti < nt; ti++) ut.push_back(make_int2(f, (ti << 16) | tj));
            // E rows of the rest of the super-panel only (rows below cend
            // receive the super-panel's update at once, planned below)
            const int nte = (c0 + kTile - 1) / kTile;
            const int ntr = cend > c0 ? (cend - c0 + kTile - 1) / kTile : 0;
            for (int ti = 0; ti < ntr; ti++)
              for (int tc = 0; tc < nte; tc++) et.push_back(make_int2(f, (ti << 16) | tc));
          }
          st.diag_cnt = (int)df.size() - st.diag_off;
          st.panel_cnt = (int)pf.size() - st.panel_off;
          st.esc_cnt = (int)es.size() - st.esc_off;
          st.upd_cnt = (int)ut.size() - st.upd_off;
          st.etile_cnt = (int)et.size() - st.etile_off;
          L.steps.push_back(st);
        }
        const bool bigt = sizeof(T) == 4;  // FP32: 128 x 128 tiles; FP64 keeps 64 x 64 (FP64-pipe bound)
        const int tile = bigt ? kBT : kTile;
        Step st{S0, (int)df.size(), 0, (int)pf.size(), 0, (int)es.size(), 0,
                (int)ut.size(), 0, (int)et.size(), 0, SP, 0, bigt};
        for (int f : large) {
          int m = B.f_m[(size_t)f], k = B.f_k[(size_t)f];
          if (S0 >= k) continue;
          const int c1 = S0 + std::min(SP, k - S0);
          const int nt = (m - c1 + tile - 1) / tile;
          for (int tj = 0; tj < nt; tj++)
            for (int ti = tj; ti < nt; ti++) ut.push_back(make_int2(f, (ti << 16) | tj));
          // E rows below the super-panel, all its columns at once:
          // E[c1:m, 0:c1] -= L[c1:m, S0:c1] E[S0:c1, 0:c1] (FP32 with tcgen05:
          // 128 x 128 tiles in the trailing update's launch; else 64 x 64
          // tiles of mf_update)
          const int etw = bigt && tune.tensor_update == 1 ? kBT : kTile;
          const int nte = (c1 + etw - 1) / etw, ntr = (m - c1 + etw - 1) / etw;
          for (int ti = 0; ti < ntr; ti++)
            for (int tc = 0; tc < nte; tc++) et.push_back(make_int2(f, (ti << 16) | tc));
        }
        st.upd_cnt = (int)ut.size() - st.upd_off;
        st.etile_cnt = (int)et.size() - st.etile_off;
        if (st.upd_cnt || st.etile_cnt) L.steps.push_back(st);
      }
    }
    pan_fronts.upload(pn);
    // kernel attributes are per function, shared by every batch of this
    // precision: always the device maximum, never a batch's own size
    CK(cudaFuncSetAttribute(mf_factor_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 1024));
    panel_tasks.upload(pf);
    esc_tasks.upload(es);
    diag_fronts.upload(df);
    asm_tasks.upload(at);
    upd_tasks.upload(ut);
    etile_tasks.upload(et);
    // solve work lists: warp kernels for the small fronts; one task per 32-row
    // block (forward) and per 32-column block (backward) of the others, the
    // longest first
    std::vector<int> ss;
    std::vector<int2> fw, bw;
    std::vector<TaskFront> fwm, bwm;
    size_t fwd_smem_max = 0, bwd_smem_max = 0;
    slevels.assign((size_t)nlevels, SolveLevel());
    for (int l = 0; l < nlevels; l++) {
      SolveLevel &L = slevels[(size_t)l];
      std::vector<std::pair<int, int>> sm[3];  // (k, front) per bucket
      L.fwd_off = (int)fw.size();
      L.bwd_off = (int)bw.size();
      L.fwd_smem = L.bwd_smem = 0;
      std::vector<std::pair<int, int2>> fl, bl;
      int64_t fwd_bytes = 0, bwd_bytes = 0;
      // a level with few small fronts solves them with the CTA-per-task
      // kernels too: a group of lanes per front leaves the GPU nearly idle
      // while it walks the columns of a large-k front
      int nsmall = 0;
      for (int q = B.lvl_ptr[(size_t)l]; q < B.lvl_ptr[(size_t)l + 1]; q++)
        nsmall += B.f_m[(size_t)B.lvl_fronts[(size_t)q]] <= kSolveSmall;
      const bool thin = nsmall < tune.small_min_fronts;
      for (int q = B.lvl_ptr[(size_t)l]; q < B.lvl_ptr[(size_t)l + 1]; q++) {
        int f = B.lvl_fronts[(size_t)q];
        int m = B.f_m[(size_t)f], k = B.f_k[(size_t)f];
        if (m <= kSolveSmall && !thin) { sm[m <= 32 ? 0 : m <= 64 ? 1 : 2].push_back({k, f}); continue; }
        // forward tasks: runs of row chunks of at least tune.fwd_task_bytes of E each
        const int RC = FwdRows<T>::N, nch = (m + RC - 1) / RC;
        for (int c = 0; c < nch;) {
          int c1 = c;
          int64_t bytes = 0;
          do {
            const int r0 = c1 * RC, K = r0 < k ? std::min(k, r0 + RC) : k;
            bytes += (int64_t)RC * K * (int64_t)sizeof(T);
            c1++;
          } while (c1 < nch && bytes < tune.fwd_task_bytes);
          fl.push_back({(int)std::min<int64_t>(bytes, 1 << 30), make_int2(f, (c << 16) | (c1 - c))});
          fwd_bytes += bytes;
          c = c1;
        }
        for (int J = 0; 32 * J < k; J++) {
          bl.push_back({m - 32 * J, make_int2(f, J)});
          bwd_bytes += (int64_t)32 * (m - 32 * J) * (int64_t)sizeof(T);
        }
        L.fwd_smem = std::max(L.fwd_smem, (size_t)round4(m) * sizeof(T));
        L.bwd_smem = std::max(L.bwd_smem, (size_t)round4(m) * sizeof(T));
      }
      std::stable_sort(fl.begin(), fl.end(), [](const std::pair<int, int2> &a, const std::pair<int, int2> &b) { return a.first > b.first; });
      std::stable_sort(bl.begin(), bl.end(), [](const std::pair<int, int2> &a, const std::pair<int, int2> &b) { return a.first > b.first; });
      for (auto &e : fl) fw.push_back(e.second);
      for (auto &e : bl) bw.push_back(e.second);
      for (auto &e : fl) {
        const int f = e.second.x;
        fwm.push_back(TaskFront{B.f_m[(size_t)f], B.f_k[(size_t)f], eo[(size_t)f]});
      }
      for (auto &e : bl) {
        const int f = e.second.x;
        bwm.push_back(TaskFront{B.f_m[(size_t)f], B.f_k[(size_t)f], eo[(size_t)f]});
      }
      // fronts of similar pivot counts share a warp
      L.small_off = (int)ss.size();
      int cnt[3];
      for (int bk = 0; bk < 3; bk++) {
        std::stable_sort(sm[bk].begin(), sm[bk].end(),
                         [](const std::pair<int, int> &a, const std::pair<int, int> &b) { return a.first > b.first; });
        for (auto &e : sm[bk]) ss.push_back(e.second);
        cnt[bk] = (int)sm[bk].size();
      }
      // 256-thread CTAs: 32 fronts of bucket 0, 16 of bucket 1, 8 of bucket 2
      L.sb = SmallBuckets{cnt[0], cnt[1], cnt[2], (cnt[0] + 31) / 32, (cnt[1] + 15) / 16};
      L.small_cta = L.sb.nb0 + L.sb.nb1 + (cnt[2] + 7) / 8;
      L.fwd_cnt = (int)fw.size() - L.fwd_off;
      L.bwd_cnt = (int)bw.size() - L.bwd_off;
      L.fwd_lean = L.fwd_cnt && fwd_bytes / L.fwd_cnt < tune.lean_task_bytes;
      L.bwd_lean = L.bwd_cnt && bwd_bytes / L.bwd_cnt < tune.lean_task_bytes;
      fwd_smem_max = std::max(fwd_smem_max, L.fwd_smem);
      bwd_smem_max = std::max(bwd_smem_max, L.bwd_smem);
    }
    solve_small.upload(ss);
    fwd_tasks.upload(fw);
    bwd_tasks.upload(bw);
    fwd_tmeta.upload(fwm);
    bwd_tmeta.upload(bwm);
    set_solve_attrs<kEThreads>(optin, fwd_smem_max, bwd_smem_max);
    set_solve_attrs<kELeanThreads>(optin, fwd_smem_max, bwd_smem_max);
    queue = tune.schedule == 1;
    pdl = tune.pdl == 1;
    overlap = tune.factor_overlap == 1;
    tiny_threads = tune.tiny_threads;
    tensor_update = tune.tensor_update;
    q_wait_cycles = tune.queue_wait_cycles;
    q_skip_publish = tune.queue_skip_publish;
    if constexpr (sizeof(T) == 4)
      if (tensor_update == 1)
        CK(cudaFuncSetAttribute(mf_update_big_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    if (queue) plan_queue(B, ss, fw, bw, fwd_smem_max, bwd_smem_max);
  }

  template <int NT>
  void set_solve_attrs(int optin, size_t fwd_smem_max, size_t bwd_smem_max) {
    cudaFuncAttributes fa{}, fb{};
    CK(cudaFuncGetAttributes(&fa, mf_fwd_big<T, NT>));
    CK(cudaFuncGetAttributes(&fb, mf_bwd_big<T, NT>));
    if (fwd_smem_max + fa.sharedSizeBytes > (size_t)optin || bwd_smem_max + fb.sharedSizeBytes > (size_t)optin)
      throw CudaError{cudaErrorInvalidValue, "front too large for the shared-memory solve"};
    CK(cudaFuncSetAttribute(mf_fwd_big<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            optin - (int)fa.sharedSizeBytes));
    CK(cudaFuncSetAttribute(mf_bwd_big<T, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            optin - (int)fb.sharedSizeBytes));
  }

  int factor(const double *vals, int *status, cudaStream_t s) {
    int launches = 0;
    if (overlap && !aux) {  // the side stream takes the calling stream's priority
      int prio = 0;
      CK(cudaStreamGetPriority(s, &prio));
      CK(cudaStreamCreateWithPriority(&aux, cudaStreamNonBlocking, prio));
      CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
    for (int l = 0; l < nlevels; l++) {
      const Level &L = levels[(size_t)l];
      // the one-CTA fronts on the side stream when the level also has large
      // fronts, joined before the next level
      const bool fork = overlap && (L.tiny_cnt || L.pan_cnt) && (L.asm_cnt || !L.steps.empty());
      cudaStream_t sp = s;
      if (fork) {
        CK(cudaEventRecord(ev_fork, s));
        CK(cudaStreamWaitEvent(aux, ev_fork, 0));
        sp = aux;
      }
      if (L.tiny_cnt) {  // small fronts: narrow CTAs, more of them per SM
        mf_factor_panel<T><<<L.tiny_cnt, tiny_threads, L.tiny_smem, sp>>>(view, pan_fronts.p + L.tiny_off, vals,
                                                                          arena.p, E.p, status);
        launches++;
      }
      if (L.pan_cnt) {
        mf_factor_panel<T><<<L.pan_cnt, L.pan_maxm > kPanWideRows ? kPanThreadsWide : kPanThreads, L.pan_smem, sp>>>(
            view, pan_fronts.p + L.pan_off, vals, arena.p, E.p, status);
        launches++;
      }
      if (fork) CK(cudaEventRecord(ev_join, aux));
      if (L.asm_cnt) {
        mf_assemble_large<T><<<L.asm_cnt, kMfThreads, 0, s>>>(view, asm_tasks.p + L.asm_off, vals, arena.p,
                                                              status);
        launches++;
      }
      for (const Step &st : L.steps) {
        if (st.diag_cnt) {
          mf_diag<T><<<st.diag_cnt, diag_threads<T>(), 0, s>>>(view, diag_fronts.p + st.diag_off, st.j0, arena.p,
                                                                status);
          launches++;
        }
        if (st.panel_cnt + st.esc_cnt) {
          mf_panel<T><<<st.panel_cnt + st.esc_cnt, kMfThreads, 0, s>>>(
              view, panel_tasks.p + st.panel_off, st.panel_cnt, esc_tasks.p + st.esc_off, st.j0, arena.p, E.p);
          launches++;
        }
        if (st.big) {
          if constexpr (sizeof(T) == 4) {  // planned for FP32 batches only
            if (tensor_update == 1) {  // trailing-update tiles, then the super-panel's E tiles
              if (st.upd_cnt + st.etile_cnt) {
                mf_update_big_tc<<<st.upd_cnt + st.etile_cnt, 256, kTcSmem, s>>>(
                    view, upd_tasks.p + st.upd_off, st.upd_cnt, etile_tasks.p + st.etile_off, st.j0, st.kw,
                    reinterpret_cast<float *>(arena.p), reinterpret_cast<float *>(E.p), status, 1);
                launches++;
              }
            } else if (st.upd_cnt) {
              mf_update_big_tf32<<<st.upd_cnt, 256, 0, s>>>(view, upd_tasks.p + st.upd_off, st.j0, st.kw,
                                                            reinterpret_cast<float *>(arena.p));
              launches++;
            }
            if (tensor_update != 1 && st.etile_cnt) {  // the super-panel's E update
              mf_update<T><<<st.etile_cnt, kMfThreads, 0, s>>>(view, upd_tasks.p + st.upd_off, 0,
                                                               etile_tasks.p + st.etile_off, st.j0, st.kw, 0,
                                                               arena.p, E.p, status);
              launches++;
            }
          }
        } else if (st.upd_cnt + st.etile_cnt) {
          mf_update<T><<<st.upd_cnt + st.etile_cnt, kMfThreads, 0, s>>>(
              view, upd_tasks.p + st.upd_off, st.upd_cnt, etile_tasks.p + st.etile_off, st.j0, st.kw,
              st.cend_base, arena.p, E.p, status);
          launches++;
        }
      }
      if (fork) CK(cudaStreamWaitEvent(s, ev_join, 0));
    }
    return launches;
  }

  // The task lists of the dependency-driven solves: the level plan's tasks in
  // level order (forward leaves first, backward roots first; per level the
  // large-front tasks, then the small-front CTAs), and for every task the
  // tasks producing its inputs (forward: all tasks of the children of its
  // fronts; backward: all tasks of their parents).
  void plan_queue(const MfBatch &B, const std::vector<int> &ss, const std::vector<int2> &fw,
                  const std::vector<int2> &bw, size_t fwd_smem_max, size_t bwd_smem_max) {
    const int nf = B.nfronts;
    std::vector<int4> qt[2];
    std::vector<std::vector<int>> prod[2];   // per front: its tasks
    std::vector<std::vector<int>> cover[2];  // per task: its fronts
    for (int dir = 0; dir < 2; dir++) {
      prod[dir].assign((size_t)nf, {});
      for (int li = 0; li < nlevels; li++) {
        const int l = dir == 0 ? li : nlevels - 1 - li;
        const SolveLevel &L = slevels[(size_t)l];
        const int boff = dir == 0 ? L.fwd_off : L.bwd_off, bcnt = dir == 0 ? L.fwd_cnt : L.bwd_cnt;
        for (int i = boff; i < boff + bcnt; i++) {
          const int f = dir == 0 ? fw[(size_t)i].x : bw[(size_t)i].x;
          prod[dir][(size_t)f].push_back((int)qt[dir].size());
          cover[dir].push_back({f});
          qt[dir].push_back(make_int4(1, l, i, 0));
        }
        const SmallBuckets &sb = L.sb;
        for (int c = 0; c < L.small_cta; c++) {
          std::vector<int> fr;
          int first, cnt, per;
          if (c < sb.nb0) { first = c * 32; cnt = sb.cnt0; per = 32; }
          else if (c < sb.nb0 + sb.nb1) { first = sb.cnt0 + (c - sb.nb0) * 16; cnt = sb.cnt0 + sb.cnt1; per = 16; }
          else { first = sb.cnt0 + sb.cnt1 + (c - sb.nb0 - sb.nb1) * 8; cnt = sb.cnt0 + sb.cnt1 + sb.cnt2; per = 8; }
          for (int q = first; q < std::min(first + per, cnt); q++) {
            const int f = ss[(size_t)(L.small_off + q)];
            fr.push_back(f);
            prod[dir][(size_t)f].push_back((int)qt[dir].size());
          }
          cover[dir].push_back(fr);
          qt[dir].push_back(make_int4(0, l, c, 0));
        }
      }
    }
    std::vector<int> dptr[2], dep[2];
    for (int dir = 0; dir < 2; dir++) {
      dptr[dir].assign(1, 0);
      std::vector<int> d;
      for (size_t t = 0; t < qt[dir].size(); t++) {
        d.clear();
        for (int f : cover[dir][t]) {
          if (dir == 0) {
            for (int ci = B.f_child_ptr[(size_t)f]; ci < B.f_child_ptr[(size_t)f + 1]; ci++)
              for (int u : prod[0][(size_t)B.f_children[(size_t)ci]]) d.push_back(u);
          } else if (B.f_parent[(size_t)f] >= 0) {
            for (int u : prod[1][(size_t)B.f_parent[(size_t)f]]) d.push_back(u);
          }
        }
        std::sort(d.begin(), d.end());
        d.erase(std::unique(d.begin(), d.end()), d.end());
        for (int u : d)
          if (u >= (int)t) throw CudaError{cudaErrorInvalidValue, "solve queue: a dependency does not come first"};
        dep[dir].insert(dep[dir].end(), d.begin(), d.end());
        dptr[dir].push_back((int)dep[dir].size());
      }
    }
    qf_tasks.upload(qt[0]); qb_tasks.upload(qt[1]);
    qf_dep_ptr.upload(dptr[0]); qf_dep.upload(dep[0]);
    qb_dep_ptr.upload(dptr[1]); qb_dep.upload(dep[1]);
    qf_n = (int)qt[0].size();
    qb_n = (int)qt[1].size();
    std::vector<int> so((size_t)nlevels);
    std::vector<SmallBuckets> sbv((size_t)nlevels);
    for (int l = 0; l < nlevels; l++) { so[(size_t)l] = slevels[(size_t)l].small_off; sbv[(size_t)l] = slevels[(size_t)l].sb; }
    q_small_off.upload(so);
    q_sb.upload(sbv);
    q_counter.alloc(2);
    q_smem = std::max({(size_t)8 * kSolveSmall * sizeof(T), fwd_smem_max, bwd_smem_max});
    CK(cudaFuncSetAttribute(mf_fwd_queue<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)q_smem));
    CK(cudaFuncSetAttribute(mf_bwd_queue<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)q_smem));
    int dev = 0, nsm = 0, occ_f = 0, occ_b = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, mf_fwd_queue<T>, 256, q_smem));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, mf_bwd_queue<T>, 256, q_smem));
    q_grid = nsm * std::max(1, std::min(occ_f, occ_b));
    q_done.alloc((size_t)(qf_n + qb_n));  // one right-hand side; ensure_multi grows it
    q_k = 1;
  }

  // several right-hand sides: local vectors k at k*xlen (xlm, ylm) and k*ulen (um)
  DBuf<T> xlm, ylm, um;
  int mk = 0;
  int64_t ulen = 0;
  void ensure_multi(int K) {
    if (mk == K) return;
    if (queue && q_k < K) {
      q_done.alloc((size_t)(qf_n + qb_n) * K);
      q_k = K;
    }
    xlm.alloc((size_t)xlen * K);
    ylm.alloc((size_t)xlen * K);
    um.alloc((size_t)std::max<int64_t>(ulen, 1) * K);
    mk = K;
  }

  // forward + backward solve: right-hand side in xl, solution back in xl
  // (nrhs > 1: the nrhs right-hand sides in xlm, solutions back in xlm)
  int solve(cudaStream_t s, int nrhs = 1, int *status = nullptr) {
    int launches = 0;
    T *xl_ = nrhs > 1 ? xlm.p : xl.p, *yl_ = nrhs > 1 ? ylm.p : yl.p, *u_ = nrhs > 1 ? um.p : u.p;
    const int64_t xs = nrhs > 1 ? xlen : 0, us = nrhs > 1 ? std::max<int64_t>(ulen, 1) : 0;
    if (queue && status && q_k >= nrhs) {
      CK(cudaMemsetAsync(q_counter.p, 0, 2 * sizeof(int), s));
      CK(cudaMemsetAsync(q_done.p, 0, (size_t)(qf_n + qb_n) * nrhs * sizeof(int), s));
      mf_fwd_queue<T><<<q_grid, 256, q_smem, s>>>(view, QueueView{qf_tasks.p, qf_dep_ptr.p, qf_dep.p, qf_n,
                                                                   q_wait_cycles, q_skip_publish},
                                                  solve_small.p, q_small_off.p, q_sb.p, fwd_tasks.p, fwd_tmeta.p, E.p,
                                                  xl_, yl_,
                                                  u_, q_counter.p, q_done.p, status, nrhs, xs, us);
      mf_bwd_queue<T><<<q_grid, 256, q_smem, s>>>(view, QueueView{qb_tasks.p, qb_dep_ptr.p, qb_dep.p, qb_n,
                                                                   q_wait_cycles, -1},
                                                  solve_small.p, q_small_off.p, q_sb.p, bwd_tasks.p, bwd_tmeta.p, E.p,
                                                  yl_, xl_,
                                                  q_counter.p + 1, q_done.p + (size_t)qf_n * nrhs, status, nrhs, xs);
      return 2;
    }
    for (int l = 0; l < nlevels; l++) {
      const SolveLevel &L = slevels[(size_t)l];
      if (L.small_cta) {
        launch_level(pdl, mf_fwd_small<T>, L.small_cta * nrhs, 256, 0, s, view,
                     (const int *)(solve_small.p + L.small_off), L.sb, (const T *)E.p, (const T *)xl_, yl_, u_, nrhs,
                     xs, us);
        launches++;
      }
      if (L.fwd_cnt) {
        launch_level(pdl, L.fwd_lean ? mf_fwd_big<T, kELeanThreads> : mf_fwd_big<T, kEThreads>, L.fwd_cnt * nrhs,
                     L.fwd_lean ? kELeanThreads : kEThreads, L.fwd_smem, s, view,
                     (const int2 *)(fwd_tasks.p + L.fwd_off), (const TaskFront *)(fwd_tmeta.p + L.fwd_off),
                     (const T *)E.p, (const T *)xl_, yl_, u_, nrhs, xs, us);
        launches++;
      }
    }
    for (int l = nlevels - 1; l >= 0; l--) {
      const SolveLevel &L = slevels[(size_t)l];
      if (L.bwd_cnt) {
        launch_level(pdl, L.bwd_lean ? mf_bwd_big<T, kELeanThreads> : mf_bwd_big<T, kEThreads>, L.bwd_cnt * nrhs,
                     L.bwd_lean ? kELeanThreads : kEThreads, L.bwd_smem, s, view,
                     (const int2 *)(bwd_tasks.p + L.bwd_off), (const TaskFront *)(bwd_tmeta.p + L.bwd_off),
                     (const T *)E.p, (const T *)yl_, xl_, nrhs, xs);
        launches++;
      }
      if (L.small_cta) {
        launch_level(pdl, mf_bwd_small<T>, L.small_cta * nrhs, 256, 0, s, view,
                     (const int *)(solve_small.p + L.small_off), L.sb, (const T *)E.p, (const T *)yl_, xl_, nrhs, xs);
        launches++;
      }
    }
    return launches;
  }
};

}  // namespace dg

using namespace dg;

// symmetric Gauss-Seidel subdomain data (fine_method 2): the arena holds
// every subdomain's rows in increasing global order; rows of a subdomain are
// grouped into dependency levels for the forward and the backward sweep
struct SgsDevice {
  DBuf<int64_t> rp, sd_ptr;
  DBuf<int> ci, gidx, sd_lev_f, sd_lev_b, lev_f, lev_b, rows_f, rows_b;
  DBuf<double> va, dg, x;
  int nsd = 0;
  std::vector<int> gidx_h;
  SgsView view{};

  // levels of one sweep over the rows [q0, q1) of a subdomain (local CSR),
  // in increasing (fwd) or decreasing order: a row comes after every row it
  // shares an entry with (either direction) that precedes it in the sweep
  static void levels(const std::vector<int64_t> &rp, const std::vector<int> &ci, int q0, int q1, bool fwd,
                     std::vector<int> &lev, std::vector<int> &minlev) {
    for (int q = q0; q < q1; q++) minlev[(size_t)q] = 0;
    for (int t = 0; t < q1 - q0; t++) {
      const int q = fwd ? q0 + t : q1 - 1 - t;
      int L = minlev[(size_t)q];
      for (int64_t e = rp[(size_t)q]; e < rp[(size_t)q + 1]; e++) {
        const int c = ci[(size_t)e];
        if (c != q && (fwd ? c < q : c > q)) L = std::max(L, lev[(size_t)c] + 1);
      }
      lev[(size_t)q] = L;
      for (int64_t e = rp[(size_t)q]; e < rp[(size_t)q + 1]; e++) {
        const int c = ci[(size_t)e];
        if (c != q && (fwd ? c > q : c < q)) minlev[(size_t)c] = std::max(minlev[(size_t)c], L + 1);
      }
    }
  }

  void build(const Csr &A, const std::vector<int64_t> &sdp, const std::vector<int> &sd_nodes) {
    nsd = (int)sdp.size() - 1;
    const int64_t len = sdp.back();
    gidx_h.assign((size_t)len, 0);
    for (int s = 0; s < nsd; s++) {
      std::vector<int> nodes(sd_nodes.begin() + sdp[(size_t)s], sd_nodes.begin() + sdp[(size_t)s + 1]);
      std::sort(nodes.begin(), nodes.end());
      for (size_t t = 0; t < nodes.size(); t++) gidx_h[(size_t)sdp[(size_t)s] + t] = nodes[t] - 1;
    }
    std::vector<int> loc((size_t)A.nrows, -1);
    std::vector<int64_t> rph((size_t)len + 1, 0);
    std::vector<int> cih;
    std::vector<double> vah, dgh((size_t)len, 0.0);
    for (int s = 0; s < nsd; s++) {
      for (int64_t q = sdp[(size_t)s]; q < sdp[(size_t)s + 1]; q++) loc[(size_t)gidx_h[(size_t)q]] = (int)q;
      for (int64_t q = sdp[(size_t)s]; q < sdp[(size_t)s + 1]; q++) {
        const int g = gidx_h[(size_t)q];
        for (int64_t e = A.ptr[(size_t)g]; e < A.ptr[(size_t)g + 1]; e++) {
          const int c = A.col[(size_t)e];
          if (loc[(size_t)c] < 0) continue;
          cih.push_back(loc[(size_t)c]);
          vah.push_back(A.val[(size_t)e]);
          if (c == g) dgh[(size_t)q] = A.val[(size_t)e];
        }
        rph[(size_t)q + 1] = (int64_t)cih.size();
      }
      for (int64_t q = sdp[(size_t)s]; q < sdp[(size_t)s + 1]; q++) loc[(size_t)gidx_h[(size_t)q]] = -1;
    }
    std::vector<int> lf((size_t)len), lb((size_t)len), ml((size_t)len);
    std::vector<int> sdlf(1, 0), sdlb(1, 0), levf(1, 0), levb(1, 0), rowf, rowb;
    for (int s = 0; s < nsd; s++) {
      const int q0 = (int)sdp[(size_t)s], q1 = (int)sdp[(size_t)s + 1];
      levels(rph, cih, q0, q1, true, lf, ml);
      levels(rph, cih, q0, q1, false, lb, ml);
      for (int dir = 0; dir < 2; dir++) {
        const std::vector<int> &lv = dir == 0 ? lf : lb;
        std::vector<int> &rows = dir == 0 ? rowf : rowb;
        std::vector<int> &lev = dir == 0 ? levf : levb;
        std::vector<int> &sdl = dir == 0 ? sdlf : sdlb;
        int nl = 0;
        for (int q = q0; q < q1; q++) nl = std::max(nl, lv[(size_t)q] + 1);
        std::vector<std::vector<int>> byl((size_t)nl);
        for (int q = q0; q < q1; q++) byl[(size_t)lv[(size_t)q]].push_back(q);
        for (auto &b : byl) {
          rows.insert(rows.end(), b.begin(), b.end());
          lev.push_back((int)rows.size());
        }
        sdl.push_back((int)lev.size() - 1);
      }
    }
    rp.upload(rph); ci.upload(cih); va.upload(vah); dg.upload(dgh); gidx.upload(gidx_h);
    sd_ptr.upload(sdp);
    sd_lev_f.upload(sdlf); sd_lev_b.upload(sdlb); lev_f.upload(levf); lev_b.upload(levb);
    rows_f.upload(rowf); rows_b.upload(rowb);
    x.alloc((size_t)std::max<int64_t>(len, 1));
    view = SgsView{rp.p, ci.p, va.p, dg.p, gidx.p, sd_lev_f.p, sd_lev_b.p, lev_f.p, lev_b.p, rows_f.p, rows_b.p};
  }
};

// Per-system PCG state of stacked vectors: the systems of a batch
// (dg_set_systems, vs = 0) or several right-hand sides of one matrix
// (dg_solve_multi, vector k at k*vs).  Chunks of at most kBatchChunk
// positions, none across two systems; one partial sum per chunk.
struct BatchCtx {
  int nsys = 0, nchunks = 0;
  int64_t vs = 0;
  DBuf<int> cb, csys, sys_cptr, state, iters, dit;
  DBuf<double> bsc, part_rz, part_rzo, part_pq, part_rr;
  int *host_counts = nullptr, *d_host_counts = nullptr;  // mapped pinned
  cudaGraphExec_t exec = nullptr;
  int exec_nodes = 0;
  BatchCtx() = default;
  BatchCtx(const BatchCtx &) = delete;
  BatchCtx &operator=(const BatchCtx &) = delete;
  ~BatchCtx() {
    if (exec) cudaGraphExecDestroy(exec);
    if (host_counts) cudaFreeHost(host_counts);
  }
  // row[k] .. row[k+1]: the positions of system k in the stacked vectors
  void build(const std::vector<int64_t> &row, int64_t vstride) {
    if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    nsys = (int)row.size() - 1;
    vs = vstride;
    std::vector<int> hb(1, 0), hs, hp(1, 0);
    for (int k = 0; k < nsys; k++) {
      for (int64_t r = row[(size_t)k]; r < row[(size_t)k + 1]; r += kBatchChunk) {
        hb.push_back((int)std::min<int64_t>(r + kBatchChunk, row[(size_t)k + 1]));
        hs.push_back(k);
      }
      hp.push_back((int)hs.size());
    }
    nchunks = (int)hs.size();
    cb.upload(hb); csys.upload(hs); sys_cptr.upload(hp);
    state.alloc((size_t)nsys); iters.alloc((size_t)nsys); dit.alloc(1);
    bsc.alloc((size_t)nsys * BS_N);
    CK(cudaMemset(state.p, 0, (size_t)nsys * sizeof(int)));
    CK(cudaMemset(bsc.p, 0, (size_t)nsys * BS_N * sizeof(double)));
    for (auto *v : {&part_rz, &part_rzo, &part_pq, &part_rr}) {
      v->alloc((size_t)nchunks);
      CK(cudaMemset(v->p, 0, (size_t)nchunks * sizeof(double)));
    }
    if (!host_counts) {
      CK(cudaHostAlloc(&host_counts, 4 * sizeof(int), cudaHostAllocMapped));
      CK(cudaHostGetDevicePointer(&d_host_counts, host_counts, 0));
    }
  }
};

// the PCG vectors of one stacked solve
struct Vecs {
  double *b, *x, *r, *p, *q, *z, *zold;
};

struct dg_handle {
  Controls ctl;
  std::string ctl_text;           // words given through dg_set_option (applied first)
  std::string ctl_dir = ".";
  std::string err;
  int n = 0;
  std::vector<int> ii, jj;
  std::vector<double> vv, rhs;
  bool have_matrix = false, have_rhs = false, ready = false;
  std::vector<int> part;
  // elemental input kept for the element gradients: local (0-based) unknown of
  // every element freedom, element offsets, matrices
  bool have_elements = false;
  std::vector<int> el_eptr, el_local;
  std::vector<int> el_free, el_lg;  // global freedoms of the elements; global freedom of every unknown
  int el_ngf = 0;
  // node coordinates of elemental input (the geometric coarse grid of doug_geom)
  bool have_geometry = false;
  NodeGeometry geo;
  std::vector<int64_t> el_off;
  std::vector<double> el_mat;
  DBuf<int> d_el_eptr, d_el_local, d_gi, d_gj, d_el_run, d_el_ridx;
  DBuf<int64_t> d_el_rptr;
  DBuf<double> d_el_c;
  int el_nrun = 0;
  bool elem_mv = false;           // PCG products with the element matrices
  DBuf<int64_t> d_el_off;
  DBuf<double> d_el_mat;
  bool el_sym = false;             // the matvec reads packed lower triangles
  DBuf<int64_t> d_el_poff;
  DBuf<double> d_el_pack;
  bool factored = false;          // the device holds factors of the current setup
  int nparts = 0;
  // batched independent systems (dg_set_systems): system k owns the rows
  // [sys_row[k], sys_row[k+1]) and the triplets [sys_tri[k], sys_tri[k+1])
  int nsys = 0;
  std::vector<int64_t> sys_row, sys_tri;
  BatchCtx bt;                    // the systems of a batch
  // several right-hand sides of one matrix (dg_solve_multi): mr_k right-hand
  // sides, stacked vectors
  BatchCtx mr;
  int mr_k = 0;
  DBuf<double> mb, mx, mrr, mp, mq, mz, mzold;
  std::vector<int> sys_iters, sys_state;
  std::vector<double> sys_relres, sys_seconds;
  SetupResult S;
  MfBatch Bsub, Bco;
  double t_setup = 0;
  int precision = 0;
  int lanes = 8;
  int r_lanes = 32;               // lanes per row of the restriction R
  int pull_grid = kRedBlocks;     // CTAs of the single-system pull kernel: one wave
  // device
  int device = 0;
  DBuf<int64_t> Ap, Rp, Pp;
  DBuf<int> pull_ptr, pull_idx;   // per node: its positions in the subdomain arena
  DBuf<int> Ac, Rc, Pc, cpos, status;
  DBuf<double> Av, ACv, Rv, Pv, b, x, r, p, q, z, zold, hb, hx;
  DBuf<float> Rvf, Pvf;
  DBuf<double> part_rz, part_rzo, part_pq, part_rr, sc;
  std::unique_ptr<MfDevice<double>> sub64, co64;
  std::unique_ptr<MfDevice<float>> sub32;
  std::unique_ptr<SgsDevice> sgs;
  double *host_out = nullptr;     // mapped pinned
  int *host_status = nullptr;
  double *d_host_out = nullptr;
  int *d_host_status = nullptr;
  cudaEvent_t ev[10]{};
  cudaStream_t s2 = nullptr;        // coarse-level stream (runs beside the subdomain solves)
  cudaStream_t s2f = nullptr;       // high-priority stream of the coarse factorisation
  cudaStream_t sf = nullptr;        // low-priority stream of the subdomain factorisation
  cudaEvent_t fine_ev = nullptr;
  cudaStream_t s3 = nullptr;        // capture stream of the iteration graph
  cudaGraphExec_t iter_exec = nullptr;
  int iter_nodes = 0;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  ~dg_handle() {
    if (iter_exec) cudaGraphExecDestroy(iter_exec);
    if (s2) cudaStreamDestroy(s2);
    if (s2f) cudaStreamDestroy(s2f);
    if (sf) cudaStreamDestroy(sf);
    if (fine_ev) cudaEventDestroy(fine_ev);
    if (s3) cudaStreamDestroy(s3);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (host_out) cudaFreeHost(host_out);
    if (host_status) cudaFreeHost(host_status);
    for (auto &e : ev) if (e) cudaEventDestroy(e);
  }
};

namespace {

dg_status fail(dg_handle *h, dg_status s, const std::string &msg) {
  h->err = msg;
  return s;
}

dg_status cuda_fail(dg_handle *h, const CudaError &e) {
  h->err = std::string("CUDA error in ") + e.what + ": " + cudaGetErrorString(e.e);
  return DG_CUDA_ERROR;
}

// host Lanczos eigenvalue range of the CG tridiagonal (pcg.F90:465-491):
// bisection with Sturm counts, an independent method from the reference's QL
double tridiag_cond(const std::vector<double> &alpha, const std::vector<double> &beta) {
  int it = (int)alpha.size();
  if (it < 1) return 0.0;
  std::vector<double> d((size_t)it), e((size_t)it, 0.0);
  d[0] = 1.0 / alpha[0];
  for (int i = 1; i < it; i++) {
    if (alpha[(size_t)i] == 0 || beta[(size_t)i] < 0) return 0.0;
    d[(size_t)i] = 1.0 / alpha[(size_t)i] + beta[(size_t)i] / alpha[(size_t)i - 1];
    e[(size_t)i] = -std::sqrt(beta[(size_t)i]) / alpha[(size_t)i - 1];
  }
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < it; i++) {
    double rr = (i > 0 ? std::fabs(e[(size_t)i]) : 0) + (i + 1 < it ? std::fabs(e[(size_t)i + 1]) : 0);
    lo = std::min(lo, d[(size_t)i] - rr);
    hi = std::max(hi, d[(size_t)i] + rr);
  }
  auto count_below = [&](double xv) {  // eigenvalues < xv
    int c = 0;
    double q = d[0] - xv;
    if (q < 0) c++;
    for (int i = 1; i < it; i++) {
      if (q == 0) q = 1e-300;
      q = d[(size_t)i] - xv - e[(size_t)i] * e[(size_t)i] / q;
      if (q < 0) c++;
    }
    return c;
  };
  auto kth = [&](int kidx) {  // kidx-th smallest (0-based)
    double a = lo, b = hi;
    for (int t = 0; t < 200; t++) {
      double mid = 0.5 * (a + b);
      if (count_below(mid) > kidx) b = mid; else a = mid;
    }
    return 0.5 * (a + b);
  };
  double lmin = kth(0), lmax = kth(it - 1);
  return lmin != 0 ? lmax / lmin : 0.0;
}

// lanes per CSR row: about 12 entries per lane (each lane loads four at a time)
int lanes_for(const Csr &A) {
  double avg = A.nrows ? (double)A.nnz() / A.nrows : 1;
  if (avg <= 12) return 1;
  if (avg <= 24) return 2;
  if (avg <= 48) return 4;
  if (avg <= 96) return 8;
  if (avg <= 192) return 16;
  return 32;
}

template <int L>
void launch_spmv(int grid, cudaStream_t s, dg_handle *h, int first, int flexible) {
  cg_direction<<<grid, kVecThreads, 0, s>>>(h->n, h->z.p, h->p.p, h->part_rz.p, h->part_rzo.p, h->sc.p, first,
                                            flexible);
  spmv_pq<L><<<grid, kVecThreads, 0, s>>>(h->n, h->Ap.p, h->Ac.p, h->Av.p, h->p.p, h->q.p, h->part_pq.p);
}
template <int L>
void launch_resid(int grid, cudaStream_t s, dg_handle *h, const double *xx, const double *bb, double *rr) {
  residual<L><<<grid, kVecThreads, 0, s>>>(h->n, h->Ap.p, h->Ac.p, h->Av.p, xx, bb, rr, h->part_rr.p);
}
void spmv_any(int lanes, int grid, cudaStream_t s, dg_handle *h, int first, int flexible) {
  if (h->elem_mv) {  // matrix-free product with the element matrices
    cg_direction<<<grid, kVecThreads, 0, s>>>(h->n, h->z.p, h->p.p, h->part_rz.p, h->part_rzo.p, h->sc.p, first,
                                              flexible);
    if (h->el_sym)
      elem_contrib<true><<<h->el_nrun, 256, 0, s>>>(h->d_el_run.p, h->d_el_eptr.p, h->d_el_local.p,
                                                    h->d_el_poff.p, h->d_el_pack.p, h->p.p, h->d_el_c.p);
    else
      elem_contrib<false><<<h->el_nrun, 256, 0, s>>>(h->d_el_run.p, h->d_el_eptr.p, h->d_el_local.p,
                                                     h->d_el_off.p, h->d_el_mat.p, h->p.p, h->d_el_c.p);
    elem_pull_pq<<<grid, kVecThreads, 0, s>>>(h->n, h->d_el_rptr.p, h->d_el_ridx.p, h->d_el_c.p, h->p.p, h->q.p,
                                              h->part_pq.p);
    return;
  }
  switch (lanes) {
    case 1: launch_spmv<1>(grid, s, h, first, flexible); break;
    case 2: launch_spmv<2>(grid, s, h, first, flexible); break;
    case 4: launch_spmv<4>(grid, s, h, first, flexible); break;
    case 8: launch_spmv<8>(grid, s, h, first, flexible); break;
    case 16: launch_spmv<16>(grid, s, h, first, flexible); break;
    default: launch_spmv<32>(grid, s, h, first, flexible); break;
  }
}
void resid_any(int lanes, int grid, cudaStream_t s, dg_handle *h, const double *xx, const double *bb, double *rr) {
  switch (lanes) {
    case 1: launch_resid<1>(grid, s, h, xx, bb, rr); break;
    case 2: launch_resid<2>(grid, s, h, xx, bb, rr); break;
    case 4: launch_resid<4>(grid, s, h, xx, bb, rr); break;
    case 8: launch_resid<8>(grid, s, h, xx, bb, rr); break;
    case 16: launch_resid<16>(grid, s, h, xx, bb, rr); break;
    default: launch_resid<32>(grid, s, h, xx, bb, rr); break;
  }
}

// x_c = R r with L lanes per coarse row
template <typename TR>
void restrict_any(int lanes, int grid, cudaStream_t s, const int64_t *Rp, const int *Rc, const TR *Rv, const double *r,
                  const int *cpos, double *xc, int nc, int K, int64_t rs, int64_t xcs) {
  switch (lanes) {
    case 1: restrict_to_coarse<TR, 1><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
    case 2: restrict_to_coarse<TR, 2><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
    case 4: restrict_to_coarse<TR, 4><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
    case 8: restrict_to_coarse<TR, 8><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
    case 16: restrict_to_coarse<TR, 16><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
    default: restrict_to_coarse<TR, 32><<<grid, kVecThreads, 0, s>>>(Rp, Rc, Rv, r, cpos, xc, nc, K, rs, xcs); break;
  }
}

// stacked systems / right-hand sides: the chunked product and residual
template <int L>
void launch_bt(cudaStream_t s, dg_handle *h, BatchCtx &c, const Vecs &v, int resid, int want, double *rr) {
  if (resid)
    bt_residual<L><<<c.nchunks, kVecThreads, 0, s>>>(c.cb.p, c.csys.p, c.state.p, want, h->Ap.p, h->Ac.p, h->Av.p,
                                                     v.x, v.b, rr, c.part_rr.p, c.vs);
  else
    bt_spmv_pq<L><<<c.nchunks, kVecThreads, 0, s>>>(c.cb.p, c.csys.p, c.state.p, h->Ap.p, h->Ac.p, h->Av.p, v.p, v.q,
                                                    c.part_pq.p, c.vs);
}
void bt_any(cudaStream_t s, dg_handle *h, BatchCtx &c, const Vecs &v, int resid, int want = -1,
            double *rr = nullptr) {
  switch (h->lanes) {
    case 1: launch_bt<1>(s, h, c, v, resid, want, rr); break;
    case 2: launch_bt<2>(s, h, c, v, resid, want, rr); break;
    case 4: launch_bt<4>(s, h, c, v, resid, want, rr); break;
    case 8: launch_bt<8>(s, h, c, v, resid, want, rr); break;
    case 16: launch_bt<16>(s, h, c, v, resid, want, rr); break;
    default: launch_bt<32>(s, h, c, v, resid, want, rr); break;
  }
}
void bt_step(BatchCtx &c, cudaStream_t s, int step, int first, int mixed, double tol2, const double *pa,
             const double *pb) {
  bt_scalars<<<1, 1024, 0, s>>>(c.nsys, c.sys_cptr.p, step, first, mixed, mixed, tol2, pa, pb, c.bsc.p, c.state.p,
                                c.iters.p, c.dit.p, c.d_host_counts);
}

// q = A r with L lanes per row and the r.q partials (any CSR on the device)
void spmv_lanes(int lanes, cudaStream_t s, int n, const int64_t *Ap, const int *Ac, const double *Av,
                const double *r, double *q, double *part) {
  const int g = kRedBlocks;
  switch (lanes) {
    case 1: spmv_pq<1><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
    case 2: spmv_pq<2><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
    case 4: spmv_pq<4><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
    case 8: spmv_pq<8><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
    case 16: spmv_pq<16><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
    default: spmv_pq<32><<<g, kVecThreads, 0, s>>>(n, Ap, Ac, Av, r, q, part); break;
  }
}

// Robust coarse space (coarse_method 2) on the GPU.  B p = sum_i R_i^T
// A_i^-1 R_i p is one gather into the supports, one batched FP64
// multifrontal solve of all support matrices A_i = A(S_i, S_i) and one pull
// sum (supports in order).  B g = 1 is solved by CG preconditioned with A
// itself (B is locally a multiple of A^-1), to ||r||/||r0|| <= 1e-14 or until
// the residual stops falling: the reference's CG (pcg_forRCS,
// pcg_robust.f90:37-120) asks for ||r||/||r0|| <= tol^2, so it too solves to
// rounding level.  Then q_i = A_i^-1 g(S_i) (RobustRestrictMtxBuild,
// RobustCoarseMtx.f90:175-202) with the same factors.
bool robust_restriction_gpu(const Controls &c, const Csr &A, const std::vector<int64_t> &sp,
                            const std::vector<int> &sn, std::vector<double> &q, std::string &err,
                            bool &no_device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    no_device = true;
    err = "no CUDA device is visible; the robust coarse space is built on the GPU";
    return false;
  }
  cudaStream_t s = nullptr;
  double *host_out = nullptr, *d_host_out = nullptr;
  int *host_status = nullptr, *d_host_status = nullptr;
  bool ok = false;
  try {
    const int n = A.nrows;
    std::vector<int> sn1(sn.size());
    for (size_t k = 0; k < sn.size(); k++) sn1[k] = sn[k] + 1;
    MfBatch Bs;
    MfOptions mo;
    mo.leaf = c.nd_leaf;
    mf_build_subdomains(A, sp, sn1, mo, Bs);
    MfTune tune;
    tune.panel_rows = c.panel_rows;
    tune.fwd_task_bytes = (int64_t)c.fwd_task_kb * 1024;
    tune.lean_task_bytes = (int64_t)c.lean_task_kb * 1024;
    tune.small_min_fronts = c.thin_level_fronts;
    tune.tensor_update = c.tensor_update;
    tune.super_panel = c.super_panel;
    tune.queue_wait_cycles = c.queue_wait_cycles;
    tune.queue_skip_publish = c.queue_skip_publish;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CK(cudaHostAlloc(&host_out, 16 * sizeof(double), cudaHostAllocMapped));
    CK(cudaHostAlloc(&host_status, sizeof(int), cudaHostAllocMapped));
    CK(cudaHostGetDevicePointer(&d_host_out, host_out, 0));
    CK(cudaHostGetDevicePointer(&d_host_status, host_status, 0));
    MfDevice<double> dev;
    dev.upload(Bs, tune);
    DBuf<double> Av, x, r, z, p, qv, part_rz, part_pq, part_rr, sc;
    DBuf<int64_t> Ap;
    DBuf<int> Ac, status, pull_ptr, pull_idx;
    Av.upload(A.val); Ap.upload(A.ptr); Ac.upload(A.col);
    for (auto *v : {&x, &r, &z, &p, &qv}) v->alloc((size_t)n);
    for (auto *v : {&part_rz, &part_pq, &part_rr}) v->alloc(kRedBlocks);
    sc.alloc(8);
    status.alloc(1);
    CK(cudaMemset(sc.p, 0, 8 * sizeof(double)));
    CK(cudaMemset(status.p, 0, sizeof(int)));
    {  // pull lists: support arena positions of every node, supports in order
      std::vector<int> pp((size_t)n + 1, 0);
      for (int g : Bs.gidx) pp[(size_t)g + 1]++;
      for (int i = 0; i < n; i++) pp[(size_t)i + 1] += pp[(size_t)i];
      std::vector<int> idx((size_t)pp[(size_t)n]);
      std::vector<int> fill(pp.begin(), pp.end() - 1);
      for (int k = 0; k < (int)Bs.gidx.size(); k++) idx[(size_t)fill[(size_t)Bs.gidx[(size_t)k]]++] = k;
      pull_ptr.upload(pp);
      pull_idx.upload(idx);
    }
    dev.factor(Av.p, status.p, s);
    int stv = 0;
    CK(cudaMemcpyAsync(&stv, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (stv & ERR_NOT_SPD) throw CudaError{cudaSuccess, "robust coarse space: a support matrix is not positive definite"};
    const std::vector<double> ones((size_t)n, 1.0);
    CK(cudaMemcpy(r.p, ones.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemset(x.p, 0, (size_t)n * sizeof(double)));
    CK(cudaMemset(p.p, 0, (size_t)n * sizeof(double)));
    const int lanes = lanes_for(A), grid = kRedBlocks;
    const double init = (double)n;  // ||1||^2
    double best = init;
    int since_best = 0;
    for (int it = 1; it <= 10000; it++) {
      spmv_lanes(lanes, s, n, Ap.p, Ac.p, Av.p, r.p, z.p, part_rz.p);  // z = A r, r.z
      cg_direction<<<grid, kVecThreads, 0, s>>>(n, z.p, p.p, part_rz.p, part_rz.p, sc.p, it == 1, 0);
      gather_subdomains<double><<<grid, kVecThreads, 0, s>>>(p.p, dev.gidx.p, dev.xl.p, dev.xlen);
      dev.solve(s);
      pull_prolong_dot<double, double><<<grid, kVecThreads, 0, s>>>(
          n, pull_ptr.p, pull_idx.p, dev.xl.p, nullptr, nullptr, nullptr, nullptr, 1, p.p, qv.p, nullptr,
          part_pq.p, nullptr);  // q = B p, p.q
      cg_update<<<grid, kVecThreads, 0, s>>>(n, p.p, qv.p, x.p, r.p, sc.p, part_pq.p, part_rr.p);
      cg_finish<<<1, 32, 0, s>>>(sc.p, part_rr.p, 0, d_host_out, status.p, d_host_status);
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(s));
      const double res = host_out[0];
      if (!(res == res) || !(host_out[5] > 0.0))
        throw CudaError{cudaSuccess, "robust coarse space: CG breakdown in B g = 1"};
      if (res <= 1e-28 * init) break;
      if (res < 0.25 * best) { best = res; since_best = 0; }
      else if (++since_best >= 25) break;  // stagnated at rounding level
    }
    // q_i = A_i^-1 g(S_i), back in support order
    gather_subdomains<double><<<grid, kVecThreads, 0, s>>>(x.p, dev.gidx.p, dev.xl.p, dev.xlen);
    dev.solve(s);
    std::vector<double> xl((size_t)dev.xlen);
    CK(cudaMemcpyAsync(xl.data(), dev.xl.p, xl.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    q.assign(sn.size(), 0.0);
    std::vector<int> posn((size_t)n, -1);
    for (size_t i = 0; i + 1 < sp.size(); i++) {
      for (int64_t k = sp[i]; k < sp[i + 1]; k++) posn[(size_t)sn[(size_t)k]] = (int)(k - sp[i]);
      for (int64_t a = Bs.xoff[i]; a < Bs.xoff[i + 1]; a++)
        q[(size_t)(sp[i] + posn[(size_t)Bs.gidx[(size_t)a]])] = xl[(size_t)a];
      for (int64_t k = sp[i]; k < sp[i + 1]; k++) posn[(size_t)sn[(size_t)k]] = -1;
    }
    ok = true;
  } catch (const CudaError &e) {
    err = e.e == cudaSuccess ? std::string(e.what) : std::string("CUDA error in ") + e.what + ": " + cudaGetErrorString(e.e);
  } catch (const std::exception &ex) {
    err = std::string("robust coarse space: ") + ex.what();
  }
  if (s) cudaStreamDestroy(s);
  if (host_out) cudaFreeHost(host_out);
  if (host_status) cudaFreeHost(host_status);
  return ok;
}

// host setup (aggregation, R, AC, subdomains; skipped with reuse_host when
// it is current), symbolic analysis and device upload
dg_status do_setup(dg_handle *h, bool reuse_host = false) {
  if (!h->have_matrix) return fail(h, DG_NOT_READY, "no matrix: call dg_set_matrix_coo or dg_load_ctl first");
  std::string err;
  Controls c = h->ctl;
  ctl_finish(c);
  double t0 = wall();
  if (!(reuse_host && h->S.n == h->n && h->S.n > 0)) {
    if (c.executable == 1) {  // doug_geom (geom.F90:62-116)
      if (h->nsys > 0) return fail(h, DG_BAD_INPUT, "batched systems run the doug_aggr setup only");
      if (!build_setup_geom(c, h->n, h->ii, h->jj, h->vv, h->part.empty() ? nullptr : &h->part, h->nparts,
                            h->have_elements ? &h->el_free : nullptr, h->have_elements ? &h->el_lg : nullptr,
                            h->have_geometry ? &h->geo : nullptr, h->S, err))
        return fail(h, DG_BAD_INPUT, err);
    } else if (c.coarse_method == 3 && h->nsys == 0) {
      // smoothed aggregation over nodal blocks with rigid-body modes: the node
      // of every unknown from the freedom map of the element mesh
      if (!h->have_elements || !h->have_geometry)
        return fail(h, DG_BAD_INPUT, "coarse_method 3 needs elemental input with node coordinates "
                                     "(coords_file / freemap_file or dg_set_node_geometry)");
      std::vector<int> unode((size_t)h->n);
      for (int u = 0; u < h->n; u++) unode[(size_t)u] = h->geo.freemap[(size_t)h->el_lg[(size_t)u] - 1] - 1;
      if (!build_setup_rbm(c, h->n, h->ii, h->jj, h->vv, h->part.empty() ? nullptr : &h->part, h->nparts, unode,
                           h->geo.nsd, h->geo.coords, h->S, err))
        return fail(h, DG_BAD_INPUT, err);
    } else if (h->nsys > 0) {
      if (!h->part.empty()) return fail(h, DG_BAD_INPUT, "a partition vector cannot be combined with batched systems");
      if (!build_setup_systems(c, h->sys_row, h->sys_tri, h->ii, h->jj, h->vv, h->S, err))
        return fail(h, DG_BAD_INPUT, err);
    } else {
      bool no_device = false;
      const RobustHook hook = [&](const Csr &A, const std::vector<int64_t> &sp, const std::vector<int> &sn,
                                  std::vector<double> &q, std::string &e) {
        return robust_restriction_gpu(c, A, sp, sn, q, e, no_device);
      };
      int ndev_setup = 0;
      const bool on_device = cudaGetDeviceCount(&ndev_setup) == cudaSuccess && ndev_setup > 0;
      if (!build_setup(c, h->n, h->ii, h->jj, h->vv, h->part.empty() ? nullptr : &h->part, h->nparts, h->S, err,
                       &hook, on_device))
        return fail(h, no_device ? DG_NO_DEVICE : DG_BAD_INPUT, err);
    }
  }
  MfTune tune;
  tune.panel_rows = c.panel_rows;
  tune.fwd_task_bytes = (int64_t)c.fwd_task_kb * 1024;
  tune.lean_task_bytes = (int64_t)c.lean_task_kb * 1024;
  tune.small_min_fronts = c.thin_level_fronts;
  tune.tensor_update = c.tensor_update;
  tune.super_panel = c.super_panel;
  tune.queue_wait_cycles = c.queue_wait_cycles;
  tune.queue_skip_publish = c.queue_skip_publish;
  tune.schedule = c.solve_schedule;
  tune.pdl = c.solve_pdl;
  tune.factor_overlap = c.factor_overlap;
  MfOptions mo;
  mo.leaf = c.nd_leaf;
  const bool timing = std::getenv("DG_SETUP_TIMING") != nullptr;
  const double t1 = wall();
  try {
    if (c.fine_method == 1) mf_build_subdomains(h->S.A, h->S.sd_ptr, h->S.sd_nodes, mo, h->Bsub);
    const double t2 = wall();
    if (c.levels > 1) mf_build_single(h->S.AC, mo, h->Bco);
    if (timing)
      fprintf(stderr, "[setup] host setup %.3f s, subdomain analysis %.3f s, coarse analysis %.3f s\n", t1 - t0,
              t2 - t1, wall() - t2);
  } catch (const std::exception &ex) {
    return fail(h, DG_BAD_INPUT, std::string("symbolic analysis failed: ") + ex.what());
  }
  h->t_setup = wall() - t0;
  h->precision = c.precision;
  // device upload
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(h, DG_NO_DEVICE, "no CUDA device is visible; the solver has no CPU fallback");
  try {
    CK(cudaGetDevice(&h->device));
    const SetupResult &S = h->S;
    int n = h->n;
    h->factored = false;
    {  // input triplets (0-based) for the matrix gradient; element data for the element gradient
      const int shift = (!h->ii.empty() && h->ii[0] == 0) ? 0 : 1;  // 0-based input is accepted
      std::vector<int> gi(h->ii.size()), gj(h->jj.size());
      for (size_t k = 0; k < gi.size(); k++) { gi[k] = h->ii[k] - shift; gj[k] = h->jj[k] - shift; }
      h->d_gi.upload(gi);
      h->d_gj.upload(gj);
      h->elem_mv = false;
      if (h->have_elements) {
        h->d_el_eptr.upload(h->el_eptr); h->d_el_local.upload(h->el_local);
        h->d_el_off.upload(h->el_off); h->d_el_mat.upload(h->el_mat);
        if (c.elemental_matvec == 1) {
          // bitwise symmetric element matrices are read as packed lower
          // triangles (the same values, 46 % fewer bytes for 12 x 12)
          const int nell = (int)h->el_eptr.size() - 1;
          bool sym = true;
          for (int e = 0; e < nell && sym; e++) {
            const int nf = h->el_eptr[(size_t)e + 1] - h->el_eptr[(size_t)e];
            const double *A = &h->el_mat[(size_t)h->el_off[(size_t)e]];
            for (int j = 0; j < nf && sym; j++)
              for (int i = j + 1; i < nf; i++)
                if (!(A[(size_t)j * nf + i] == A[(size_t)i * nf + j])) { sym = false; break; }
          }
          std::vector<int64_t> poff(1, 0);
          if (sym) {
            for (int e = 0; e < nell; e++) {
              const int64_t nf = h->el_eptr[(size_t)e + 1] - h->el_eptr[(size_t)e];
              poff.push_back(poff.back() + nf * (nf + 1) / 2);
            }
            std::vector<double> pack((size_t)poff.back());
            for (int e = 0; e < nell; e++) {
              const int nf = h->el_eptr[(size_t)e + 1] - h->el_eptr[(size_t)e];
              const double *A = &h->el_mat[(size_t)h->el_off[(size_t)e]];
              double *P = &pack[(size_t)poff[(size_t)e]];
              for (int j = 0, o = 0; j < nf; j++)
                for (int i = j; i < nf; i++) P[o++] = A[(size_t)j * nf + i];
            }
            h->d_el_poff.upload(poff);
            h->d_el_pack.upload(pack);
          }
          h->el_sym = sym;
          const std::vector<int64_t> &moff = sym ? poff : h->el_off;
          // element runs of at most kElemChunk matrix values, kElemFree
          // freedoms and kElemRun elements; per row, its contribution slots
          // in element order
          std::vector<int> run(1, 0);
          for (int e = 0; e < nell; e++) {
            const int64_t sz = moff[(size_t)e + 1] - moff[(size_t)e];
            const int nf = h->el_eptr[(size_t)e + 1] - h->el_eptr[(size_t)e];
            if (sz > kElemChunk || nf > kElemFree)
              throw CudaError{cudaErrorInvalidValue, "element matrix larger than the matvec stage"};
            const int r0 = run.back();
            if (moff[(size_t)e + 1] - moff[(size_t)r0] > kElemChunk ||
                h->el_eptr[(size_t)e + 1] - h->el_eptr[(size_t)r0] > kElemFree || e + 1 - r0 > kElemRun)
              run.push_back(e);
          }
          run.push_back(nell);
          std::vector<int64_t> rptr((size_t)n + 1, 0);
          for (int l : h->el_local) rptr[(size_t)l + 1]++;
          for (int i = 0; i < n; i++) rptr[(size_t)i + 1] += rptr[(size_t)i];
          std::vector<int> ridx(h->el_local.size());
          std::vector<int64_t> fillp(rptr.begin(), rptr.end() - 1);
          for (size_t t = 0; t < h->el_local.size(); t++) ridx[(size_t)fillp[(size_t)h->el_local[t]]++] = (int)t;
          h->d_el_run.upload(run);
          h->el_nrun = (int)run.size() - 1;
          h->d_el_rptr.upload(rptr);
          h->d_el_ridx.upload(ridx);
          h->d_el_c.alloc(std::max<size_t>(h->el_local.size(), 1));
          h->elem_mv = true;
        }
      }
    }
    h->Ap.upload(S.A.ptr); h->Ac.upload(S.A.col); h->Av.upload(S.A.val);
    h->lanes = lanes_for(S.A);
    for (auto *v : {&h->b, &h->x, &h->r, &h->p, &h->q, &h->z, &h->zold, &h->hb, &h->hx}) v->alloc((size_t)n);
    if (h->nsys > 0) h->bt.build(h->sys_row, 0);
    h->mr_k = 0;  // the right-hand-side stacks are rebuilt on demand
    if (h->mr.exec) { cudaGraphExecDestroy(h->mr.exec); h->mr.exec = nullptr; }
    for (auto *v : {&h->part_rz, &h->part_rzo, &h->part_pq, &h->part_rr}) {
      v->alloc(kRedBlocks);
      CK(cudaMemset(v->p, 0, kRedBlocks * sizeof(double)));
    }
    h->sc.alloc(8);
    CK(cudaMemset(h->sc.p, 0, 8 * sizeof(double)));
    h->status.alloc(1);
    CK(cudaMemset(h->status.p, 0, sizeof(int)));
    if (!h->host_out) {
      CK(cudaHostAlloc(&h->host_out, 16 * sizeof(double), cudaHostAllocMapped));
      CK(cudaHostAlloc(&h->host_status, sizeof(int), cudaHostAllocMapped));
      CK(cudaHostGetDevicePointer(&h->d_host_out, h->host_out, 0));
      CK(cudaHostGetDevicePointer(&h->d_host_status, h->host_status, 0));
      for (auto &e : h->ev) CK(cudaEventCreate(&e));
      // factorisations: the coarse chain (a few fronts per level, one long
      // chain of panel steps at the top) gets the highest priority, so that
      // its CTAs start as soon as an SM has room; the subdomain chain, wide
      // enough to fill the rest, the lowest.  In the iterations the coarse
      // solve's stream has the lowest priority beside the subdomain solves.
      int prio_lo = 0, prio_hi = 0;
      CK(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
      CK(cudaStreamCreateWithPriority(&h->s2, cudaStreamNonBlocking, prio_lo));
      CK(cudaStreamCreateWithPriority(&h->s2f, cudaStreamNonBlocking, prio_hi));
      CK(cudaStreamCreateWithPriority(&h->sf, cudaStreamNonBlocking, prio_lo));
      CK(cudaEventCreateWithFlags(&h->fine_ev, cudaEventDisableTiming));
      CK(cudaStreamCreateWithFlags(&h->s3, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming));
    }
    if (h->iter_exec) { cudaGraphExecDestroy(h->iter_exec); h->iter_exec = nullptr; }
    // transfer operators
    h->Rp.upload(S.R.ptr); h->Rc.upload(S.R.col); h->Rv.upload(S.R.val);
    h->r_lanes = lanes_for(S.R);
    {  // the pull kernel holds 64 registers: a 1024-CTA grid would be 1.7 waves
      int dev = 0, nsm = 0, occ = 0;
      CK(cudaGetDevice(&dev));
      CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      if (c.precision == 1)
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pull_prolong_dot<float, float>, kVecThreads, 0));
      else
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pull_prolong_dot<double, double>, kVecThreads, 0));
      h->pull_grid = std::max(1, std::min(kRedBlocks, nsm * std::max(occ, 1)));
    }
    h->Pp.upload(S.P.ptr); h->Pv.upload(S.P.val);
    std::vector<float> rf(S.R.val.begin(), S.R.val.end()), pf(S.P.val.begin(), S.P.val.end());
    h->Rvf.upload(rf); h->Pvf.upload(pf);
    h->ACv.upload(S.AC.val);
    // subdomain batch
    h->sub64.reset(); h->sub32.reset(); h->co64.reset(); h->sgs.reset();
    if (c.fine_method == 1 || c.fine_method == 2) {
      const std::vector<int> *arena_rows = &h->Bsub.gidx;
      if (c.fine_method == 2) {
        h->sgs.reset(new SgsDevice());
        h->sgs->build(S.A, S.sd_ptr, S.sd_nodes);
        arena_rows = &h->sgs->gidx_h;
      } else if (h->precision == 1) {
        h->sub32.reset(new MfDevice<float>()); h->sub32->upload(h->Bsub, tune);
      } else {
        h->sub64.reset(new MfDevice<double>()); h->sub64->upload(h->Bsub, tune);
      }
      // pull lists: subdomain arena positions of every node, subdomain order
      if (arena_rows->size() >= (size_t)INT_MAX)
        throw CudaError{cudaErrorInvalidValue, "subdomain arena beyond 32-bit positions"};
      std::vector<int> pp((size_t)n + 1, 0);
      for (int g : *arena_rows) pp[(size_t)g + 1]++;
      for (int i = 0; i < n; i++) pp[(size_t)i + 1] += pp[(size_t)i];
      std::vector<int> idx((size_t)pp[(size_t)n]);
      std::vector<int> fill(pp.begin(), pp.end() - 1);
      for (int q = 0; q < (int)arena_rows->size(); q++)
        idx[(size_t)fill[(size_t)(*arena_rows)[(size_t)q]]++] = q;
      h->pull_ptr.upload(pp);
      h->pull_idx.upload(idx);
    } else {
      h->pull_ptr.alloc(1); h->pull_idx.alloc(1);
    }
    if (c.levels > 1) {
      h->co64.reset(new MfDevice<double>());
      h->co64->upload(h->Bco, tune);
      std::vector<int> cp((size_t)S.AC.nrows, 0);
      for (int64_t q = 0; q < (int64_t)h->Bco.gidx.size(); q++) cp[(size_t)h->Bco.gidx[(size_t)q]] = (int)q;
      h->cpos.upload(cp);
      // prolongation columns as positions in the coarse solver's vector
      std::vector<int> pcp(S.P.col.size());
      for (size_t e = 0; e < pcp.size(); e++) pcp[e] = cp[(size_t)S.P.col[e]];
      h->Pc.upload(pcp);
    } else {
      h->cpos.alloc(1);
      h->Pc.alloc(1);
    }
    CK(cudaDeviceSynchronize());
  } catch (const CudaError &e) {
    return cuda_fail(h, e);
  }
  h->factored = false;
  h->ready = true;
  return DG_OK;
}

// what one solve applies, from the control words
struct SolvePlan {
  bool fine = false, sgs = false, coarse = false, mixed = false;
  int sgs_iters = 3, mode = 0;
};

SolvePlan plan_of(const dg_handle *h, const Controls &c) {
  SolvePlan pl;
  pl.fine = (c.fine_method == 1 || c.fine_method == 2) && c.method != 0;
  pl.sgs = c.fine_method == 2;
  pl.sgs_iters = c.num_iters <= 0 ? 3 : c.num_iters;  // aggr.F90:221
  pl.coarse = c.levels > 1 && c.method != 0;
  pl.mixed = h->precision == 1;
  if (c.method == 0) pl.mode |= 4;
  else if (c.fine_method == 0) pl.mode |= 4;
  else pl.mode |= 1;
  // (the reference adds the coarse correction only for method 1, pcg.F90:191-193)
  if (pl.coarse && (c.method == 1 || c.method == 5)) pl.mode |= 2;  // method 5: pcg.F90:205-208
  if (pl.mixed) pl.mode |= 8;
  return pl;
}

// numeric factorisations (the reference factorises lazily in the first
// preconditioner call, subsolvers.F90:78-101, pcg.F90:166-178): the coarse
// factorisation on the high-priority stream beside the subdomain
// factorisations on the low-priority one.  Returns the number of kernels.
int factor_all(dg_handle *h, const SolvePlan &pl, cudaStream_t s) {
  int launches = 0;
  if (pl.coarse) {
    CK(cudaEventRecord(h->fork_ev, s));
    CK(cudaStreamWaitEvent(h->s2f, h->fork_ev, 0));
    launches += h->co64->factor(h->ACv.p, h->status.p, h->s2f);
    CK(cudaEventRecord(h->join_ev, h->s2f));
  }
  if (pl.fine && !pl.sgs) {
    CK(cudaEventRecord(h->fork_ev, s));
    CK(cudaStreamWaitEvent(h->sf, h->fork_ev, 0));
    launches += pl.mixed ? h->sub32->factor(h->Av.p, h->status.p, h->sf)
                         : h->sub64->factor(h->Av.p, h->status.p, h->sf);
    CK(cudaEventRecord(h->fine_ev, h->sf));
    CK(cudaStreamWaitEvent(s, h->fine_ev, 0));
  }
  if (pl.coarse) CK(cudaStreamWaitEvent(s, h->join_ev, 0));
  return launches;
}

// z = M r and the r.z partials: restriction + coarse solve on the second
// stream beside the subdomain solves, then the pull sum with the
// prolongation.  pg: grid of the pull kernel; cb: the chunk table of batched
// systems (one chunk per CTA) or null.  Returns the number of kernels.
// The stacked vectors and partial sums of one solve: the handle's own
// vectors for a single system; ctx's for stacked systems / right-hand sides.
struct StackArgs {
  Vecs v;
  double *part_rz, *part_rzo;
  int pg;                  // grid of the pull kernel
  const int *cb = nullptr, *csys = nullptr;
  int nrhs = 1;            // > 1: right-hand sides of one matrix
};

int precondition(dg_handle *h, const SolvePlan &pl, cudaStream_t st, bool profile, const StackArgs &a) {
  const int grid = kRedBlocks;
  const int n = h->n, K = a.nrhs;
  const int64_t vs = K > 1 ? n : 0;
  int nl = 0;
  MfDevice<double> *co = h->co64.get();
  double *xc_buf = nullptr;
  if (pl.coarse) {  // restriction + coarse solve on the second stream
    xc_buf = K > 1 ? co->xlm.p : co->xl.p;
    const int64_t xcs = K > 1 ? co->xlen : 0;
    CK(cudaEventRecord(h->fork_ev, st));
    CK(cudaStreamWaitEvent(h->s2, h->fork_ev, 0));
    if (profile) CK(cudaEventRecord(h->ev[4], h->s2));
    if (pl.mixed) restrict_any<float>(h->r_lanes, grid, h->s2, h->Rp.p, h->Rc.p, h->Rvf.p, a.v.r, h->cpos.p, xc_buf,
                                       h->S.R.nrows, K, vs, xcs);
    else restrict_any<double>(h->r_lanes, grid, h->s2, h->Rp.p, h->Rc.p, h->Rv.p, a.v.r, h->cpos.p, xc_buf,
                              h->S.R.nrows, K, vs, xcs);
    nl += 1 + co->solve(h->s2, K, h->status.p);
    if (profile) CK(cudaEventRecord(h->ev[5], h->s2));
    CK(cudaEventRecord(h->join_ev, h->s2));
  }
  if (profile) CK(cudaEventRecord(h->ev[3], st));
  const void *xl_fine = nullptr;
  int64_t xls = 0;
  if (pl.fine && pl.sgs) {
    sgs_subdomains<<<h->sgs->nsd, kSgsThreads, 0, st>>>(h->sgs->view, h->sgs->sd_ptr.p, pl.sgs_iters, a.v.r,
                                                         h->sgs->x.p);
    xl_fine = h->sgs->x.p;
    nl++;
  } else if (pl.fine) {
    if (pl.mixed) {
      MfDevice<float> *d = h->sub32.get();
      float *xl = K > 1 ? d->xlm.p : d->xl.p;
      gather_subdomains<float><<<grid, kVecThreads, 0, st>>>(a.v.r, d->gidx.p, xl, d->xlen, K, vs);
      nl += 1 + d->solve(st, K, h->status.p);
      xl_fine = xl;
      xls = K > 1 ? d->xlen : 0;
    } else {
      MfDevice<double> *d = h->sub64.get();
      double *xl = K > 1 ? d->xlm.p : d->xl.p;
      gather_subdomains<double><<<grid, kVecThreads, 0, st>>>(a.v.r, d->gidx.p, xl, d->xlen, K, vs);
      nl += 1 + d->solve(st, K, h->status.p);
      xl_fine = xl;
      xls = K > 1 ? d->xlen : 0;
    }
  }
  if (profile) CK(cudaEventRecord(h->ev[8], st));
  if (pl.coarse) CK(cudaStreamWaitEvent(st, h->join_ev, 0));
  const double *xc = xc_buf;
  const int64_t xcs = (pl.coarse && K > 1) ? co->xlen : 0;
  if (pl.sgs && pl.mixed)
    pull_prolong_dot<double, float><<<a.pg, kVecThreads, 0, st>>>(
        n, h->pull_ptr.p, h->pull_idx.p, (const double *)xl_fine, h->Pp.p, h->Pc.p, h->Pvf.p, xc,
        pl.mode, a.v.r, a.v.z, a.v.zold, a.part_rz, a.part_rzo, a.cb, a.csys, vs, xls, xcs);
  else if (pl.sgs)
    pull_prolong_dot<double, double><<<a.pg, kVecThreads, 0, st>>>(
        n, h->pull_ptr.p, h->pull_idx.p, (const double *)xl_fine, h->Pp.p, h->Pc.p, h->Pv.p, xc,
        pl.mode, a.v.r, a.v.z, a.v.zold, a.part_rz, a.part_rzo, a.cb, a.csys, vs, xls, xcs);
  else if (pl.mixed)
    pull_prolong_dot<float, float><<<a.pg, kVecThreads, 0, st>>>(
        n, h->pull_ptr.p, h->pull_idx.p, (const float *)xl_fine, h->Pp.p, h->Pc.p, h->Pvf.p, xc,
        pl.mode, a.v.r, a.v.z, a.v.zold, a.part_rz, a.part_rzo, a.cb, a.csys, vs, xls, xcs);
  else
    pull_prolong_dot<double, double><<<a.pg, kVecThreads, 0, st>>>(
        n, h->pull_ptr.p, h->pull_idx.p, (const double *)xl_fine, h->Pp.p, h->Pc.p, h->Pv.p, xc,
        pl.mode, a.v.r, a.v.z, a.v.zold, a.part_rz, a.part_rzo, a.cb, a.csys, vs, xls, xcs);
  return nl + 1;
}

// Stacked solves: the independent systems of a batch (c = h->bt) or K
// right-hand sides of one matrix (c = h->mr, nrhs = K).  Every system /
// right-hand side runs its own pcg_weigs (pcg.F90:289-462) with its own
// scalars and stopping test; the factorisations, preconditioner applications
// and products share the launches.  A system that stops is frozen (its rows
// are skipped by the direction, product and update kernels).  d_b, d_x: the
// stacked vectors (length ntot).
dg_status do_solve_stacked(dg_handle *h, BatchCtx &bc, const Vecs &V, int nrhs, int64_t ntot, const double *d_b,
                           double *d_x, dg_stats *st, cudaStream_t s) {
  Controls c = h->ctl;
  ctl_finish(c);
  const int n = h->n, K = bc.nsys, nch = bc.nchunks;
  const SolvePlan pl = plan_of(h, c);
  const int mixed = pl.mixed ? 1 : 0;
  const double tol = c.solve_tolerance, tol2 = tol * tol;
  const int maxit = c.solve_maxiters == -1 ? 100000 : c.solve_maxiters;
  int launches = 0;
  dg_stats out{};
  out.n = n;
  out.nsubdomains = (int)h->S.sd_ptr.size() - 1;
  out.ncoarse = h->S.AC.nrows;
  out.factor_nnz = h->Bsub.factor_nnz;
  out.factor_gflop = h->Bsub.factor_flops * 1e-9;
  out.t_setup_s = h->t_setup;
  StackArgs sa;
  sa.v = V;
  sa.part_rz = bc.part_rz.p;
  sa.part_rzo = bc.part_rzo.p;
  sa.pg = nch;
  sa.cb = bc.cb.p;
  sa.csys = nrhs > 1 ? bc.csys.p : nullptr;
  sa.nrhs = nrhs;
  try {
    const double t0 = wall();
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
    CK(cudaEventRecord(h->ev[0], s));
    if (!(c.reuse_factors && h->factored)) {
      SolvePlan fp = pl;
      fp.fine = pl.fine && !pl.sgs;
      launches += factor_all(h, fp, s);
    }
    CK(cudaEventRecord(h->ev[1], s));
    CK(cudaMemcpyAsync(V.b, d_b, (size_t)ntot * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(V.x, 0, (size_t)ntot * sizeof(double), s));
    CK(cudaMemsetAsync(V.p, 0, (size_t)ntot * sizeof(double), s));
    CK(cudaMemsetAsync(V.zold, 0, (size_t)ntot * sizeof(double), s));
    bt_any(s, h, bc, V, 1, -1, V.r);  // r = b - A x0 for every system
    bt_step(bc, s, BT_INIT, 0, mixed, tol2, bc.part_rr.p, nullptr);
    launches += 2;
    CK(cudaGetLastError());
    int stv = 0;
    CK(cudaMemcpyAsync(&stv, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (stv & ERR_NOT_SPD) {
      h->factored = false;
      return fail(h, DG_SINGULAR, "a subdomain or coarse matrix is not positive definite");
    }
    h->factored = true;
    const bool prof = c.profile != 0;
    double t_sub = 0, t_co = 0, t_sp = 0;
    auto lap = [&](int a, int b) -> double {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, h->ev[a], h->ev[b]));
      return ms * 1e-3;
    };
    auto iteration = [&](cudaStream_t q, int first, bool replace, bool profile) -> int {
      int nl = precondition(h, pl, q, profile, sa);
      bt_step(bc, q, BT_RHO, first, mixed, tol2, bc.part_rz.p, bc.part_rzo.p);
      if (profile) CK(cudaEventRecord(h->ev[6], q));
      bt_direction<<<nch, kVecThreads, 0, q>>>(bc.cb.p, bc.csys.p, bc.state.p, bc.bsc.p, V.z, V.p, first);
      bt_any(q, h, bc, V, 0);
      if (profile) CK(cudaEventRecord(h->ev[7], q));
      bt_step(bc, q, BT_ALPHA, first, mixed, tol2, bc.part_pq.p, nullptr);
      bt_update<<<nch, kVecThreads, 0, q>>>(bc.cb.p, bc.csys.p, bc.state.p, bc.bsc.p, V.p, V.q, V.x, V.r,
                                            bc.part_rr.p);
      nl += 5;
      if (replace) {  // FP64 residual replacement, r = b - A x, of the iterating systems
        bt_any(q, h, bc, V, 1, BT_ACTIVE, V.r);
        nl++;
      }
      bt_step(bc, q, BT_FINISH, first, mixed, tol2, bc.part_rr.p, nullptr);
      return nl + 1;
    };
    if (!bc.exec) {
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(h->s3, cudaStreamCaptureModeThreadLocal));
      bc.exec_nodes = iteration(h->s3, 0, false, false);
      CK(cudaStreamEndCapture(h->s3, &g));
      CK(cudaGraphInstantiate(&bc.exec, g, 0));
      CK(cudaGraphDestroy(g));
    }
    std::vector<double> t_end(1, wall() - t0);
    int it = 0, active = K;
    while (active > 0 && it < maxit) {
      it++;
      const int first = it == 1;
      const bool replace = pl.mixed && c.replace_every > 0 && it % c.replace_every == 0;
      if (!first && !replace && !prof) {
        CK(cudaGraphLaunch(bc.exec, s));
        launches += bc.exec_nodes;
      } else {
        launches += iteration(s, first, replace, prof);
      }
      CK(cudaGetLastError());
      CK(cudaStreamSynchronize(s));
      if (prof) {
        t_sub += lap(3, 8);
        if (pl.coarse) t_co += lap(4, 5);
        t_sp += lap(6, 7);
      }
      if (bc.host_counts[1] > 0) {  // the FP64 true residual confirms the systems the recurrence stopped
        bt_any(s, h, bc, V, 1, BT_CHECK, V.r);
        bt_step(bc, s, BT_CONFIRM, 0, mixed, tol2, bc.part_rr.p, nullptr);
        launches += 2;
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
      }
      t_end.push_back(wall() - t0);
      active = bc.host_counts[0];
    }
    CK(cudaEventRecord(h->ev[2], s));
    // true residuals for the report (into q, which is free now)
    bt_any(s, h, bc, V, 1, -1, V.q);
    bt_step(bc, s, BT_REPORT, 0, mixed, tol2, bc.part_rr.p, nullptr);
    launches += 2;
    CK(cudaMemcpyAsync(d_x, V.x, (size_t)ntot * sizeof(double), cudaMemcpyDeviceToDevice, s));
    std::vector<double> bs((size_t)K * BS_N);
    h->sys_iters.assign((size_t)K, 0);
    h->sys_state.assign((size_t)K, 0);
    CK(cudaMemcpyAsync(bs.data(), bc.bsc.p, bs.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h->sys_iters.data(), bc.iters.p, (size_t)K * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h->sys_state.data(), bc.state.p, (size_t)K * sizeof(int), cudaMemcpyDeviceToHost, s));
    int stw = 0;
    CK(cudaMemcpyAsync(&stw, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (stw & ERR_WAIT) return fail(h, DG_CUDA_ERROR, "a dependency wait of the subdomain solve timed out");
    float ms_f = 0, ms_i = 0;
    CK(cudaEventElapsedTime(&ms_f, h->ev[0], h->ev[1]));
    CK(cudaEventElapsedTime(&ms_i, h->ev[1], h->ev[2]));
    h->sys_relres.assign((size_t)K, 0.0);
    h->sys_seconds.assign((size_t)K, 0.0);
    dg_status rc = DG_OK;
    double init_sum = 0, res_sum = 0, worst = 0;
    for (int k = 0; k < K; k++) {
      const double *sc = &bs[(size_t)k * BS_N];
      const double rel = std::sqrt(sc[BS_TRUE] / sc[BS_INIT]);
      h->sys_relres[(size_t)k] = rel;
      worst = std::max(worst, rel);
      init_sum += sc[BS_INIT];
      res_sum += sc[BS_RES];
      const int ik = std::min<int>(std::max(h->sys_iters[(size_t)k], 0), it);
      h->sys_seconds[(size_t)k] = t_end[(size_t)ik];
      const int stt = h->sys_state[(size_t)k];
      if (stt == BT_BREAKDOWN) {
        rc = DG_BREAKDOWN;
        h->err = "CG breakdown in system " + std::to_string(k + 1) + ": p.q <= 0 or NaN";
      } else if (stt != BT_DONE && rc == DG_OK) {
        rc = DG_NOT_CONVERGED;
      }
    }
    out.iterations = it;
    out.init_norm = std::sqrt(init_sum);
    out.final_norm = std::sqrt(res_sum);
    out.true_rel_residual = worst;
    out.cond_num = 0.0;
    out.t_subsolve_s = t_sub;
    out.t_coarse_s = t_co;
    out.t_spmv_s = t_sp;
    {
      const double tsz = pl.mixed ? 4.0 : 8.0;
      out.subsolve_bytes = 2.0 * (double)h->Bsub.factor_nnz * tsz;
      out.coarse_bytes = 2.0 * (double)h->Bco.factor_nnz * 8.0;
      out.spmv_bytes = 12.0 * (double)h->S.A.nnz() + 8.0 * (n + 1) + 8.0 * n * 5.0;
    }
    out.t_factor_s = ms_f * 1e-3;
    out.t_iterate_s = ms_i * 1e-3;
    out.t_total_s = out.t_factor_s + out.t_iterate_s;
    out.gpu_launches = launches;
    if (st) *st = out;
    return rc;
  } catch (const CudaError &e) {
    return cuda_fail(h, e);
  }
}

// K right-hand sides of the handle's matrix solved together: the stacked
// vectors (right-hand side k at k*n), per-right-hand-side CG scalars, one
// factorisation, every solve kernel over all K (the CTAs reading the same E
// are adjacent).
dg_status do_solve_multi(dg_handle *h, int K, const double *d_b, double *d_x, dg_stats *st, cudaStream_t s) {
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  if (h->nsys > 0) return fail(h, DG_BAD_INPUT, "several right-hand sides of batched systems: stack them as systems");
  if (K < 1) return fail(h, DG_BAD_INPUT, "number of right-hand sides must be >= 1");
  if ((int64_t)K * h->n >= (int64_t)INT_MAX) return fail(h, DG_BAD_INPUT, "too many right-hand sides for n");
  Controls c = h->ctl;
  ctl_finish(c);
  if (c.fine_method == 2) return fail(h, DG_BAD_INPUT, "several right-hand sides: fine_method 2 is not supported");
  if (h->elem_mv) return fail(h, DG_BAD_INPUT, "several right-hand sides: use the assembled products (elemental_matvec 0)");
  try {
    if (h->mr_k != K) {
      const int64_t nt = (int64_t)K * h->n;
      std::vector<int64_t> row((size_t)K + 1);
      for (int k = 0; k <= K; k++) row[(size_t)k] = (int64_t)k * h->n;
      h->mr.build(row, h->n);
      for (auto *v : {&h->mb, &h->mx, &h->mrr, &h->mp, &h->mq, &h->mz, &h->mzold}) v->alloc((size_t)nt);
      if (h->sub32) h->sub32->ensure_multi(K);
      if (h->sub64) h->sub64->ensure_multi(K);
      if (h->co64) h->co64->ensure_multi(K);
      h->mr_k = K;
    }
  } catch (const CudaError &e) {
    return cuda_fail(h, e);
  }
  const Vecs V{h->mb.p, h->mx.p, h->mrr.p, h->mp.p, h->mq.p, h->mz.p, h->mzold.p};
  return do_solve_stacked(h, h->mr, V, K, (int64_t)K * h->n, d_b, d_x, st, s);
}

// the solve: numeric factorisation + PCG (pcg_weigs, pcg.F90:289-462)
dg_status do_solve(dg_handle *h, const double *d_b, double *d_x, dg_stats *st, cudaStream_t s) {
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  if (h->nsys > 0) {
    const Vecs V{h->b.p, h->x.p, h->r.p, h->p.p, h->q.p, h->z.p, h->zold.p};
    return do_solve_stacked(h, h->bt, V, 1, h->n, d_b, d_x, st, s);
  }
  Controls c = h->ctl;
  ctl_finish(c);
  const int n = h->n;
  const int grid = kRedBlocks;
  const SolvePlan pl = plan_of(h, c);
  const bool fine = pl.fine, sgs = pl.sgs, coarse = pl.coarse, mixed = pl.mixed;
  int launches = 0;
  dg_stats out{};
  out.n = n;
  out.nsubdomains = (int)h->S.sd_ptr.size() - 1;
  out.ncoarse = h->S.AC.nrows;
  out.factor_nnz = h->Bsub.factor_nnz;
  out.factor_gflop = h->Bsub.factor_flops * 1e-9;
  out.t_setup_s = h->t_setup;
  try {
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), s));
    CK(cudaEventRecord(h->ev[0], s));
    const bool refactor = !(c.reuse_factors && h->factored);
    if (refactor) {
      SolvePlan fp = pl;
      fp.fine = pl.fine && !pl.sgs;
      launches += factor_all(h, fp, s);
    }
    CK(cudaEventRecord(h->ev[1], s));
    CK(cudaMemcpyAsync(h->b.p, d_b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(h->x.p, 0, (size_t)n * sizeof(double), s));
    CK(cudaMemsetAsync(h->p.p, 0, (size_t)n * sizeof(double), s));
    CK(cudaMemsetAsync(h->zold.p, 0, (size_t)n * sizeof(double), s));
    // r = b - A x0, init_norm = r.r
    resid_any(h->lanes, grid, s, h, h->x.p, h->b.p, h->r.p);
    cg_finish<<<1, 32, 0, s>>>(h->sc.p, h->part_rr.p, 1, h->d_host_out, h->status.p, h->d_host_status);
    launches += 2;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    if (*h->host_status & ERR_NOT_SPD) {
      h->factored = false;
      return fail(h, DG_SINGULAR, "a subdomain or coarse matrix is not positive definite");
    }
    h->factored = true;
    double init = h->host_out[0];
    if (init == 0.0) {
      init = 1.0;
      double one = 1.0;
      CK(cudaMemcpy(h->sc.p + SC_INIT, &one, sizeof(double), cudaMemcpyHostToDevice));
    }
    out.init_norm = std::sqrt(init);
    const double tol = c.solve_tolerance;
    const int maxit = c.solve_maxiters == -1 ? 100000 : c.solve_maxiters;
    double ratio = 1.0, res = init;
    int it = 0;
    std::vector<double> alphas, betas;
    dg_status rc = DG_OK;
    const bool prof = c.profile != 0;
    double t_sub = 0, t_co = 0, t_sp = 0;
    auto lap = [&](int a, int b) -> double {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, h->ev[a], h->ev[b]));
      return ms * 1e-3;
    };
    // one PCG iteration's launches on stream st (coarse branch forked to s2);
    // returns the number of kernels
    auto iteration = [&](cudaStream_t st, int first, bool replace, bool profile) -> int {
      StackArgs sa;
      sa.v = Vecs{h->b.p, h->x.p, h->r.p, h->p.p, h->q.p, h->z.p, h->zold.p};
      sa.part_rz = h->part_rz.p;
      sa.part_rzo = h->part_rzo.p;
      sa.pg = h->pull_grid;
      int nl = precondition(h, pl, st, profile, sa);
      if (profile) CK(cudaEventRecord(h->ev[6], st));
      spmv_any(h->lanes, grid, st, h, first, mixed ? 1 : 0);
      if (profile) CK(cudaEventRecord(h->ev[7], st));
      cg_update<<<grid, kVecThreads, 0, st>>>(n, h->p.p, h->q.p, h->x.p, h->r.p, h->sc.p, h->part_pq.p,
                                              h->part_rr.p);
      nl += 4;
      if (replace) {  // FP64 residual replacement: r = b - A x
        resid_any(h->lanes, grid, st, h, h->x.p, h->b.p, h->r.p);
        nl++;
      }
      cg_finish<<<1, 32, 0, st>>>(h->sc.p, h->part_rr.p, 0, h->d_host_out, h->status.p, h->d_host_status);
      nl++;
      return nl;
    };
    // the steady-state iteration is captured once into a CUDA graph
    if (!h->iter_exec && c.profile == 0) {
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(h->s3, cudaStreamCaptureModeThreadLocal));
      h->iter_nodes = iteration(h->s3, 0, false, false);
      CK(cudaStreamEndCapture(h->s3, &g));
      CK(cudaGraphInstantiate(&h->iter_exec, g, 0));
      CK(cudaGraphDestroy(g));
    }
    while (ratio > tol * tol && it < maxit) {
      it++;
      const int first = it == 1;
      const bool replace = mixed && c.replace_every > 0 && it % c.replace_every == 0;
      if (!first && !replace && !prof && h->iter_exec) {
        CK(cudaGraphLaunch(h->iter_exec, s));
        launches += h->iter_nodes;
      } else {
        launches += iteration(s, first, replace, prof);
      }
      CK(cudaGetLastError());  // a failed launch must not pass as a converged step
      CK(cudaStreamSynchronize(s));
      if (*h->host_status & ERR_WAIT) return fail(h, DG_CUDA_ERROR, "a dependency wait of the subdomain solve timed out");
      if (prof) {
        t_sub += lap(3, 8);
        if (coarse) t_co += lap(4, 5);
        t_sp += lap(6, 7);
      }
      res = h->host_out[0];
      double alpha = h->host_out[2], beta = h->host_out[3], pq = h->host_out[5];
      alphas.push_back(alpha);
      betas.push_back(beta);
      if (!(pq > 0.0) || std::isnan(res)) { rc = DG_BREAKDOWN; h->err = "CG breakdown: p.q <= 0 or NaN"; break; }
      ratio = res / init;
      if (mixed && !(ratio > tol * tol)) {
        // confirm with the true FP64 residual before stopping
        resid_any(h->lanes, grid, s, h, h->x.p, h->b.p, h->r.p);
        cg_finish<<<1, 32, 0, s>>>(h->sc.p, h->part_rr.p, 0, h->d_host_out, h->status.p, h->d_host_status);
        launches += 2;
        CK(cudaStreamSynchronize(s));
        res = h->host_out[0];
        ratio = res / init;
      }
    }
    CK(cudaEventRecord(h->ev[2], s));
    if (rc == DG_OK && ratio > tol * tol && it >= maxit) rc = DG_NOT_CONVERGED;
    // true residual for the report (into q, which is free now)
    resid_any(h->lanes, grid, s, h, h->x.p, h->b.p, h->q.p);
    cg_finish<<<1, 32, 0, s>>>(h->sc.p, h->part_rr.p, 2, h->d_host_out, h->status.p, h->d_host_status);
    launches += 2;
    CK(cudaMemcpyAsync(d_x, h->x.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    float ms_f = 0, ms_i = 0;
    CK(cudaEventElapsedTime(&ms_f, h->ev[0], h->ev[1]));
    CK(cudaEventElapsedTime(&ms_i, h->ev[1], h->ev[2]));
    out.iterations = it;
    out.final_norm = std::sqrt(res);
    out.true_rel_residual = std::sqrt(h->host_out[0] / init);
    out.cond_num = tridiag_cond(alphas, betas);
    out.t_factor_s = ms_f * 1e-3;
    out.t_iterate_s = ms_i * 1e-3;
    out.t_total_s = out.t_factor_s + out.t_iterate_s;
    out.gpu_launches = launches;
    {
      const double tsz = mixed ? 4.0 : 8.0;
      out.subsolve_bytes = 2.0 * (double)h->Bsub.factor_nnz * tsz;
      out.coarse_bytes = 2.0 * (double)h->Bco.factor_nnz * 8.0;
      const double nnz = (double)h->S.A.nnz();
      // direction update (z, p read, p written) + SpMV (A, p read, q written)
      out.spmv_bytes = 12.0 * nnz + 8.0 * (n + 1) + 8.0 * n * 5.0;
      out.t_subsolve_s = t_sub;
      out.t_coarse_s = t_co;
      out.t_spmv_s = t_sp;
    }
    if (st) *st = out;
    return rc;
  } catch (const CudaError &e) {
    return cuda_fail(h, e);
  }
}

std::string dirname_of(const std::string &p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? "." : p.substr(0, k);
}
std::string resolve(const std::string &dir, const std::string &f) {
  if (f.empty() || f[0] == '/') return f;
  return dir + "/" + f;
}

}  // namespace

extern "C" {

dg_status dg_create(dg_handle **h) {
  if (!h) return DG_BAD_INPUT;
  *h = new (std::nothrow) dg_handle();
  return *h ? DG_OK : DG_BAD_INPUT;
}

void dg_destroy(dg_handle *h) { delete h; }

const char *dg_last_error(const dg_handle *h) { return h ? h->err.c_str() : "null handle"; }

dg_status dg_set_option(dg_handle *h, const char *name, const char *value) {
  if (!h || !name || !value) return DG_BAD_INPUT;
  std::string w1(name), w2(value), err;
  for (auto &ch : w1) ch = (char)tolower((unsigned char)ch);
  if (w1 == "precision") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "precision must be 0 or 1");
    h->ctl.precision = v;
    h->ready = false;  // the subdomain factors change precision: set up again
    return DG_OK;
  }
  if (w1 == "replace_every") {
    int v;
    if (!parse_i10(w2, v)) return fail(h, DG_BAD_INPUT, "bad replace_every");
    h->ctl.replace_every = v;
    return DG_OK;
  }
  if (w1 == "solve_pdl") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "solve_pdl must be 0 or 1");
    h->ctl.solve_pdl = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "factor_overlap") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "factor_overlap must be 0 or 1");
    h->ctl.factor_overlap = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "queue_wait_cycles" || w1 == "queue_skip_publish") {
    // failure tests of the dependency-driven schedule: a short wait limit and
    // a forward task whose done flag is never published
    long long v = 0;
    try {
      size_t used = 0;
      v = std::stoll(w2, &used);
      if (used != w2.size()) throw std::invalid_argument(w2);
    } catch (const std::exception &) {
      return fail(h, DG_BAD_INPUT, "bad " + w1);
    }
    if (w1 == "queue_wait_cycles") {
      if (v < 1) return fail(h, DG_BAD_INPUT, "queue_wait_cycles must be positive");
      h->ctl.queue_wait_cycles = v;
    } else {
      if (v < -1 || v > INT_MAX) return fail(h, DG_BAD_INPUT, "bad queue_skip_publish");
      h->ctl.queue_skip_publish = (int)v;
    }
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "super_panel") {
    int v;
    if (!parse_i10(w2, v) || v < 32 || v % 32 != 0 || v > 1024)
      return fail(h, DG_BAD_INPUT, "super_panel must be a multiple of 32 in [32, 1024]");
    h->ctl.super_panel = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "tensor_update") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "tensor_update must be 0 or 1");
    h->ctl.tensor_update = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "device_setup") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "device_setup must be 0 or 1");
    h->ctl.device_setup = v;
    h->S.n = 0;  // the host setup runs again
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "solve_schedule") {
    int v;
    if (!parse_i10(w2, v) || v < 0 || v > 1) return fail(h, DG_BAD_INPUT, "solve_schedule must be 0 or 1");
    h->ctl.solve_schedule = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "panel_rows" || w1 == "fwd_task_kb" || w1 == "lean_task_kb" || w1 == "thin_level_fronts") {
    int v;
    if (!parse_i10(w2, v) || v < (w1 == "thin_level_fronts" ? 0 : 1)) return fail(h, DG_BAD_INPUT, "bad " + w1);
    (w1 == "panel_rows" ? h->ctl.panel_rows : w1 == "fwd_task_kb" ? h->ctl.fwd_task_kb
     : w1 == "lean_task_kb" ? h->ctl.lean_task_kb : h->ctl.thin_level_fronts) = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "elemental_matvec") {
    int v;
    if (!parse_i10(w2, v)) return fail(h, DG_BAD_INPUT, "bad elemental_matvec");
    h->ctl.elemental_matvec = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "reuse_factors") {
    int v;
    if (!parse_i10(w2, v)) return fail(h, DG_BAD_INPUT, "bad reuse_factors");
    h->ctl.reuse_factors = v;
    return DG_OK;
  }
  if (w1 == "profile") {
    int v;
    if (!parse_i10(w2, v)) return fail(h, DG_BAD_INPUT, "bad profile");
    h->ctl.profile = v;
    return DG_OK;
  }
  if (w1 == "nd_leaf") {
    int v;
    if (!parse_i10(w2, v) || v < 2) return fail(h, DG_BAD_INPUT, "nd_leaf must be >= 2");
    h->ctl.nd_leaf = v;
    h->ready = false;
    return DG_OK;
  }
  if (w1 == "omega") {
    char *end = nullptr;
    double v = strtod(w2.c_str(), &end);
    if (*end || !(v > 0)) return fail(h, DG_BAD_INPUT, "bad omega");
    h->ctl.omega = v;
    return DG_OK;
  }
  if (!ctl_apply(h->ctl, w1, w2, err)) return fail(h, DG_BAD_INPUT, err);
  h->ready = false;
  return DG_OK;
}

// elemental input: assemble on the host (one process) and keep the result as
// the matrix and right-hand side of the handle
static dg_status set_elements(dg_handle *h, const ElementMesh &M) {
  int n = 0;
  std::vector<int> ii, jj, lg;
  std::vector<double> vv, b;
  assemble_elements(M, n, ii, jj, vv, b, lg);
  if (n <= 0 || vv.empty()) return fail(h, DG_BAD_INPUT, "elements: the assembled matrix is empty");
  dg_status s = dg_set_matrix_coo(h, n, (int)vv.size(), ii.data(), jj.data(), vv.data());
  if (s != DG_OK) return s;
  s = dg_set_rhs(h, b.data());
  if (s != DG_OK) return s;
  std::vector<int> gl((size_t)M.ngf + 1, -1);
  for (size_t l = 0; l < lg.size(); l++) gl[(size_t)lg[l]] = (int)l;
  h->el_eptr = M.eptr;
  h->el_local.resize(M.efree.size());
  for (size_t q = 0; q < M.efree.size(); q++) h->el_local[q] = gl[(size_t)M.efree[q]];
  h->el_off = M.emat_off;
  h->el_mat = M.emat;
  h->el_free = M.efree;
  h->el_lg = lg;
  h->el_ngf = M.ngf;
  h->have_elements = true;
  h->have_geometry = false;
  return DG_OK;
}

dg_status dg_load_ctl(dg_handle *h, const char *path) {
  if (!h || !path) return DG_BAD_INPUT;
  FILE *f = fopen(path, "rb");
  if (!f) return fail(h, DG_BAD_INPUT, std::string("Unable to open DOUG control file: ") + path);
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  fclose(f);
  std::string err;
  if (!ctl_parse_text(h->ctl, text, err)) return fail(h, DG_BAD_INPUT, err);
  h->ctl_dir = dirname_of(path);
  Controls &c = h->ctl;
  if (c.input_type == 1) {  // elemental input (Distribution.F90:62-64)
    ElementMesh M;
    if (!read_elemental(resolve(h->ctl_dir, c.info_file), resolve(h->ctl_dir, c.freedom_lists_file),
                        resolve(h->ctl_dir, c.elemmat_rhs_file), c.number_of_blocks, M, err))
      return fail(h, DG_BAD_INPUT, err);
    dg_status st = set_elements(h, M);
    if (st != DG_OK || c.coords_file.empty() || c.freemap_file.empty()) return st;
    // Mesh_readFileCoords / Mesh_readFileFreemap (Mesh.F90:470-520)
    NodeGeometry G;
    if (!read_geometry(resolve(h->ctl_dir, c.coords_file), resolve(h->ctl_dir, c.freemap_file), M.nsd, M.nnode,
                       M.ngf, G, err))
      return fail(h, DG_BAD_INPUT, err);
    h->geo = std::move(G);
    h->have_geometry = true;
    return DG_OK;
  }
  if (c.input_type == 3) {  // generated structured problem (Distribution.F90:67-70)
    int n = 0;
    std::vector<int> ii, jj;
    std::vector<double> vv, b;
    structured_laplace(c.grid_size, n, ii, jj, vv, b);
    dg_status st = dg_set_matrix_coo(h, n, (int)vv.size(), ii.data(), jj.data(), vv.data());
    if (st != DG_OK) return st;
    return dg_set_rhs(h, b.data());
  }
  if (c.input_type != 2)
    return fail(h, DG_BAD_INPUT, "input_type " + std::to_string(c.input_type) +
                                     ": elemental (1), assembled (2) and structured (3) input are supported");
  std::vector<int> ii, jj;
  std::vector<double> vv;
  int n = 0;
  if (!read_assembled(resolve(h->ctl_dir, c.assembled_mtx_file), c.assembled_mtx_format, n, ii, jj, vv, err))
    return fail(h, DG_BAD_INPUT, err);
  dg_status s = dg_set_matrix_coo(h, n, (int)vv.size(), ii.data(), jj.data(), vv.data());
  if (s != DG_OK) return s;
  if (!c.assembled_rhs_file.empty()) {
    std::vector<double> b;
    if (!read_vector(resolve(h->ctl_dir, c.assembled_rhs_file), c.assembled_rhs_format, n, b, err))
      return fail(h, DG_BAD_INPUT, err);
    return dg_set_rhs(h, b.data());
  }
  return DG_OK;
}

dg_status dg_set_matrix_coo(dg_handle *h, int n, int nnz, const int *rows, const int *cols, const double *vals) {
  if (!h || n <= 0 || nnz <= 0 || !rows || !cols || !vals) return DG_BAD_INPUT;
  h->have_elements = false;  // set_elements sets it again after this call
  h->nsys = 0;
  h->S.n = 0;
  h->n = n;
  h->ii.assign(rows, rows + nnz);
  h->jj.assign(cols, cols + nnz);
  h->vv.assign(vals, vals + nnz);
  h->have_matrix = true;
  h->ready = false;
  if (!h->have_rhs || (int)h->rhs.size() != n) { h->rhs.assign((size_t)n, 1.0); h->have_rhs = false; }
  return DG_OK;
}

dg_status dg_set_systems(dg_handle *h, int nsys, const int *n_sys, const long long *nnz_sys, const int *rows,
                         const int *cols, const double *vals, const double *b) {
  if (!h || nsys <= 0 || !n_sys || !nnz_sys || !rows || !cols || !vals) return DG_BAD_INPUT;
  std::vector<int64_t> sr(1, 0), stri(1, 0);
  for (int k = 0; k < nsys; k++) {
    if (n_sys[k] <= 0 || nnz_sys[k] <= 0)
      return fail(h, DG_BAD_INPUT, "system " + std::to_string(k + 1) + ": no unknowns or no entries");
    sr.push_back(sr.back() + n_sys[k]);
    stri.push_back(stri.back() + nnz_sys[k]);
  }
  if (sr.back() > INT_MAX / 2) return fail(h, DG_BAD_INPUT, "batched systems: too many unknowns in total");
  const size_t ntri = (size_t)stri.back();
  std::vector<int> ii(ntri), jj(ntri);
  for (int k = 0; k < nsys; k++)
    for (int64_t q = stri[(size_t)k]; q < stri[(size_t)k + 1]; q++) {
      const int a = rows[q], c = cols[q];
      if (a < 1 || a > n_sys[k] || c < 1 || c > n_sys[k])
        return fail(h, DG_BAD_INPUT, "system " + std::to_string(k + 1) + ": entry " +
                                         std::to_string(q - stri[(size_t)k] + 1) +
                                         " out of range (indices are 1-based within each system)");
      ii[(size_t)q] = a + (int)sr[(size_t)k];
      jj[(size_t)q] = c + (int)sr[(size_t)k];
    }
  h->have_elements = false;
  h->n = (int)sr.back();
  h->ii.swap(ii);
  h->jj.swap(jj);
  h->vv.assign(vals, vals + ntri);
  h->nsys = nsys;
  h->sys_row = sr;
  h->sys_tri = stri;
  h->S.n = 0;
  h->have_matrix = true;
  h->ready = false;
  if (b) { h->rhs.assign(b, b + h->n); h->have_rhs = true; }
  else { h->rhs.assign((size_t)h->n, 1.0); h->have_rhs = false; }
  return DG_OK;
}

dg_status dg_get_system_stats(const dg_handle *h, int *iterations, int *status, double *rel_residual,
                              double *seconds) {
  if (!h) return DG_BAD_INPUT;
  if (h->sys_iters.empty()) return DG_NOT_READY;
  for (int k = 0; k < (int)h->sys_iters.size(); k++) {
    const int stt = h->sys_state[(size_t)k];
    if (iterations) iterations[k] = h->sys_iters[(size_t)k];
    if (status) status[k] = stt == BT_DONE ? DG_OK : stt == BT_BREAKDOWN ? DG_BREAKDOWN : DG_NOT_CONVERGED;
    if (rel_residual) rel_residual[k] = h->sys_relres[(size_t)k];
    if (seconds) seconds[k] = h->sys_seconds[(size_t)k];
  }
  return DG_OK;
}

dg_status dg_set_elements(dg_handle *h, int nell, int ngf, const int *eptr, const int *efree,
                          const double *emat, const double *erhs) {
  if (!h || nell <= 0 || ngf <= 0 || !eptr || !efree || !emat || !erhs) return DG_BAD_INPUT;
  ElementMesh M;
  M.nell = nell;
  M.ngf = ngf;
  M.eptr.assign(eptr, eptr + nell + 1);
  if (M.eptr[0] != 0) return fail(h, DG_BAD_INPUT, "elements: eptr[0] must be 0");
  for (int e = 0; e < nell; e++)
    if (M.eptr[(size_t)e + 1] < M.eptr[(size_t)e]) return fail(h, DG_BAD_INPUT, "elements: freedom list offsets decrease");
  const int64_t nfree = M.eptr.back();
  M.efree.assign(efree, efree + nfree);
  M.erhs.assign(erhs, erhs + nfree);
  M.emat_off.assign(1, 0);
  for (int e = 0; e < nell; e++) {
    const int64_t nf = M.eptr[(size_t)e + 1] - M.eptr[(size_t)e];
    M.emat_off.push_back(M.emat_off.back() + nf * nf);
    M.mfrelt = std::max<int>(M.mfrelt, (int)nf);
  }
  M.emat.assign(emat, emat + M.emat_off.back());
  std::string err;
  if (!check_elements(M, err)) return fail(h, DG_BAD_INPUT, err);
  return set_elements(h, M);
}

dg_status dg_set_node_geometry(dg_handle *h, int nsd, int nnode, const double *coords, const int *freemap) {
  if (!h || nsd < 2 || nsd > 3 || nnode <= 0 || !coords || !freemap) return DG_BAD_INPUT;
  if (!h->have_elements) return fail(h, DG_NOT_READY, "node geometry: give the elements first");
  NodeGeometry G;
  G.nsd = nsd;
  G.nnode = nnode;
  G.coords.assign(coords, coords + (size_t)nsd * nnode);
  G.freemap.assign(freemap, freemap + h->el_ngf);
  for (int f = 0; f < h->el_ngf; f++)
    if (G.freemap[(size_t)f] < 1 || G.freemap[(size_t)f] > nnode)
      return fail(h, DG_BAD_INPUT, "freemap: freedom " + std::to_string(f + 1) + " maps to node " +
                                       std::to_string(G.freemap[(size_t)f]));
  h->geo = std::move(G);
  h->have_geometry = true;
  h->S.n = 0;
  h->ready = false;
  return DG_OK;
}

dg_status dg_get_coarse_coords(const dg_handle *h, int *nsd, int *ncoarse, double *xyz) {
  if (!h || h->S.coarse_xyz.empty() || !h->have_geometry) return DG_NOT_READY;
  const int d = h->geo.nsd;
  if (nsd) *nsd = d;
  if (ncoarse) *ncoarse = (int)(h->S.coarse_xyz.size() / (size_t)d);
  if (xyz) std::copy(h->S.coarse_xyz.begin(), h->S.coarse_xyz.end(), xyz);
  return DG_OK;
}

dg_status dg_set_rhs(dg_handle *h, const double *b) {
  if (!h || !b || h->n <= 0) return DG_BAD_INPUT;
  h->rhs.assign(b, b + h->n);
  h->have_rhs = true;
  return DG_OK;
}

dg_status dg_set_partition(dg_handle *h, const int *part, int nparts) {
  if (!h || !part || nparts <= 0 || h->n <= 0) return DG_BAD_INPUT;
  for (int i = 0; i < h->n; i++)
    if (part[i] < 1 || part[i] > nparts) return fail(h, DG_BAD_INPUT, "partition id out of range");
  h->part.assign(part, part + h->n);
  h->nparts = nparts;
  h->ready = false;
  return DG_OK;
}

dg_status dg_setup(dg_handle *h) {
  if (!h) return DG_BAD_INPUT;
  return do_setup(h);
}

dg_status dg_autotune(dg_handle *h, double *best_seconds, int *chosen) {
  if (!h) return DG_BAD_INPUT;
  if (!h->have_matrix) return fail(h, DG_NOT_READY, "no matrix: call dg_set_matrix_coo or dg_load_ctl first");
  // candidates: nested-dissection leaf x panel cutover x forward task size;
  // each is timed by a full solve (factorisations + PCG) of the stored rhs,
  // the host aggregation / restriction / coarse matrix are built once
  struct Cand { int leaf, panel_rows, fwd_kb, lean_kb; };
  const Cand cands[] = {{24, 512, 96, 80}, {16, 512, 96, 80}, {32, 512, 96, 80}, {24, 256, 96, 80},
                        {24, 512, 64, 48}, {24, 512, 160, 96}};
  const Controls keep = h->ctl;
  double best = 1e300;
  Cand pick = cands[0];
  bool host_ready = false;
  for (const Cand &cd : cands) {
    h->ctl = keep;
    h->ctl.nd_leaf = cd.leaf;
    h->ctl.panel_rows = cd.panel_rows;
    h->ctl.fwd_task_kb = cd.fwd_kb;
    h->ctl.lean_task_kb = cd.lean_kb;
    h->ready = false;
    dg_status st = do_setup(h, host_ready);
    if (st != DG_OK) { h->ctl = keep; return st; }
    host_ready = true;
    const size_t bytes = (size_t)h->n * sizeof(double);
    if (cudaMemcpy(h->hb.p, h->rhs.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(h, DG_CUDA_ERROR, "H2D copy failed");
    dg_stats ss{};
    double t = 0;
    for (int rep = 0; rep < 2; rep++) {  // the first solve also captures the iteration graph
      st = do_solve(h, h->hb.p, h->hx.p, &ss, 0);
      if (st != DG_OK && st != DG_NOT_CONVERGED) { h->ctl = keep; return st; }
      t = ss.t_total_s;
    }
    if (t < best) { best = t; pick = cd; }
  }
  h->ctl = keep;
  h->ctl.nd_leaf = pick.leaf;
  h->ctl.panel_rows = pick.panel_rows;
  h->ctl.fwd_task_kb = pick.fwd_kb;
  h->ctl.lean_task_kb = pick.lean_kb;
  h->ready = false;
  dg_status st = do_setup(h, true);
  if (best_seconds) *best_seconds = best;
  if (chosen) {
    chosen[0] = pick.leaf; chosen[1] = pick.panel_rows;
    chosen[2] = pick.fwd_kb; chosen[3] = pick.lean_kb;
  }
  return st;
}

dg_status dg_solve_multi(dg_handle *h, int nrhs, const double *b, double *x, dg_stats *stats) {
  if (!h || !x || nrhs < 1) return DG_BAD_INPUT;
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  const size_t bytes = (size_t)h->n * (size_t)nrhs * sizeof(double);
  double *db = nullptr, *dx = nullptr;
  if (cudaMalloc(&db, bytes) != cudaSuccess || cudaMalloc(&dx, bytes) != cudaSuccess) {
    cudaFree(db);
    return fail(h, DG_CUDA_ERROR, "device memory for the right-hand sides");
  }
  dg_status st = DG_OK;
  if (b) {
    if (cudaMemcpy(db, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess) st = fail(h, DG_CUDA_ERROR, "H2D copy failed");
  } else {
    for (int k = 0; k < nrhs && st == DG_OK; k++)
      if (cudaMemcpy(db + (size_t)k * h->n, h->rhs.data(), (size_t)h->n * sizeof(double), cudaMemcpyHostToDevice) !=
          cudaSuccess)
        st = fail(h, DG_CUDA_ERROR, "H2D copy failed");
  }
  if (st == DG_OK) st = do_solve_multi(h, nrhs, db, dx, stats, 0);
  if ((st == DG_OK || st == DG_NOT_CONVERGED) && cudaMemcpy(x, dx, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    st = fail(h, DG_CUDA_ERROR, "D2H copy failed");
  cudaFree(db);
  cudaFree(dx);
  return st;
}

dg_status dg_solve_multi_device(dg_handle *h, int nrhs, const double *d_b, double *d_x, dg_stats *stats,
                                void *stream) {
  if (!h || !d_b || !d_x) return DG_BAD_INPUT;
  return do_solve_multi(h, nrhs, d_b, d_x, stats, (cudaStream_t)stream);
}

dg_status dg_solve_device(dg_handle *h, const double *d_b, double *d_x, dg_stats *stats, void *stream) {
  if (!h || !d_b || !d_x) return DG_BAD_INPUT;
  return do_solve(h, d_b, d_x, stats, (cudaStream_t)stream);
}

dg_status dg_solve(dg_handle *h, const double *b, double *x, dg_stats *stats) {
  if (!h || !x) return DG_BAD_INPUT;
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  const double *src = b ? b : h->rhs.data();
  size_t bytes = (size_t)h->n * sizeof(double);
  // the handle's own device vectors (allocated by dg_setup) carry b and x
  if (cudaMemcpy(h->hb.p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    return fail(h, DG_CUDA_ERROR, "H2D copy failed");
  dg_status s = do_solve(h, h->hb.p, h->hx.p, stats, 0);
  if ((s == DG_OK || s == DG_NOT_CONVERGED) && cudaMemcpy(x, h->hx.p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    s = fail(h, DG_CUDA_ERROR, "D2H copy failed");
  return s;
}

dg_status dg_write_solution(dg_handle *h, const double *x) {
  if (!h || !x) return DG_BAD_INPUT;
  std::string err;
  if (h->ctl.solution_file.empty()) return fail(h, DG_BAD_INPUT, "no solution_file in the control words");
  if (!write_solution(resolve(h->ctl_dir, h->ctl.solution_file), h->ctl.solution_format, x, h->n, err))
    return fail(h, DG_BAD_INPUT, err);
  return DG_OK;
}

dg_status dg_get_setup_phases(const dg_handle *h, double *aggregation_s, double *coarse_s, int *on_device,
                              double *total_s) {
  if (!h) return DG_BAD_INPUT;
  if (h->S.n == 0) return DG_NOT_READY;
  if (aggregation_s) *aggregation_s = h->S.t_aggregation;
  if (coarse_s) *coarse_s = h->S.t_coarse;
  if (on_device) *on_device = h->S.coarse_on_device ? 1 : 0;
  if (total_s) *total_s = h->t_setup;
  return DG_OK;
}

dg_status dg_get_sizes(const dg_handle *h, int *n, int *nf, int *nc, int *nsd, long long *tot, int *rnnz, int *acnnz) {
  if (!h) return DG_BAD_INPUT;
  if (!h->ready && h->S.n == 0) return DG_NOT_READY;
  if (n) *n = h->n;
  if (nf) *nf = h->S.fine.nagr;
  if (nc) *nc = h->S.coarse.nagr;
  if (nsd) *nsd = (int)h->S.sd_ptr.size() - 1;
  if (tot) *tot = (long long)h->S.sd_nodes.size();
  if (rnnz) *rnnz = (int)h->S.R_i.size();
  if (acnnz) *acnnz = (int)h->S.AC_i.size();
  return DG_OK;
}

dg_status dg_get_aggregates(const dg_handle *h, int *fine_num, int *coarse_num) {
  if (!h || h->S.n == 0) return DG_NOT_READY;
  if (fine_num) std::copy(h->S.fine.num.begin(), h->S.fine.num.end(), fine_num);
  if (coarse_num) std::copy(h->S.coarse.num.begin(), h->S.coarse.num.end(), coarse_num);
  return DG_OK;
}

dg_status dg_get_subdomains(const dg_handle *h, long long *starts, int *nodes) {
  if (!h || h->S.n == 0) return DG_NOT_READY;
  if (starts) for (size_t q = 0; q < h->S.sd_ptr.size(); q++) starts[q] = h->S.sd_ptr[q];
  if (nodes) std::copy(h->S.sd_nodes.begin(), h->S.sd_nodes.end(), nodes);
  return DG_OK;
}

dg_status dg_get_restriction(const dg_handle *h, int *ri, int *rj, double *rv) {
  if (!h || h->S.n == 0) return DG_NOT_READY;
  if (ri) std::copy(h->S.R_i.begin(), h->S.R_i.end(), ri);
  if (rj) std::copy(h->S.R_j.begin(), h->S.R_j.end(), rj);
  if (rv) std::copy(h->S.R_v.begin(), h->S.R_v.end(), rv);
  return DG_OK;
}

dg_status dg_get_coarse_matrix(const dg_handle *h, int *ci, int *cj, double *cv) {
  if (!h || h->S.n == 0) return DG_NOT_READY;
  if (ci) std::copy(h->S.AC_i.begin(), h->S.AC_i.end(), ci);
  if (cj) std::copy(h->S.AC_j.begin(), h->S.AC_j.end(), cj);
  if (cv) std::copy(h->S.AC_v.begin(), h->S.AC_v.end(), cv);
  return DG_OK;
}

dg_status dg_grad_matrix(dg_handle *h, const double *d_lambda, const double *d_x, double *d_grad,
                         void *cuda_stream) {
  if (!h || !d_lambda || !d_x || !d_grad) return DG_BAD_INPUT;
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  const int64_t nnz = (int64_t)h->d_gi.n;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  grad_coo<<<(unsigned)std::min<int64_t>((nnz + 255) / 256, 65535), 256, 0, s>>>(nnz, h->d_gi.p, h->d_gj.p,
                                                                             d_lambda, d_x, d_grad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, DG_CUDA_ERROR, std::string("grad_coo: ") + cudaGetErrorString(e));
  return DG_OK;
}

dg_status dg_grad_elements(dg_handle *h, const double *d_lambda, const double *d_x, double *d_grad,
                           void *cuda_stream) {
  if (!h || !d_lambda || !d_x || !d_grad) return DG_BAD_INPUT;
  if (!h->ready) return fail(h, DG_NOT_READY, "dg_setup has not run");
  if (!h->have_elements) return fail(h, DG_BAD_INPUT, "the matrix was not given as elements");
  const int nell = (int)h->el_eptr.size() - 1;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  grad_elements<<<(nell + 7) / 8, 256, 0, s>>>(nell, h->d_el_eptr.p, h->d_el_local.p, h->d_el_off.p,
                                               h->d_el_mat.p, d_lambda, d_x, d_grad);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, DG_CUDA_ERROR, std::string("grad_elements: ") + cudaGetErrorString(e));
  return DG_OK;
}

dg_status dg_get_input(const dg_handle *h, int *n, int *nnz, int *rows, int *cols, double *vals, double *rhs) {
  if (!h) return DG_BAD_INPUT;
  if (!h->have_matrix) return DG_NOT_READY;
  if (n) *n = h->n;
  if (nnz) *nnz = (int)h->vv.size();
  if (rows) std::copy(h->ii.begin(), h->ii.end(), rows);
  if (cols) std::copy(h->jj.begin(), h->jj.end(), cols);
  if (vals) std::copy(h->vv.begin(), h->vv.end(), vals);
  if (rhs) std::copy(h->rhs.begin(), h->rhs.end(), rhs);
  return DG_OK;
}

}  // extern "C"
