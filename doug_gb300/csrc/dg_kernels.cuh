// sm_103a kernels of the GB300 solve path.
//
//   * batched multifrontal Cholesky (assembly + extend-add + partial
//     factorisation), one launch per assembly-tree level for all subdomains;
//   * multifrontal forward / backward solves, one launch per level;
//   * Schwarz gather and deterministic "pull" sum of subdomain solutions
//     (the reference adds subdomain solutions in subdomain order,
//     src/solvers/subsolvers.F90:68-73, then the coarse correction,
//     src/solvers/pcg.F90:191-193; the pull kernel adds in that same order);
//   * restriction / prolongation with R and P = R^T (src/solvers/pcg.F90:149,188);
//   * CSR SpMV fused with the CG direction update and the p.q partial sums;
//   * fused PCG vector updates with deterministic two-pass reductions.
//
// The level kernels wait only at hardware barriers (__syncthreads,
// __syncwarp, griddepcontrol.wait).  The optional dependency-driven solve
// schedule (mf_fwd_queue / mf_bwd_queue, option solve_schedule 1) polls the
// done flags of its producer tasks with clock64 + __nanosleep; every such
// wait is bounded, and on timeout it sets ERR_WAIT in the error word, skips
// the task's remaining waits and returns, and the host reports DG_CUDA_ERROR.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dg_tc.cuh"

namespace dg {

constexpr int kRedBlocks = 1024;   // partial-sum slots of every reduction
constexpr int kVecThreads = 256;

// device error word bits
enum : int { ERR_NOT_SPD = 1, ERR_NAN = 2, ERR_BREAKDOWN = 4, ERR_WAIT = 8 };

// one entry of a front's child list (child ci of f_children): the child's
// relative-row map offset, update-vector offset and update-row count, for
// the forward solves' right-hand-side assembly in one load
struct ChildEdge {
  int64_t relmap, uoff;
  int rc, pad;
};

// the front of a large-front solve task, stored beside the task so that the
// task's first E loads need one load of the task list only
struct __align__(16) TaskFront {
  int m, k;
  int64_t e_off;
};

struct MfView {  // device pointers of one multifrontal batch
  const int64_t *f_off;
  const int *f_m, *f_k;
  const int64_t *f_rows, *f_xoff;
  const int *f_p0;
  const int64_t *f_uoff, *f_woff;
  const int *f_child_ptr, *f_children;
  const int64_t *f_relmap, *f_asm;
  const int *rows, *relmap;
  const int64_t *asm_tgt, *asm_sp, *asm_src;
  const int64_t *e_off;        // offset of the front's elimination matrix E (m x k, ld round4(m))
  const ChildEdge *ch_edge;    // per child-list entry: see ChildEdge
};

__host__ __device__ __forceinline__ int round4(int x) { return (x + 3) & ~3; }

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// block sum in a fixed order (result valid in thread 0)
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    s = lane < NT / 32 ? sh[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

// sum of the kRedBlocks partials in a fixed order, by one warp; every lane
// of warp 0 gets the result
__device__ __forceinline__ double sum_partials(const double *part) {
  double s = 0.0;
  int lane = threadIdx.x & 31;
  for (int q = lane; q < kRedBlocks; q += 32) s += part[q];
  s = warp_sum(s);
  return __shfl_sync(0xffffffffu, s, 0);
}

// ---------------------------------------------------------------------------
// multifrontal numeric factorisation, one CTA per front of a level
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T tsqrt(T x);
template <>
__device__ __forceinline__ double tsqrt<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }

constexpr int kMfThreads = 256;
constexpr int kNB = 32;      // panel width
constexpr int kTile = 64;    // trailing-update tile (64 x 64 per CTA step, 4x4 per thread)

// Every factorisation kernel also produces the front's elimination matrix
//     E = [ L11^-1 ; -L21 L11^-1 ]     (m x k, column-major, ld = round4(m)),
// the partial forward elimination applied to the identity columns [I ; 0]:
// pivot j scales row j of E by 1/L(j,j) and subtracts L(i,j) times it from
// the rows i > j.  A forward solve of the front is then the product
// [y ; u] = E b1 + [0 ; b2] and a backward solve x1 = E^T [y ; x2]; neither
// has a dependency chain inside the front.  E needs L only while the panel
// that produced it is current, so the factor columns of the arena are dead
// once E is formed; the update (Schur complement) block stays in the arena
// for the parent's extend-add.

// Extend-add of column b of a child's update block into column pb of the
// parent (Dst = the parent's column base; row r of the column at
// Dst[r * stride]): rows a >= b, by the lanes of one warp.  kEaBatch rows
// per lane are loaded (child values, target rows, old target values) before
// any is stored, so a warp keeps many independent loads in flight; the
// targets of one child column are distinct.
constexpr int kEaBatch = 4;

template <typename T>
__device__ __forceinline__ void extend_add_column(T *__restrict__ Dst, const int *__restrict__ rel,
                                                  const T *__restrict__ Ucol, int b, int rc, int lane,
                                                  int stride = 1) {
  for (int a0 = b + lane; a0 < rc; a0 += 32 * kEaBatch) {
    int row[kEaBatch];
    T val[kEaBatch], old[kEaBatch];
#pragma unroll
    for (int u = 0; u < kEaBatch; u++) {
      const int a = a0 + 32 * u;
      row[u] = a < rc ? rel[a] * stride : 0;
      val[u] = a < rc ? Ucol[a] : T(0);
    }
#pragma unroll
    for (int u = 0; u < kEaBatch; u++)
      if (a0 + 32 * u < rc) old[u] = Dst[row[u]];
#pragma unroll
    for (int u = 0; u < kEaBatch; u++)
      if (a0 + 32 * u < rc) Dst[row[u]] = old[u] + val[u];
  }
}

// 16-byte vectors of T in shared memory
template <typename T> struct SVec;
template <> struct SVec<float> {
  static constexpr int N = 4;
  using V = float4;
  __device__ static __forceinline__ float get(const V &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
  __device__ static __forceinline__ void set(V &v, int q, float x) {
    if (q == 0) v.x = x; else if (q == 1) v.y = x; else if (q == 2) v.z = x; else v.w = x;
  }
};
template <> struct SVec<double> {
  static constexpr int N = 2;
  using V = double2;
  __device__ static __forceinline__ double get(const V &v, int q) { return q == 0 ? v.x : v.y; }
  __device__ static __forceinline__ void set(V &v, int q, double x) { if (q == 0) v.x = x; else v.y = x; }
};

// Row stride (elements) of the one-CTA kernel's panel and E in shared
// memory: whole 16-byte vectors, an odd number of them, so that the vectors
// of 8 consecutive rows fall into 8 different bank groups.
template <typename T> __host__ __device__ constexpr int pan_ld(int k) {
  const int vn = 16 / (int)sizeof(T);
  int nv = (k + vn - 1) / vn;
  if ((nv & 1) == 0) nv++;
  return nv * vn;
}
// shared memory of one front: panel and E (m x pan_ld(k) each), the
// multiplier row (pan_ld(k))
template <typename T> __host__ __device__ constexpr size_t pan_smem(int m, int k) {
  return ((size_t)2 * m + 1) * pan_ld<T>(k) * sizeof(T);
}

// Fronts whose pivot panel (m x k) and E (m x k) fit in shared memory: one
// CTA per front.  The pivot columns are assembled straight into shared
// memory, the update block in the arena; the panel is factored and E formed
// in shared memory, E is written out, and the update block receives
// -L21 L21^T in 4x4 register blocks.  Panel and E are row-major in shared
// memory (row i at i * pan_ld(k)): a thread updates its rows 16 bytes at a
// time against the broadcast multiplier row, and the update block reads
// 16-byte pieces of two rows per step.
constexpr int kPanThreads = 128;       // fronts of up to kPanWideRows rows
constexpr int kPanThreadsWide = 256;   // larger fronts
constexpr int kPanWideRows = 160;

template <typename T>
__global__ void __launch_bounds__(kPanThreadsWide)
mf_factor_panel(MfView v, const int *__restrict__ fronts, const double *__restrict__ vals,
                T *__restrict__ arena, T *__restrict__ E, int *__restrict__ status) {
  using SV = SVec<T>;
  using V = typename SV::V;
  constexpr int VN = SV::N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f], r = m - k;
  const int ldk = pan_ld<T>(k), nv = ldk / VN;
  T *P = reinterpret_cast<T *>(smem_raw);  // m x k panel, row-major, row stride ldk
  T *Es = P + (size_t)m * ldk;              // m x k elimination matrix, row-major
  T *lmul = Es + (size_t)m * ldk;           // step j: L(c, j) for j < c < k, zero elsewhere
  const int64_t off = v.f_off[f];
  T *F = arena + off;
  const int tid = threadIdx.x, nt = blockDim.x;
  // 1. zero: panel, E = [I ; 0] and the multiplier row in shared memory,
  //    update block in the arena
  for (int i = tid; i < m; i += nt) {
    V *pr = reinterpret_cast<V *>(P + (size_t)i * ldk);
    V *er = reinterpret_cast<V *>(Es + (size_t)i * ldk);
    for (int q = 0; q < nv; q++) {
      V z, e;
#pragma unroll
      for (int u = 0; u < VN; u++) {
        SV::set(z, u, T(0));
        SV::set(e, u, (q * VN + u == i && i < k) ? T(1) : T(0));
      }
      pr[q] = z;
      er[q] = e;
    }
  }
  for (int c = tid; c < ldk; c += nt) lmul[c] = T(0);
  for (int c = 0; c < r; c++)
    for (int i = c + tid; i < r; i += nt) F[(int64_t)(k + c) * m + k + i] = T(0);
  __syncthreads();
  // 2. original entries (each target once, duplicates summed in order)
  for (int64_t e = v.f_asm[f] + tid; e < v.f_asm[f + 1]; e += nt) {
    double sv = 0.0;
    for (int64_t q = v.asm_sp[e]; q < v.asm_sp[e + 1]; q++) sv += vals[v.asm_src[q]];
    const int64_t t = v.asm_tgt[e] - off;
    if (t < (int64_t)m * k) {
      const int col = (int)(t / m), row = (int)(t - (int64_t)col * m);
      P[(size_t)row * ldk + col] = (T)sv;
    } else {
      F[t] = (T)sv;
    }
  }
  __syncthreads();
  // 3. extend-add of the children's update matrices, children in order
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int mc = v.f_m[c], kc = v.f_k[c], rc = mc - kc;
    const T *U = arena + v.f_off[c] + (int64_t)kc * mc + kc;
    const int *rel = v.relmap + v.f_relmap[c];
    const int lane = tid & 31, wid = tid >> 5, nw = nt / 32;
    for (int b = wid; b < rc; b += nw) {
      const int col = rel[b];
      if (col < k) extend_add_column<T>(P + col, rel, U + (int64_t)b * mc, b, rc, lane, ldk);
      else extend_add_column<T>(F + (int64_t)col * m, rel, U + (int64_t)b * mc, b, rc, lane);
    }
    __syncthreads();
  }
  // 4. factor the panel and eliminate E.  Every thread takes the pivot from
  //    shared memory itself; the scaled column j goes to the multiplier row
  //    (panel rows) beside the panel.  A thread then updates each of its
  //    rows i > j 16 bytes at a time: panel columns (j, k) against the
  //    multiplier row, E columns [0, j] against E's row j.  Entries left of
  //    column j + 1 (panel) or right of column j (E) inside a vector keep
  //    their values; upper-triangle and padding entries of the panel are
  //    never read.  Each element receives the updates of the pivots in
  //    increasing order.
  for (int j = 0; j < k; j++) {
    T d = P[(size_t)j * ldk + j];
    if (!(d > T(0))) {
      if (tid == 0) atomicOr(status, ERR_NOT_SPD);
      d = T(1);
    }
    const T p = tsqrt<T>(d);
    for (int i = j + 1 + tid; i < m; i += nt) {
      const T x = P[(size_t)i * ldk + j] / p;
      P[(size_t)i * ldk + j] = x;
      if (i < k) lmul[i] = x;
    }
    for (int c = tid; c <= j; c += nt) Es[(size_t)j * ldk + c] /= p;
    if (tid == 0) lmul[j] = T(0);  // held L(j, j-1); column j is no multiplier of step j
    __syncthreads();
    if (tid == 0) P[(size_t)j * ldk + j] = p;  // read by no thread before the next step
    const V *lm = reinterpret_cast<const V *>(lmul);
    const V *ej = reinterpret_cast<const V *>(Es + (size_t)j * ldk);
    const int qp0 = (j + 1) / VN, qp1 = (k + VN - 1) / VN, qe1 = j / VN;
    for (int i = j + 1 + tid; i < m; i += nt) {
      const T lij = P[(size_t)i * ldk + j];
      V *pr = reinterpret_cast<V *>(P + (size_t)i * ldk);
      V *er = reinterpret_cast<V *>(Es + (size_t)i * ldk);
      for (int q = qp0; q < qp1; q++) {
        const V a = pr[q], b = lm[q];
        V o;
#pragma unroll
        for (int u = 0; u < VN; u++) {
          const T nvl = SV::get(a, u) - lij * SV::get(b, u);
          SV::set(o, u, q * VN + u > j ? nvl : SV::get(a, u));
        }
        pr[q] = o;
      }
      for (int q = 0; q <= qe1; q++) {
        const V a = er[q], b = ej[q];
        V o;
#pragma unroll
        for (int u = 0; u < VN; u++) {
          const T nvl = SV::get(a, u) - lij * SV::get(b, u);
          SV::set(o, u, q * VN + u <= j ? nvl : SV::get(a, u));
        }
        er[q] = o;
      }
    }
    __syncthreads();
  }
  // 5. E -> global (column-major, ld round4(m)); the padding rows stay zero
  {
    const int ld = round4(m);
    T *Eg = E + v.e_off[f];
    for (int c = 0; c < k; c++)
      for (int i = tid; i < m; i += nt) Eg[(int64_t)c * ld + i] = Es[(size_t)i * ldk + c];
  }
  // 6. update block: F[k:m, k:m] -= L21 L21^T (lower), 4x4 blocks per thread;
  //    L21 rows read VN columns at a time (padding columns are zero)
  const int nb4 = (r + 3) / 4;
  for (int q = tid; q < nb4 * nb4; q += nt) {
    const int bi = q % nb4, bc = q / nb4;
    if (bi < bc) continue;
    const int i0 = k + 4 * bi, c0 = k + 4 * bc;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int b = 0; b < 4; b++) acc[a][b] = T(0);
    const V *li[4], *lc[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      li[a] = reinterpret_cast<const V *>(P + (size_t)min(i0 + a, m - 1) * ldk);
      lc[a] = reinterpret_cast<const V *>(P + (size_t)min(c0 + a, m - 1) * ldk);
    }
    const int qk = (k + VN - 1) / VN;
    for (int qq = 0; qq < qk; qq++) {
      V xi[4], xc[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        xi[a] = li[a][qq];
        xc[a] = lc[a][qq];
      }
#pragma unroll
      for (int u = 0; u < VN; u++) {
        if (qq * VN + u < k) {
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] += SV::get(xi[a], u) * SV::get(xc[b], u);
        }
      }
    }
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int col = c0 + b;
      if (col >= m) continue;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int row = i0 + a;
        if (row < m && row >= col) F[(int64_t)col * m + row] -= acc[a][b];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// large fronts: assembly by column chunks, then for every panel step one
// launch that factors the panels and one that applies the trailing update
// tile by tile, so that one front occupies many SMs.
// ---------------------------------------------------------------------------
constexpr int kAsmCols = 64;

__device__ __forceinline__ int64_t lower_bound64(const int64_t *a, int64_t lo, int64_t hi, int64_t key) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int lower_bound32(const int *a, int lo, int hi, int key) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Right-looking Cholesky of the lower triangle of D[0..jb)[0..jb) by one
// warp: lane i keeps row i in registers, column j of L is broadcast by
// shuffles.  Per element the same operations in the same order as the
// column-by-column algorithm (scale by the pivot's square root, then
// D[i][c] -= D[i][j] D[c][j] for j = 0, 1, ...).
template <typename T>
__device__ __forceinline__ void chol_warp(T (*D)[kNB + 1], int jb, int *status) {
  const int lane = threadIdx.x & 31;
  T a[kNB];
#pragma unroll
  for (int c = 0; c < kNB; c++) a[c] = D[lane][c];
#pragma unroll
  for (int j = 0; j < kNB; j++) {
    if (j < jb) {
      T d = __shfl_sync(0xffffffffu, a[j], j);
      if (!(d > T(0))) {
        if (lane == 0) atomicOr(status, ERR_NOT_SPD);
        d = T(1);
      }
      const T p = tsqrt<T>(d);
      if (lane == j) a[j] = p;
      else if (lane > j) a[j] /= p;
      const T lij = a[j];
#pragma unroll
      for (int c = j + 1; c < kNB; c++) {
        const T lcj = __shfl_sync(0xffffffffu, lij, c);
        if (c < jb && lane >= c) a[c] -= lij * lcj;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < kNB; c++) D[lane][c] = a[c];
}

// The same right-looking Cholesky by a whole CTA in shared memory, one
// pivot per step: for FP64, whose square roots and divisions are too slow
// for one warp's chain on the FP64 pipe
template <typename T>
__device__ __forceinline__ void chol_cta(T (*D)[kNB + 1], int jb, int *status) {
  const int tid = threadIdx.x;
  for (int j = 0; j < jb; j++) {
    if (tid == 0) {
      T d = D[j][j];
      if (!(d > T(0))) { atomicOr(status, ERR_NOT_SPD); d = T(1); }
      D[j][j] = tsqrt<T>(d);
    }
    __syncthreads();
    const T p = D[j][j];
    for (int i = j + 1 + tid; i < jb; i += blockDim.x) D[i][j] /= p;
    __syncthreads();
    const int w = jb - j - 1;
    for (int q = tid; q < w * w; q += blockDim.x) {
      const int i = j + 1 + q / w, c = j + 1 + q % w;
      if (i >= c) D[i][c] -= D[i][j] * D[c][j];
    }
    __syncthreads();
  }
}

// FP32: one warp per front (chol_warp); FP64: kMfThreads per front (chol_cta)
template <typename T> __host__ __device__ constexpr int diag_threads() { return sizeof(T) == 4 ? 32 : kMfThreads; }

// Factor the jb x jb diagonal block at column j0 of a front in place (F: the
// front's arena block, ld m): its lower part into shared memory, FP32 by one
// warp in registers, FP64 by the whole CTA; every thread of the CTA calls it,
// after a barrier that makes the block's final values visible.
template <typename T>
__device__ __forceinline__ void factor_diag_block(T *__restrict__ F, int m, int j0, int jb, int *status) {
  __shared__ T D[kNB][kNB + 1];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int q = tid; q < kNB * kNB; q += nt) {  // lower part, zeros elsewhere
    const int c = q / kNB, i = q % kNB;  // column-major walk: coalesced over rows
    D[i][c] = (i >= c && i < jb) ? F[(int64_t)(j0 + c) * m + j0 + i] : T(0);
  }
  __syncthreads();
  if constexpr (sizeof(T) == 4) {
    if (tid < 32) chol_warp<T>(D, jb, status);
  } else {
    chol_cta<T>(D, jb, status);
  }
  __syncthreads();
  for (int q = tid; q < jb * jb; q += nt) {
    const int c = q / jb, i = q % jb;
    if (i >= c) F[(int64_t)(j0 + c) * m + j0 + i] = D[i][c];
  }
}

// The diagonal block of a panel step in a launch of its own: only where no
// earlier kernel of the chain finishes the block (the first step of an FP32
// super-panel after the mma.sync trailing update, tensor_update 0)
template <typename T>
__global__ void __launch_bounds__(diag_threads<T>())
mf_diag(MfView v, const int *__restrict__ fronts, int j0, T *__restrict__ arena, int *__restrict__ status) {
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  factor_diag_block<T>(arena + v.f_off[f], m, j0, min(kNB, k - j0), status);
}

// task = {front, first column of the chunk}.  The CTA of chunk 0 then
// factors the front's first diagonal block (the first panel step's).
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_assemble_large(MfView v, const int2 *__restrict__ tasks, const double *__restrict__ vals,
                  T *__restrict__ arena, int *__restrict__ status) {
  const int f = tasks[blockIdx.x].x, c0 = tasks[blockIdx.x].y;
  const int m = v.f_m[f];
  const int c1 = min(c0 + kAsmCols, m);
  const int64_t off = v.f_off[f];
  T *F = arena + off;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = kMfThreads / 32;
  for (int c = c0 + wid; c < c1; c += nw)
    for (int i = c + lane; i < m; i += 32) F[(int64_t)c * m + i] = T(0);
  __syncthreads();
  const int64_t lo = lower_bound64(v.asm_tgt, v.f_asm[f], v.f_asm[f + 1], off + (int64_t)c0 * m);
  const int64_t hi = lower_bound64(v.asm_tgt, lo, v.f_asm[f + 1], off + (int64_t)c1 * m);
  for (int64_t e = lo + tid; e < hi; e += kMfThreads) {
    double s = 0.0;
    for (int64_t q = v.asm_sp[e]; q < v.asm_sp[e + 1]; q++) s += vals[v.asm_src[q]];
    arena[v.asm_tgt[e]] = (T)s;
  }
  __syncthreads();
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int mc = v.f_m[c], kc = v.f_k[c], rc = mc - kc;
    const T *U = arena + v.f_off[c] + (int64_t)kc * mc + kc;
    const int *rel = v.relmap + v.f_relmap[c];
    const int blo = lower_bound32(rel, 0, rc, c0), bhi = lower_bound32(rel, blo, rc, c1);
    for (int b = blo + wid; b < bhi; b += nw)
      extend_add_column<T>(F + (int64_t)rel[b] * m, rel, U + (int64_t)b * mc, b, rc, lane);
    __syncthreads();
  }
  if (c0 == 0) factor_diag_block<T>(F, m, 0, min(kNB, v.f_k[f]), status);
}

// Panel at column j0 of a large front: its diagonal block was factored by
// the kernel that finished it (factor_diag_block: the assembly, the previous
// step's update tile (0, 0) or the super-panel's trailing-update tile (0, 0));
// mf_panel solves L21 = A21 L11^-T for row chunks of kPanelRows rows (task =
// {front, first row of the chunk}), many CTAs per front, or forms E rows of
// the panel (escale tasks, below).
constexpr int kPanelRows = 256;

// E rows of the panel (escale task = {front, first column}): E_J <- L_JJ^-1 E_J
// on kEscCols columns of [0, j0 + jb); the columns of block J start as the
// identity, so block J of E becomes L_JJ^-1
template <typename T> struct EscCols { static constexpr int N = 1024 / sizeof(T); };

template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_panel(MfView v, const int2 *__restrict__ tasks, int npanel, const int2 *__restrict__ esc, int j0,
         T *__restrict__ arena, T *__restrict__ E) {
  __shared__ T D[kNB][kNB + 1];
  const bool escale = (int)blockIdx.x >= npanel;
  const int2 task = escale ? esc[blockIdx.x - npanel] : tasks[blockIdx.x];
  const int f = task.x;
  const int m = v.f_m[f], k = v.f_k[f];
  const int jb = min(kNB, k - j0);
  T *F = arena + v.f_off[f];
  const int tid = threadIdx.x;
  for (int q = tid; q < jb * jb; q += kMfThreads) {  // the factored diagonal block
    int c = q / jb, i = q % jb;
    D[i][c] = i >= c ? F[(int64_t)(j0 + c) * m + j0 + i] : T(0);
  }
  if (escale) {
    constexpr int NC = EscCols<T>::N;
    __shared__ T Eb[NC][kNB + 1];
    const int ld = round4(m);
    T *Eg = E + v.e_off[f];
    const int c0 = task.y, nc = min(NC, j0 + jb - c0);
    for (int q = tid; q < nc * kNB; q += kMfThreads) {
      const int cc = q / kNB, t = q % kNB, c = c0 + cc;
      T e = T(0);
      if (t < jb) e = c < j0 ? Eg[(int64_t)c * ld + j0 + t] : (c - j0 == t ? T(1) : T(0));
      Eb[cc][t] = e;
    }
    __syncthreads();
    for (int cc = tid; cc < nc; cc += kMfThreads) {
      for (int t = 0; t < jb; t++) {
        T s = Eb[cc][t];
        for (int q = 0; q < t; q++) s -= D[t][q] * Eb[cc][q];
        Eb[cc][t] = s / D[t][t];
      }
    }
    __syncthreads();
    for (int q = tid; q < nc * kNB; q += kMfThreads) {
      const int cc = q / kNB, t = q % kNB;
      if (t < jb) Eg[(int64_t)(c0 + cc) * ld + j0 + t] = Eb[cc][t];
    }
    return;
  }
  __syncthreads();
  const int r0 = task.y;
  const int rb = max(r0, j0 + jb), re = min(r0 + kPanelRows, m);
  // one row per thread (no row loop: the diagonal block is read inside the
  // solve instead of being held in registers across rows)
  static_assert(kPanelRows == kMfThreads, "a row chunk has one row per thread");
  const int i = rb + tid;
  if (i < re) {
    T x[kNB];
#pragma unroll
    for (int t = 0; t < kNB; t++) x[t] = t < jb ? F[(int64_t)(j0 + t) * m + i] : T(0);
#pragma unroll
    for (int t = 0; t < kNB; t++) {
      if (t < jb) {
        T s = x[t];
#pragma unroll
        for (int q = 0; q < t; q++) s -= x[q] * D[t][q];
        x[t] = s / D[t][t];
      }
    }
#pragma unroll
    for (int t = 0; t < kNB; t++)
      if (t < jb) F[(int64_t)(j0 + t) * m + i] = x[t];
  }
}

// One 64x64 tile of an update with the L columns [jl, jl + K), K = min(kw, k - jl).
// Trailing-update tiles (task = {front, (ti << 16) | tj}, ti >= tj) cover rows
// and columns from c0 = jl + K: C -= L[rows, J] L[cols, J]^T (lower part),
// only columns below cend = min(cend_base, k) when cend_base > 0 (the update
// inside a 128-column super-panel), all columns otherwise (the trailing update
// of the whole super-panel, K up to 128, staged 32 columns at a time).  For
// blockIdx.x >= nupd the tile belongs to the E update
// E[c0:m, 0:c0] -= L[c0:m, J] E_J (task = {front, (ti << 16) | tc}, columns
// from 0; J = [jl, c0)); the columns of block J are assigned, the earlier
// ones accumulated.  A panel step (cend_base > 0) updates the E rows below
// cend only, the rest of its super-panel; the super-panel's own launch
// (cend_base 0, J = the super-panel) updates the rows below it.
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_update(MfView v, const int2 *__restrict__ tasks, int nupd, const int2 *__restrict__ etasks, int jl, int kw,
          int cend_base, T *__restrict__ arena, T *__restrict__ E, int *__restrict__ status) {
  __shared__ T As[kNB][kTile];
  __shared__ T Bs[kNB][kTile + 1];
  const bool etile = (int)blockIdx.x >= nupd;
  const int2 task = etile ? etasks[blockIdx.x - nupd] : tasks[blockIdx.x];
  const int f = task.x;
  const int ti = task.y >> 16, tj = task.y & 0xffff;
  const int m = v.f_m[f], k = v.f_k[f];
  const int K = min(kw, k - jl);
  T *F = arena + v.f_off[f];
  const int c0 = jl + K;
  const int r0 = c0 + ti * kTile;
  const int cc0 = etile ? tj * kTile : c0 + tj * kTile;
  const int cend = cend_base > 0 ? min(cend_base, k) : m;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ld = round4(m);
  T *Eg = E + v.e_off[f];
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  for (int t0 = 0; t0 < K; t0 += kNB) {
    const int tb = min(kNB, K - t0);
    if (t0 > 0) __syncthreads();  // the previous chunk is consumed
    for (int q = tid; q < kNB * kTile; q += kMfThreads) {
      int t = q / kTile, r = q % kTile;
      As[t][r] = (t < tb && r0 + r < m) ? F[(int64_t)(jl + t0 + t) * m + r0 + r] : T(0);
    }
    if (etile) {
      for (int q = tid; q < kNB * kTile; q += kMfThreads) {
        const int r = q / kNB, t = q % kNB;
        Bs[t][r] = (t < tb && cc0 + r < c0) ? Eg[(int64_t)(cc0 + r) * ld + jl + t0 + t] : T(0);
      }
    } else {
      for (int q = tid; q < kNB * kTile; q += kMfThreads) {
        int t = q / kTile, r = q % kTile;
        Bs[t][r] = (t < tb && cc0 + r < cend) ? F[(int64_t)(jl + t0 + t) * m + cc0 + r] : T(0);
      }
    }
    __syncthreads();
    for (int t = 0; t < tb; t++) {
      T ra[4], rb[4];
#pragma unroll
      for (int a = 0; a < 4; a++) ra[a] = As[t][tx + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; b++) rb[b] = Bs[t][ty + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] += ra[a] * rb[b];
    }
  }
  const int j0 = jl;
  if (etile) {
    const int rend = cend_base > 0 ? cend : m;
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int col = cc0 + ty + 16 * b;
      if (col >= c0) continue;
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int row = r0 + tx + 16 * a;
        if (row >= rend) continue;
        T *dst = Eg + (int64_t)col * ld + row;
        *dst = col >= j0 ? -acc[a][b] : *dst - acc[a][b];
      }
    }
    return;
  }
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const int col = cc0 + ty + 16 * b;
    if (col >= cend) continue;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int row = r0 + tx + 16 * a;
      if (row < m && row >= col) F[(int64_t)col * m + row] -= acc[a][b];
    }
  }
  // tile (0, 0) holds the next panel step's diagonal block (columns c0 ..,
  // inside the super-panel for a panel step): this was its last update
  if (ti == 0 && tj == 0 && c0 < (cend_base > 0 ? min(cend_base, k) : k)) {
    __syncthreads();
    factor_diag_block<T>(F, m, c0, min(kNB, k - c0), status);
  }
}

// Trailing update of a super-panel with 128 x 128 tiles (FP32): C -= L_rows L_cols^T
// for the L columns [jl, jl + K), K = min(kw, k - jl), rows and columns from
// c0 = jl + K (task = {front, (ti << 16) | tj}, ti >= tj, 128-row units).
constexpr int kBT = 128, kBK = 8;

// It runs on the tensor cores (C -= L_I L_J^T, 128 x 128 per CTA, K walked
// in chunks of 8 columns, double-buffered in shared memory with the next
// chunk's global loads issued before the current chunk is consumed), each product as three TF32 products (split 3xTF32:
// a = a_hi + a_lo with a_hi, a_lo TF32; a b ~ a_lo b_hi + a_hi b_lo + a_hi b_hi,
// FP32 accumulation), which keeps the FP32 accuracy of the factorisation.
// 8 warps, warp w owns rows 64*(w%2) .. +63 and columns 32*(w/2) .. +31 of the
// tile: 4 x 4 mma.m16n8k8 tiles.  Operands are split when they are staged.
__device__ __forceinline__ uint32_t tf32_of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int kTcPad = kBT + 8;  // row stride of the staged operands (conflict-free fragment loads)

__global__ void __launch_bounds__(256, 2)
mf_update_big_tf32(MfView v, const int2 *__restrict__ tasks, int jl, int kw, float *__restrict__ arena) {
  __shared__ __align__(16) uint32_t Ah[2][kBK][kTcPad], Al[2][kBK][kTcPad];
  __shared__ __align__(16) uint32_t Bh[2][kBK][kTcPad], Bl[2][kBK][kTcPad];
  const int f = tasks[blockIdx.x].x;
  const int ti = tasks[blockIdx.x].y >> 16, tj = tasks[blockIdx.x].y & 0xffff;
  const int m = v.f_m[f], k = v.f_k[f];
  const int K = min(kw, k - jl);
  const int c0 = jl + K, r0 = c0 + ti * kBT, cc0 = c0 + tj * kBT;
  float *F = arena + v.f_off[f];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int lt = tid >> 5, lr = (tid & 31) * 4;  // chunk column and first of 4 rows this thread stages
  const int wm = (warp & 1) * 64, wn = (warp >> 1) * 32;
  const int gid = lane >> 2, tig = lane & 3;
  float pa[4], pb[4];
  auto fetch = [&](int kc) {
    const int t = kc + lt;
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int ra = r0 + lr + u, rb = cc0 + lr + u;
      pa[u] = (t < K && ra < m) ? F[(int64_t)(jl + t) * m + ra] : 0.f;
      pb[u] = (t < K && rb < m) ? F[(int64_t)(jl + t) * m + rb] : 0.f;
    }
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const uint32_t ah = tf32_of(pa[u]), bh = tf32_of(pb[u]);
      Ah[buf][lt][lr + u] = ah;
      Al[buf][lt][lr + u] = tf32_of(pa[u] - __uint_as_float(ah));
      Bh[buf][lt][lr + u] = bh;
      Bl[buf][lt][lr + u] = tf32_of(pb[u] - __uint_as_float(bh));
    }
  };
  float acc[4][4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[a][b][q] = 0.f;
  fetch(0);
  stash(0);
  __syncthreads();
  int buf = 0;
  for (int kc = 0; kc < K; kc += kBK) {
    const bool more = kc + kBK < K;
    if (more) fetch(kc + kBK);
    // B fragments (hi and lo) of the warp's 4 column tiles
    uint32_t bh[4][2], bl[4][2];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      const int col = wn + nt * 8 + gid;
      bh[nt][0] = Bh[buf][tig][col];
      bh[nt][1] = Bh[buf][tig + 4][col];
      bl[nt][0] = Bl[buf][tig][col];
      bl[nt][1] = Bl[buf][tig + 4][col];
    }
#pragma unroll
    for (int mt = 0; mt < 4; mt++) {
      const int row = wm + mt * 16 + gid;
      const uint32_t ah[4] = {Ah[buf][tig][row], Ah[buf][tig][row + 8], Ah[buf][tig + 4][row],
                              Ah[buf][tig + 4][row + 8]};
      const uint32_t al[4] = {Al[buf][tig][row], Al[buf][tig][row + 8], Al[buf][tig + 4][row],
                              Al[buf][tig + 4][row + 8]};
#pragma unroll
      for (int nt = 0; nt < 4; nt++) {  // small terms first
        mma_tf32(acc[mt][nt], al, bh[nt]);
        mma_tf32(acc[mt][nt], ah, bl[nt]);
        mma_tf32(acc[mt][nt], ah, bh[nt]);
      }
    }
    if (more) stash(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int mt = 0; mt < 4; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int row = r0 + wm + mt * 16 + gid + (q >= 2 ? 8 : 0);
        const int col = cc0 + wn + nt * 8 + tig * 2 + (q & 1);
        if (row < m && col < m && row >= col) F[(int64_t)col * m + row] -= acc[mt][nt][q];
      }
}

// The same update on the fifth-generation tensor cores: tcgen05.mma
// kind::tf32 with the 128 x 128 FP32 accumulator in tensor memory.  The CTA
// (8 warps) stages K in chunks of 32 columns: every thread loads rows of the
// two column blocks of L (coalesced along the column), splits them into
// TF32 hi and lo parts and writes them into four 16 KB shared-memory tiles
// in the 128-byte-swizzled K-major layout (dg_tc.cuh); one thread issues the
// 3 x 4 MMAs of the chunk (lo*hi, hi*lo, hi*hi per K step of 8) and commits
// them to an mbarrier that all threads wait on (bounded: on a timeout the
// CTA sets ERR_WAIT, waits once more and frees its tensor memory) before
// the tiles are refilled.  The epilogue reads the accumulator back with
// tcgen05.ld (warp w: lanes 32 (w % 4) .., columns 64 (w / 4) ..) and
// subtracts it from the lower part of the front.  A diagonal tile (ti == tj)
// stages one block and uses it as both operands.
constexpr int kTcChunk = 32;
constexpr size_t kTcTileBytes = 128 * kTcChunk * sizeof(float);  // 16 KB
constexpr size_t kTcSmem = 4 * kTcTileBytes + 1024;                // + alignment to 1024 bytes
constexpr long long kTcWaitPolls = 1LL << 24;

__global__ void __launch_bounds__(256, 3)
mf_update_big_tc(MfView v, const int2 *__restrict__ tasks, int nupd, const int2 *__restrict__ etasks, int jl,
                 int kw, float *__restrict__ arena, float *__restrict__ E, int *__restrict__ status,
                 int fuse_diag) {
  extern __shared__ unsigned char tc_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) &
                                                          ~static_cast<uintptr_t>(1023));
  unsigned char *Ahi = base, *Alo = base + kTcTileBytes, *Bhi = base + 2 * kTcTileBytes,
                *Blo = base + 3 * kTcTileBytes;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const bool etile = (int)blockIdx.x >= nupd;
  const int2 task = etile ? etasks[blockIdx.x - nupd] : tasks[blockIdx.x];
  const int f = task.x;
  const int ti = task.y >> 16, tj = task.y & 0xffff;
  const int m = v.f_m[f], k = v.f_k[f];
  const int K = min(kw, k - jl);
  const int c0 = jl + K, r0 = c0 + ti * kBT, cc0 = etile ? tj * kBT : c0 + tj * kBT;
  const bool diag = !etile && ti == tj;
  float *F = arena + v.f_off[f];
  const int ld = round4(m);
  float *Eg = E + v.e_off[f];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 128);
  if (tid == 0) tc::mbar_init(&bar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = tc::idesc_tf32(128, 128);
  // this thread stages rows (tid & 127) and columns kk = (tid >> 7) + 2 q of
  // every chunk: 16 values of each operand, loaded together
  constexpr int NQ = 128 * kTcChunk / 256;
  const int r = tid & 127, kk0 = tid >> 7;
  const int ra = r0 + r, rb = cc0 + r;
  // E tiles: B row rr is E column cc0 + rr, 16 consecutive K values of it
  // (E rows jl + kc + te ..), read as four 16-byte vectors
  const int rr = tid >> 1, te = (tid & 1) * 16;
  const bool eok = etile && cc0 + rr < c0;
  float pa[NQ], pb[NQ];
  auto fetch = [&](int kc) {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const int t = kc + kk0 + 2 * q;
      pa[q] = (t < K && ra < m) ? F[(int64_t)(jl + t) * m + ra] : 0.f;
      if (!etile) pb[q] = (!diag && t < K && rb < m) ? F[(int64_t)(jl + t) * m + rb] : 0.f;
    }
    if (etile) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int t = kc + te + 4 * u;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (eok && t < K) x = *reinterpret_cast<const float4 *>(Eg + (int64_t)(cc0 + rr) * ld + jl + t);
        pb[4 * u] = x.x;
        pb[4 * u + 1] = t + 1 < K ? x.y : 0.f;
        pb[4 * u + 2] = t + 2 < K ? x.z : 0.f;
        pb[4 * u + 3] = t + 3 < K ? x.w : 0.f;
      }
    }
  };
  auto stash = [&]() {
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      const uint32_t off = tc::sw128_offset(r, kk0 + 2 * q);
      const uint32_t ah = tf32_of(pa[q]);
      *reinterpret_cast<uint32_t *>(Ahi + off) = ah;
      *reinterpret_cast<uint32_t *>(Alo + off) = tf32_of(pa[q] - __uint_as_float(ah));
      if (!diag && !etile) {
        const uint32_t bh = tf32_of(pb[q]);
        *reinterpret_cast<uint32_t *>(Bhi + off) = bh;
        *reinterpret_cast<uint32_t *>(Blo + off) = tf32_of(pb[q] - __uint_as_float(bh));
      }
    }
    if (etile) {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const uint32_t off = tc::sw128_offset(rr, te + 4 * u);  // 4 values in one 16-byte chunk
        uint4 h, l;
        h.x = tf32_of(pb[4 * u]);     l.x = tf32_of(pb[4 * u] - __uint_as_float(h.x));
        h.y = tf32_of(pb[4 * u + 1]); l.y = tf32_of(pb[4 * u + 1] - __uint_as_float(h.y));
        h.z = tf32_of(pb[4 * u + 2]); l.z = tf32_of(pb[4 * u + 2] - __uint_as_float(h.z));
        h.w = tf32_of(pb[4 * u + 3]); l.w = tf32_of(pb[4 * u + 3] - __uint_as_float(h.w));
        *reinterpret_cast<uint4 *>(Bhi + off) = h;
        *reinterpret_cast<uint4 *>(Blo + off) = l;
      }
    }
  };
  uint32_t parity = 0;
  bool bad = false;
  fetch(0);
  for (int kc = 0; kc < K; kc += kTcChunk) {
    stash();
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
      const uint64_t dAh = tc::sw128_desc(tc::smem_u32(Ahi)), dAl = tc::sw128_desc(tc::smem_u32(Alo));
      const uint64_t dBh = diag ? dAh : tc::sw128_desc(tc::smem_u32(Bhi));
      const uint64_t dBl = diag ? dAl : tc::sw128_desc(tc::smem_u32(Blo));
#pragma unroll
      for (int ks = 0; ks < kTcChunk / 8; ks++) {  // 8 TF32 values (32 bytes) per MMA
        const uint64_t o = (uint64_t)((ks * 32) >> 4);
        tc::mma_tf32(tmem, dAl + o, dBh + o, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
        tc::mma_tf32(tmem, dAh + o, dBl + o, idesc, 1u);
        tc::mma_tf32(tmem, dAh + o, dBh + o, idesc, 1u);
      }
      tc::mma_commit(tc::smem_u32(&bar));
    }
    // the next chunk's loads are in flight while the tensor cores work
    if (kc + kTcChunk < K) fetch(kc + kTcChunk);
    const bool ok = tc::mbar_wait(&bar, parity, kTcWaitPolls);
    parity ^= 1;
    if (__syncthreads_or(!ok)) { bad = true; break; }
  }
  if (bad) {
    if (tid == 0) atomicOr(status, ERR_WAIT);
    tc::mbar_wait(&bar, parity ^ 1, kTcWaitPolls);  // its MMAs in flight, once more (bounded)
  } else {
    tc::fence_after_sync();
    const int lg = warp & 3, ch = warp >> 2;
    const int row = r0 + 32 * lg + lane;
#pragma unroll 1
    for (int h = 0; h < 4; h++) {
      float d[16];
      tc::tmem_load16(tmem + ((uint32_t)(32 * lg) << 16) + (uint32_t)(ch * 64 + 16 * h), d);
      if (etile) {
        // E[row, col] for col < c0: the super-panel's own columns (>= jl)
        // are assigned, the earlier ones accumulated
        if (row < m) {
          const int colb = cc0 + ch * 64 + 16 * h;
          float cur[16];
#pragma unroll
          for (int c = 0; c < 16; c++) {
            const int col = colb + c;
            cur[c] = (col < jl) ? Eg[(int64_t)col * ld + row] : 0.f;
          }
#pragma unroll
          for (int c = 0; c < 16; c++) {
            const int col = colb + c;
            if (col < c0) Eg[(int64_t)col * ld + row] = cur[c] - d[c];
          }
        }
      } else if (row < m) {
        const int colb = cc0 + ch * 64 + 16 * h;
        float cur[16];
#pragma unroll
        for (int c = 0; c < 16; c++) {
          const int col = colb + c;
          cur[c] = (col < m && row >= col) ? F[(int64_t)col * m + row] : 0.f;
        }
#pragma unroll
        for (int c = 0; c < 16; c++) {
          const int col = colb + c;
          if (col < m && row >= col) F[(int64_t)col * m + row] = cur[c] - d[c];
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, 128);
  // trailing-update tile (0, 0) holds the next super-panel's first diagonal
  // block: this was its last update
  if (fuse_diag && !bad && !etile && ti == 0 && tj == 0 && c0 < k)
    factor_diag_block<float>(F, m, c0, min(kNB, k - c0), status);
}

// ---------------------------------------------------------------------------
// multifrontal solves with the elimination matrices E
//
// Forward, one level:  the front's right-hand side is b = [xl(pivots) ; 0]
// plus the children's update vectors (extend-add, children in order); then
//     y = E[0:k, :] b1   -> yl (pivots)      u = b2 + E[k:m, :] b1 -> uvec.
// Backward, one level: v = [yl(pivots) ; xl(ancestor rows)], x1 = E^T v -> xl.
// The forward writes y to a second local vector so that the CTAs of one front
// never overwrite the right-hand side another CTA still reads.
//
// E is read with 16-byte vector loads: ld = round4(m) and every E block starts
// on a multiple of 4 elements, and the padding rows m..ld-1 are zero.
// ---------------------------------------------------------------------------
template <typename T> struct Vec16;
template <> struct Vec16<float> {
  static constexpr int N = 4;
  __device__ static __forceinline__ void load(const float *p, float *o) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
  }
};
template <> struct Vec16<double> {
  static constexpr int N = 2;
  __device__ static __forceinline__ void load(const double *p, double *o) {
    const double2 t = __ldg(reinterpret_cast<const double2 *>(p));
    o[0] = t.x; o[1] = t.y;
  }
};

constexpr int kSolveSmall = 128;   // fronts of at most this many rows: one warp each
constexpr int kEThreads = 256;
constexpr int kELeanThreads = 128;
constexpr int kEUnroll = 8;        // independent E loads in flight per thread

// Small fronts are solved by groups of G lanes (G = 8, 16 or 32; 32 / G
// fronts per warp): a front of at most 4G rows, lane l of its group holding
// the rows VN*l + G*VN*p.  Levels put their small fronts into three buckets
// by size so that tiny fronts do not leave most of a warp idle.
constexpr int kSmallUnroll = 4;   // E columns per load batch of a small-front group
template <typename T> struct SmallMinBlocks { static constexpr int N = sizeof(T) == 8 ? 3 : 6; };

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane / G * G));
}

// E loads of one batch of kSmallUnroll columns [j0, j0 + kSmallUnroll) for the rows
// of one group lane; vectors wholly above the diagonal (r + VN <= j) are zero
template <typename T, int PASS, int G>
__device__ __forceinline__ void load_e_batch(const T *Ef, int ld, int m, int k, int sl, int j0,
                                             T (&e)[PASS][kSmallUnroll][Vec16<T>::N]) {
  constexpr int VN = Vec16<T>::N;
#pragma unroll
  for (int p = 0; p < PASS; p++) {
    const int r = VN * sl + G * VN * p;
#pragma unroll
    for (int u = 0; u < kSmallUnroll; u++) {
      const int j = j0 + u;
      if (r < m && j < k && r + VN > j) Vec16<T>::load(Ef + (int64_t)j * ld + r, e[p][u]);
      else {
#pragma unroll
        for (int q = 0; q < VN; q++) e[p][u][q] = T(0);
      }
    }
  }
}

// small fronts, forward: the first batch of E is loaded before the
// right-hand side is assembled.  cta: this CTA's index within its bucket.
// Programmatic dependent launch of the level solves.  pdl_trigger (at the
// start of a CTA) lets the next kernel of the stream start its CTAs once
// every CTA of this one has started; pdl_wait returns once the previous
// kernel has completed and its writes are visible.  The solve bodies issue
// their first loads of E (written by the factorisation, before any of these
// kernels) and only then wait, before they read a vector that the previous
// level wrote.  Without the launch attribute both instructions do nothing.
__device__ __forceinline__ void pdl_trigger() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}

template <typename T, int G>
__device__ __forceinline__ void fwd_small_body(const MfView &v, const int *__restrict__ fronts, int nf,
                                               const T *__restrict__ E, const T *__restrict__ xl,
                                               T *__restrict__ yl, T *__restrict__ uvec, int cta, T *wsh) {
  constexpr int VN = Vec16<T>::N, M = 4 * G, PASS = M / (G * VN), FPW = 32 / G;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int grp = lane / G, sl = lane % G;
  const unsigned gm = group_mask<G>(lane);
  const int gf = (cta * 8 + wid) * FPW + grp;
  if (gf >= nf) return;  // group-level work: no block barriers below
  T *w = wsh + (wid * FPW + grp) * M;
  const int f = fronts[gf];
  const int m = v.f_m[f], k = v.f_k[f], ld = round4(m);
  const int64_t xo = v.f_xoff[f] + v.f_p0[f];
  const T *Ef = E + v.e_off[f];
  T e[PASS][kSmallUnroll][VN];
  load_e_batch<T, PASS, G>(Ef, ld, m, k, sl, 0, e);
  // the child list is static: its first entry is read before the wait
  const int cb = v.f_child_ptr[f], ce = v.f_child_ptr[f + 1];
  ChildEdge ed = cb < ce ? v.ch_edge[cb] : ChildEdge{0, 0, 0, 0};
  pdl_wait();
  for (int i = sl; i < m; i += G) w[i] = i < k ? xl[xo + i] : T(0);
  __syncwarp(gm);
  for (int ci = cb; ci < ce; ci++) {
    if (ci > cb) ed = v.ch_edge[ci];
    const int *rel = v.relmap + ed.relmap;
    const T *u = uvec + ed.uoff;
    for (int a = sl; a < ed.rc; a += G) w[rel[a]] += __ldcg(u + a);
    __syncwarp(gm);
  }
  T acc[PASS][VN];
#pragma unroll
  for (int p = 0; p < PASS; p++)
#pragma unroll
    for (int q = 0; q < VN; q++) acc[p][q] = T(0);
  for (int j0 = 0; j0 < k; j0 += kSmallUnroll) {
    if (j0 > 0) load_e_batch<T, PASS, G>(Ef, ld, m, k, sl, j0, e);
#pragma unroll
    for (int u = 0; u < kSmallUnroll; u++) {
      const T bj = j0 + u < k ? w[j0 + u] : T(0);
#pragma unroll
      for (int p = 0; p < PASS; p++)
#pragma unroll
        for (int q = 0; q < VN; q++) acc[p][q] += e[p][u][q] * bj;
    }
  }
  T *uf = uvec + v.f_uoff[f];
#pragma unroll
  for (int p = 0; p < PASS; p++)
#pragma unroll
    for (int q = 0; q < VN; q++) {
      const int row = VN * sl + G * VN * p + q;
      if (row < k) yl[xo + row] = acc[p][q];
      else if (row < m) uf[row - k] = w[row] + acc[p][q];
    }
}

// small fronts, backward: the first batch of E is loaded before v is gathered
template <typename T, int G>
__device__ __forceinline__ void bwd_small_body(const MfView &v, const int *__restrict__ fronts, int nf,
                                               const T *__restrict__ E, const T *__restrict__ yl,
                                               T *__restrict__ xl, int cta, T *wsh) {
  constexpr int VN = Vec16<T>::N, M = 4 * G, PASS = M / (G * VN), FPW = 32 / G;
  static_assert(G >= kSmallUnroll, "a group stores one column sum per lane");
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int grp = lane / G, sl = lane % G;
  const unsigned gm = group_mask<G>(lane);
  const int gf = (cta * 8 + wid) * FPW + grp;
  if (gf >= nf) return;
  T *w = wsh + (wid * FPW + grp) * M;
  const int f = fronts[gf];
  const int m = v.f_m[f], k = v.f_k[f], ld = round4(m);
  const int64_t xo = v.f_xoff[f] + v.f_p0[f];
  const T *Ef = E + v.e_off[f];
  T e[PASS][kSmallUnroll][VN];
  load_e_batch<T, PASS, G>(Ef, ld, m, k, sl, 0, e);
  // the ancestor rows' positions are static: read before the wait (a lane
  // has at most 4 of the front's ld <= 4G rows)
  const int *rows = v.rows + v.f_rows[f];
  int rw[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int i = sl + q * G;
    rw[q] = (i >= k && i < m) ? rows[i] : 0;
  }
  pdl_wait();
  const T *xb = xl + v.f_xoff[f];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int i = sl + q * G;
    if (i < ld) w[i] = i < k ? yl[xo + i] : (i < m ? __ldcg(xb + rw[q]) : T(0));
  }
  __syncwarp(gm);
  T wr[PASS][VN];
#pragma unroll
  for (int p = 0; p < PASS; p++)
#pragma unroll
    for (int q = 0; q < VN; q++) {
      const int r = VN * sl + G * VN * p + q;
      wr[p][q] = r < ld ? w[r] : T(0);
    }
  // each column sum is reduced over the group; lane u of the batch keeps column u
  for (int c0 = 0; c0 < k; c0 += kSmallUnroll) {
    if (c0 > 0) load_e_batch<T, PASS, G>(Ef, ld, m, k, sl, c0, e);
    T s[kSmallUnroll];
#pragma unroll
    for (int u = 0; u < kSmallUnroll; u++) {
      s[u] = T(0);
#pragma unroll
      for (int p = 0; p < PASS; p++)
#pragma unroll
        for (int q = 0; q < VN; q++) s[u] += e[p][u][q] * wr[p][q];
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s[u] += __shfl_xor_sync(gm, s[u], o);
    }
    if (sl < kSmallUnroll && c0 + sl < k) {
      T out = s[0];
#pragma unroll
      for (int u = 1; u < kSmallUnroll; u++) if (sl == u) out = s[u];
      xl[xo + c0 + sl] = out;
    }
  }
}

// One launch per level for the three small-front buckets: the first
// nb.x CTAs take the fronts of <= 32 rows (8 lanes each), the next nb.y those
// of <= 64 rows (16 lanes), the rest those of <= 128 rows (32 lanes).
// fronts: the level's small fronts, bucket after bucket; cnt: bucket sizes.
struct SmallBuckets {
  int cnt0, cnt1, cnt2;   // fronts per bucket
  int nb0, nb1;           // CTAs of buckets 0 and 1
};


// Several right-hand sides (nrhs > 1): CTA x serves right-hand side x % nrhs
// of the work unit x / nrhs, so the CTAs that read the same E are adjacent;
// the vectors of right-hand side k start at k * xs (xl, yl) and k * us (u).
template <typename T>
__global__ void __launch_bounds__(256, SmallMinBlocks<T>::N)
mf_fwd_small(MfView v, const int *__restrict__ fronts, SmallBuckets sb, const T *__restrict__ E,
             const T *__restrict__ xl, T *__restrict__ yl, T *__restrict__ uvec, int nrhs = 1, int64_t xs = 0,
             int64_t us = 0) {
  __shared__ __align__(16) T wsh[8 * kSolveSmall];
  pdl_trigger();
  const int b = blockIdx.x / nrhs, rk = blockIdx.x % nrhs;
  xl += rk * xs;
  yl += rk * xs;
  uvec += rk * us;
  if (b < sb.nb0) fwd_small_body<T, 8>(v, fronts, sb.cnt0, E, xl, yl, uvec, b, wsh);
  else if (b < sb.nb0 + sb.nb1)
    fwd_small_body<T, 16>(v, fronts + sb.cnt0, sb.cnt1, E, xl, yl, uvec, b - sb.nb0, wsh);
  else
    fwd_small_body<T, 32>(v, fronts + sb.cnt0 + sb.cnt1, sb.cnt2, E, xl, yl, uvec, b - sb.nb0 - sb.nb1, wsh);
}

template <typename T>
__global__ void __launch_bounds__(256, SmallMinBlocks<T>::N)
mf_bwd_small(MfView v, const int *__restrict__ fronts, SmallBuckets sb, const T *__restrict__ E,
             const T *__restrict__ yl, T *__restrict__ xl, int nrhs = 1, int64_t xs = 0) {
  __shared__ __align__(16) T wsh[8 * kSolveSmall];
  pdl_trigger();
  const int b = blockIdx.x / nrhs, rk = blockIdx.x % nrhs;
  yl += rk * xs;
  xl += rk * xs;
  if (b < sb.nb0) bwd_small_body<T, 8>(v, fronts, sb.cnt0, E, yl, xl, b, wsh);
  else if (b < sb.nb0 + sb.nb1)
    bwd_small_body<T, 16>(v, fronts + sb.cnt0, sb.cnt1, E, yl, xl, b - sb.nb0, wsh);
  else
    bwd_small_body<T, 32>(v, fronts + sb.cnt0 + sb.cnt1, sb.cnt2, E, yl, xl, b - sb.nb0 - sb.nb1, wsh);
}

// large fronts, forward: task = {front, (first chunk << 16) | chunk count};
// a chunk is FwdRows<T>::N rows.  The CTA assembles the front's whole
// right-hand side b (m entries) once, then per chunk each warp takes every
// 8th column of E and each lane VN rows (one coalesced 512-byte row segment
// per warp and column); the 8 warp sums are added in a fixed order.
// Pivot-row chunks need the columns j < min(k, r0 + N) only, and a vector
// of rows wholly above the diagonal of E is zero and not loaded.
template <typename T> struct FwdRows { static constexpr int N = 32 * Vec16<T>::N; };

// the task body; b: shared memory for the front's right-hand side (m
// values), red: the warp sums of one chunk
template <typename T, int NT>
__device__ __forceinline__ void fwd_big_body(const MfView &v, int2 tk, TaskFront tf, const T *__restrict__ E,
                                             const T *__restrict__ xl, T *__restrict__ yl, T *__restrict__ uvec,
                                             T *b, T (*red)[FwdRows<T>::N]) {
  constexpr int VN = Vec16<T>::N, RC = FwdRows<T>::N, NW = NT / 32, UN = NT == kELeanThreads ? 4 : kEUnroll;
  const int f = tk.x;
  const int ch0 = tk.y >> 16, nch = tk.y & 0xffff;
  const int m = tf.m, k = tf.k, ld = round4(m);
  const int64_t xo = v.f_xoff[f] + v.f_p0[f];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const T *Ef = E + tf.e_off;
  // one batch: columns j + u*NW (u < UN) of the chunk's rows of this lane;
  // a vector wholly above E's diagonal (rb + VN <= column) is zero
  T e[UN][VN];
  auto load_batch = [&](int r0, int K, int j) {
    const int rb = r0 + lane * VN;
#pragma unroll
    for (int u = 0; u < UN; u++) {
      const int jj = j + u * NW;
      if (rb < m && jj < K && rb + VN > jj) Vec16<T>::load(Ef + (int64_t)jj * ld + rb, e[u]);
      else {
#pragma unroll
        for (int q = 0; q < VN; q++) e[u][q] = T(0);
      }
    }
  };
  auto chunk_cols = [&](int r0) { return r0 < k ? min(k, r0 + RC) : k; };
  load_batch(ch0 * RC, chunk_cols(ch0 * RC), wid);  // in flight while b is assembled
  // the child list is static: its first entry is read before the wait, and
  // each entry's successor while the entry is added
  const int cb = v.f_child_ptr[f], ce = v.f_child_ptr[f + 1];
  ChildEdge ed = cb < ce ? v.ch_edge[cb] : ChildEdge{0, 0, 0, 0};
  pdl_wait();
  for (int i = tid; i < m; i += NT) b[i] = i < k ? xl[xo + i] : T(0);
  __syncthreads();
  for (int ci = cb; ci < ce; ci++) {
    const ChildEdge nx = ci + 1 < ce ? v.ch_edge[ci + 1] : ed;
    const int *rel = v.relmap + ed.relmap;
    const T *u = uvec + ed.uoff;
    for (int a = tid; a < ed.rc; a += NT) b[rel[a]] += __ldcg(u + a);
    __syncthreads();
    ed = nx;
  }
  T *uf = uvec + v.f_uoff[f];
  for (int ch = ch0; ch < ch0 + nch; ch++) {
    const int r0 = ch * RC;
    const int K = chunk_cols(r0);
    T acc[VN];
#pragma unroll
    for (int q = 0; q < VN; q++) acc[q] = T(0);
    for (int j = wid; j < K; j += UN * NW) {
      if (j != wid) load_batch(r0, K, j);  // every chunk's first batch was loaded ahead
#pragma unroll
      for (int u = 0; u < UN; u++) {
        const int jj = j + u * NW;
        const T bj = jj < K ? b[jj] : T(0);  // b holds rows [0, m): columns past K are not read
#pragma unroll
        for (int q = 0; q < VN; q++) acc[q] += e[u][q] * bj;
      }
    }
    // the next chunk's first batch is in flight during this chunk's reduction
    if (ch + 1 < ch0 + nch) load_batch((ch + 1) * RC, chunk_cols((ch + 1) * RC), wid);
#pragma unroll
    for (int q = 0; q < VN; q++) red[wid][lane * VN + q] = acc[q];
    __syncthreads();
    for (int t = tid; t < RC; t += NT) {
      T s = T(0);
#pragma unroll
      for (int w = 0; w < NW; w++) s += red[w][t];
      const int row = r0 + t;
      if (row < k) yl[xo + row] = s;
      else if (row < m) uf[row - k] = b[row] + s;
    }
    __syncthreads();
  }
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT, NT == kELeanThreads ? 12 : 4)
mf_fwd_big(MfView v, const int2 *__restrict__ tasks, const TaskFront *__restrict__ tmeta, const T *__restrict__ E,
           const T *__restrict__ xl, T *__restrict__ yl, T *__restrict__ uvec, int nrhs = 1, int64_t xs = 0,
           int64_t us = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T red[NT / 32][FwdRows<T>::N];
  pdl_trigger();
  const int task = blockIdx.x / nrhs, rk = blockIdx.x % nrhs;
  fwd_big_body<T, NT>(v, tasks[task], tmeta[task], E, xl + rk * xs, yl + rk * xs, uvec + rk * us,
                      reinterpret_cast<T *>(smem_raw), red);
}

// large fronts, backward: task = {front, column block J}; x[32J .. 32J+31] from
// rows [32J, m) of E
template <typename T, int NT>
__device__ __forceinline__ void bwd_big_body(const MfView &v, int2 tk, TaskFront tf, const T *__restrict__ E,
                                             const T *__restrict__ yl, T *__restrict__ xl, T *w) {
  constexpr int VN = Vec16<T>::N, LPC = 32 / VN, NCS = NT / LPC, UN = NT == kELeanThreads ? 4 : kEUnroll;
  const int f = tk.x, J = tk.y;
  const int m = tf.m, k = tf.k, ld = round4(m);
  const int c0 = 32 * J, jb = min(32, k - c0);
  const int64_t xo = v.f_xoff[f] + v.f_p0[f];
  const T *xb = xl + v.f_xoff[f];
  const int *rows = v.rows + v.f_rows[f];
  const int tid = threadIdx.x;
  const int rq = tid % LPC, cs = tid / LPC;
  // one batch: rows i + 32u (u < UN) of column c for this lane; a vector
  // wholly above E's diagonal (i + VN <= c) is zero
  T e[UN][VN];
  auto load_batch = [&](int c, int i) {
    const T *Ec = E + tf.e_off + (int64_t)c * ld;
#pragma unroll
    for (int u = 0; u < UN; u++) {
      const int ii = i + u * 32;
      if (c - c0 < jb && ii < m && ii + VN > c) Vec16<T>::load(Ec + ii, e[u]);
      else {
#pragma unroll
        for (int q = 0; q < VN; q++) e[u][q] = T(0);
      }
    }
  };
  load_batch(c0 + cs, c0 + rq * VN);  // in flight while v is gathered
  // the ancestor rows' positions are static: the first kRowsAhead of this
  // thread are read before the wait
  constexpr int kRowsAhead = 4;
  int rw[kRowsAhead];
#pragma unroll
  for (int q = 0; q < kRowsAhead; q++) {
    const int i = c0 + tid + q * NT;
    rw[q] = (i >= k && i < m) ? rows[i] : 0;
  }
  pdl_wait();
#pragma unroll
  for (int q = 0; q < kRowsAhead; q++) {
    const int i = c0 + tid + q * NT;
    if (i < ld) w[i - c0] = i < k ? yl[xo + i] : (i < m ? __ldcg(xb + rw[q]) : T(0));
  }
  for (int i = c0 + tid + kRowsAhead * NT; i < ld; i += NT)
    w[i - c0] = i < k ? yl[xo + i] : (i < m ? __ldcg(xb + rows[i]) : T(0));
  __syncthreads();
  for (int cc = cs; cc < 32; cc += NCS) {  // uniform trip count: the shuffles below need whole groups
    const int c = c0 + cc;
    T s = T(0);
    if (cc < jb) {
      for (int i = c0 + rq * VN; i < m; i += UN * 32) {
        if (i != c0 + rq * VN) load_batch(c, i);  // every column's first batch was loaded ahead
#pragma unroll
        for (int u = 0; u < UN; u++) {
          const int ii = i + u * 32;  // w holds rows [c0, ld): rows past m are not read
          if (ii < m) {
#pragma unroll
            for (int q = 0; q < VN; q++) s += e[u][q] * w[ii + q - c0];
          }
        }
      }
    }
    // the next column's first batch is in flight during this column's reduction
    if (cc + NCS < 32) load_batch(c + NCS, c0 + rq * VN);
#pragma unroll
    for (int o = LPC / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (rq == 0 && cc < jb) xl[xo + c] = s;
  }
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT, NT == kELeanThreads ? 12 : 4)
mf_bwd_big(MfView v, const int2 *__restrict__ tasks, const TaskFront *__restrict__ tmeta, const T *__restrict__ E,
           const T *__restrict__ yl, T *__restrict__ xl, int nrhs = 1, int64_t xs = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pdl_trigger();
  const int task = blockIdx.x / nrhs, rk = blockIdx.x % nrhs;
  bwd_big_body<T, NT>(v, tasks[task], tmeta[task], E, yl + rk * xs, xl + rk * xs, reinterpret_cast<T *>(smem_raw));
}

// ---------------------------------------------------------------------------
// Dependency-driven solve (solve_schedule 1): one launch per direction.  The
// tasks of all levels form one list (forward: leaves first; backward: roots
// first; the level kernels' tasks and small-front CTAs, unchanged); a CTA
// takes the next task with an atomic counter, waits until the tasks that
// produce its fronts' inputs have published their done flags (forward: the
// children's tasks, backward: the parent's), runs the task and publishes its
// own flag.  A task's dependencies come earlier in the list, so they were
// taken by CTAs that were running when they took them: no CTA waits on work
// that has not started, whether or not all CTAs are resident.  The waits are
// bounded (kQueueWaitCycles); on a timeout the CTA records ERR_WAIT and goes
// on, and the host reports the error.  Data written by other CTAs of the same
// launch (update vectors, ancestors' solutions) is read past L1 (__ldcg).
// With nrhs right-hand sides, list entry g is task g / nrhs for right-hand
// side g % nrhs and waits for the same right-hand side's producers.
// ---------------------------------------------------------------------------
constexpr long long kQueueWaitCycles = 1000000000LL;  // default wait limit, about 0.5 s at 2 GHz

struct QueueView {
  const int4 *tasks;   // {kind (0 small CTA, 1 large-front task), level, index, 0}
  const int *dep_ptr;  // dependencies of task t: dep[dep_ptr[t] .. dep_ptr[t+1])
  const int *dep;
  int ntasks;
  long long wait_cycles;  // limit of one dependency wait (clock64 cycles)
  int skip_publish;       // list entry whose done flag is never published (-1: none; failure tests)
};

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

__device__ __forceinline__ void queue_wait(const QueueView &q, int t, int rk, int nrhs, const int *done,
                                           int *status) {
  for (int i = q.dep_ptr[t]; i < q.dep_ptr[t + 1]; i++) {
    const int *flag = done + (int64_t)q.dep[i] * nrhs + rk;
    const long long t0 = clock64();
    while (ld_volatile(flag) == 0) {
      if (clock64() - t0 > q.wait_cycles || (ld_volatile(status) & ERR_WAIT)) {
        atomicOr(status, ERR_WAIT);  // after one timeout no CTA waits any more
        return;
      }
      __nanosleep(100);
    }
  }
  __threadfence();
}

template <typename T>
__device__ __forceinline__ void queue_publish(const QueueView &q, int *done, int64_t idx) {
  __threadfence();
  if (idx == q.skip_publish) return;  // a producer that never finishes (failure tests)
  atomicExch(done + idx, 1);
}

// forward; small tasks: level lv, CTA index c of the level's small-front
// launch (fronts small_fronts + lvl_small_off[lv], buckets lvl_sb[lv])
template <typename T>
__global__ void __launch_bounds__(256, 4)
mf_fwd_queue(MfView v, QueueView q, const int *__restrict__ small_fronts, const int *__restrict__ lvl_small_off,
             const SmallBuckets *__restrict__ lvl_sb, const int2 *__restrict__ fwd_tasks,
             const TaskFront *__restrict__ fwd_tmeta, const T *__restrict__ E,
             const T *__restrict__ xl, T *__restrict__ yl, T *__restrict__ uvec, int *counter, int *done,
             int *status, int nrhs = 1, int64_t xs = 0, int64_t us = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ T red[8][FwdRows<T>::N];
  __shared__ int s_g;
  T *sm = reinterpret_cast<T *>(smem_raw);
  const int total = q.ntasks * nrhs;
  for (;;) {
    if (threadIdx.x == 0) s_g = atomicAdd(counter, 1);
    __syncthreads();
    const int g = s_g;
    if (g >= total) return;
    const int t = g / nrhs, rk = g % nrhs;
    if (threadIdx.x == 0) queue_wait(q, t, rk, nrhs, done, status);
    __syncthreads();
    const int4 tk = q.tasks[t];
    const T *xk = xl + rk * xs;
    T *yk = yl + rk * xs, *uk = uvec + rk * us;
    if (tk.x == 0) {
      const SmallBuckets sb = lvl_sb[tk.y];
      const int *fr = small_fronts + lvl_small_off[tk.y];
      const int b = tk.z;
      if (b < sb.nb0) fwd_small_body<T, 8>(v, fr, sb.cnt0, E, xk, yk, uk, b, sm);
      else if (b < sb.nb0 + sb.nb1) fwd_small_body<T, 16>(v, fr + sb.cnt0, sb.cnt1, E, xk, yk, uk, b - sb.nb0, sm);
      else fwd_small_body<T, 32>(v, fr + sb.cnt0 + sb.cnt1, sb.cnt2, E, xk, yk, uk, b - sb.nb0 - sb.nb1, sm);
    } else {
      fwd_big_body<T, 256>(v, fwd_tasks[tk.z], fwd_tmeta[tk.z], E, xk, yk, uk, sm, red);
    }
    __syncthreads();
    if (threadIdx.x == 0) queue_publish<T>(q, done, g);
  }
}

template <typename T>
__global__ void __launch_bounds__(256, 4)
mf_bwd_queue(MfView v, QueueView q, const int *__restrict__ small_fronts, const int *__restrict__ lvl_small_off,
             const SmallBuckets *__restrict__ lvl_sb, const int2 *__restrict__ bwd_tasks,
             const TaskFront *__restrict__ bwd_tmeta, const T *__restrict__ E,
             const T *__restrict__ yl, T *__restrict__ xl, int *counter, int *done, int *status, int nrhs = 1,
             int64_t xs = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_g;
  T *sm = reinterpret_cast<T *>(smem_raw);
  const int total = q.ntasks * nrhs;
  for (;;) {
    if (threadIdx.x == 0) s_g = atomicAdd(counter, 1);
    __syncthreads();
    const int g = s_g;
    if (g >= total) return;
    const int t = g / nrhs, rk = g % nrhs;
    if (threadIdx.x == 0) queue_wait(q, t, rk, nrhs, done, status);
    __syncthreads();
    const int4 tk = q.tasks[t];
    const T *yk = yl + rk * xs;
    T *xk = xl + rk * xs;
    if (tk.x == 0) {
      const SmallBuckets sb = lvl_sb[tk.y];
      const int *fr = small_fronts + lvl_small_off[tk.y];
      const int b = tk.z;
      if (b < sb.nb0) bwd_small_body<T, 8>(v, fr, sb.cnt0, E, yk, xk, b, sm);
      else if (b < sb.nb0 + sb.nb1) bwd_small_body<T, 16>(v, fr + sb.cnt0, sb.cnt1, E, yk, xk, b - sb.nb0, sm);
      else bwd_small_body<T, 32>(v, fr + sb.cnt0 + sb.cnt1, sb.cnt2, E, yk, xk, b - sb.nb0 - sb.nb1, sm);
    } else {
      bwd_big_body<T, 256>(v, bwd_tasks[tk.z], bwd_tmeta[tk.z], E, yk, xk, sm);
    }
    __syncthreads();
    if (threadIdx.x == 0) queue_publish<T>(q, done, g);
  }
}

// ---------------------------------------------------------------------------
// Symmetric Gauss-Seidel subdomain preconditioner (fine_method 2).  The
// reference runs, per subdomain, forward and backward Gauss-Seidel sweeps in
// global row order on the entries of A inside the subdomain, from x = 0
// (FinePreconditioner_sgs.F90:69-86, stationary.F90:33-88).  Here one CTA owns
// one subdomain; its rows are grouped into dependency levels of the
// (symmetrised) subdomain graph, so every row of a level depends only on rows
// of earlier levels in the sweep direction, and the result equals the
// sequential sweep (same entry order, separate multiply and subtract,
// division by the diagonal).  Levels are separated by __syncthreads.
// ---------------------------------------------------------------------------
struct SgsView {
  const int64_t *rp;        // local CSR over arena positions (entries inside the subdomain)
  const int *ci;            // column as arena position
  const double *va, *dg;    // values; diagonal (0 = row skipped, as in the reference)
  const int *gidx;          // global row of every arena position
  const int *sd_lev_f, *sd_lev_b;    // per subdomain: its range of levels
  const int *lev_f, *lev_b;          // per level: its range of rows
  const int *rows_f, *rows_b;        // rows (arena positions) grouped by level
};

constexpr int kSgsThreads = 256;

__device__ __forceinline__ void sgs_sweep(const SgsView &g, const int *sd_lev, const int *lev, const int *rows,
                                          int sd, const double *__restrict__ r, double *__restrict__ x) {
  for (int L = sd_lev[sd]; L < sd_lev[sd + 1]; L++) {
    for (int t = lev[L] + threadIdx.x; t < lev[L + 1]; t += kSgsThreads) {
      const int q = rows[t];
      const double d = g.dg[q];
      if (d == 0.0) continue;
      double xi = r[g.gidx[q]];
      for (int64_t e = g.rp[q]; e < g.rp[q + 1]; e++) {
        const int c = g.ci[e];
        if (c != q) xi = __dsub_rn(xi, __dmul_rn(g.va[e], x[c]));
      }
      x[q] = __ddiv_rn(xi, d);
    }
    __syncthreads();
  }
}

// one CTA per subdomain: x (arena, subdomain block) = SGS(iters) applied to r
__global__ void __launch_bounds__(kSgsThreads)
sgs_subdomains(SgsView g, const int64_t *__restrict__ sd_ptr, int iters, const double *__restrict__ r,
               double *__restrict__ x) {
  const int sd = blockIdx.x;
  for (int64_t q = sd_ptr[sd] + threadIdx.x; q < sd_ptr[sd + 1]; q += kSgsThreads) x[q] = 0.0;
  __syncthreads();
  for (int it = 0; it < iters; it++) {
    sgs_sweep(g, g.sd_lev_f, g.lev_f, g.rows_f, sd, r, x);
    sgs_sweep(g, g.sd_lev_b, g.lev_b, g.rows_b, sd, r, x);
  }
}

// ---------------------------------------------------------------------------
// Gradients of a loss L(x) through x = A^-1 b, given the adjoint solution
// lambda = A^-1 dL/dx (A symmetric): dL/db = lambda, dL/dA_ij = -lambda_i x_j.
// ---------------------------------------------------------------------------
// one value per input triplet (row gi, column gj, 0-based)
__global__ void grad_coo(int64_t nnz, const int *__restrict__ gi, const int *__restrict__ gj,
                         const double *__restrict__ lam, const double *__restrict__ x, double *__restrict__ g) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    g[k] = -(lam[gi[k]] * x[gj[k]]);
}

// one value per element: the derivative with respect to a factor s_e that
// scales the element's matrix, -sum_ij lambda[f_j] A_e(i,j) x[f_i] (the
// element assembly stores A_e(i,j) at row f_j, column f_i); one warp per
// element, the element's terms summed in a fixed order
__global__ void grad_elements(int nell, const int *__restrict__ eptr, const int *__restrict__ efl,
                              const int64_t *__restrict__ eoff, const double *__restrict__ emat,
                              const double *__restrict__ lam, const double *__restrict__ x, double *__restrict__ g) {
  const int lane = threadIdx.x & 31;
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (e >= nell) return;
  const int f0 = eptr[e], nf = eptr[e + 1] - f0;
  const double *Ae = emat + eoff[e];
  double s = 0.0;
  for (int q = lane; q < nf * nf; q += 32) {
    const int j = q / nf, i = q % nf;  // column j, row i of the element matrix
    s += lam[efl[f0 + j]] * Ae[q] * x[efl[f0 + i]];
  }
  s = warp_sum(s);
  if (lane == 0) g[e] = -s;
}

// ---------------------------------------------------------------------------
// Matrix-free product with stored element matrices (elemental input, option
// elemental_matvec 1): q = A p with A = sum_e of element e's matrix placed at
// its freedoms (A_e(i,j) at row f_j, column f_i, as the element assembly puts
// it).  Pass 1 stages a run of element matrices in shared memory with
// coalesced loads and forms every element's column products
// c[e, j] = sum_i A_e(i,j) p[f_i]; pass 2 sums, for every row, its element
// contributions in element order (no atomics: the result is deterministic)
// and the p.q partial sums.
// ---------------------------------------------------------------------------
constexpr int kElemChunk = 4096;  // matrix values per CTA stage (32 KB)
constexpr int kElemFree = 512;    // element freedoms per CTA stage
constexpr int kElemRun = 512;     // elements per CTA stage

// A(i, j) of an element matrix in shared memory: full column-major storage,
// or (SYM) the lower triangle column by column, column c starting at
// c*nf - c(c-1)/2 (for bitwise symmetric element matrices: the same values)
template <bool SYM>
__device__ __forceinline__ double elem_entry(const double *Me, int nf, int i, int j) {
  if (!SYM) return Me[j * nf + i];
  const int r = i >= j ? i : j, c = i >= j ? j : i;
  return Me[c * nf - (c * (c - 1)) / 2 + (r - c)];
}

// task t = elements [erun[t], erun[t+1]); the CTA stages their matrices, their
// offsets and the p values of their freedoms in shared memory (coalesced
// loads; the p gathers all in flight at once), then one thread per
// (element, column): c = sum_i A_e(i, j) p[f_i] in increasing i
template <bool SYM>
__global__ void __launch_bounds__(256)
elem_contrib(const int *__restrict__ erun, const int *__restrict__ eptr, const int *__restrict__ efl,
             const int64_t *__restrict__ eoff, const double *__restrict__ emat, const double *__restrict__ p,
             double *__restrict__ c) {
  __shared__ double Ms[kElemChunk];
  __shared__ double ps[kElemFree];
  __shared__ int ep[kElemRun + 1], eo[kElemRun + 1];
  const int e0 = erun[blockIdx.x], e1 = erun[blockIdx.x + 1], ne = e1 - e0;
  const int f0 = eptr[e0], nfr = eptr[e1] - f0;
  const int64_t m0 = eoff[e0];
  const int len = (int)(eoff[e1] - m0);
  for (int q = threadIdx.x; q < len; q += blockDim.x) Ms[q] = emat[m0 + q];
  for (int q = threadIdx.x; q <= ne; q += blockDim.x) {
    ep[q] = eptr[e0 + q] - f0;
    eo[q] = (int)(eoff[e0 + q] - m0);
  }
  for (int q = threadIdx.x; q < nfr; q += blockDim.x) ps[q] = p[efl[f0 + q]];
  __syncthreads();
  for (int t = threadIdx.x; t < nfr; t += blockDim.x) {
    int lo = 0, hi = ne - 1;  // element of item t: the last e with ep[e] <= t
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ep[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const int fe = ep[lo], nf = ep[lo + 1] - fe, j = t - fe;
    const double *Me = Ms + eo[lo];
    const double *pe = ps + fe;
    double s = 0.0;
    // fused multiply-adds: FP64 issue, not DRAM, bounds this product on GB300
    for (int i = 0; i < nf; i++) s = __fma_rn(elem_entry<SYM>(Me, nf, i, j), pe[i], s);
    c[f0 + t] = s;
  }
}

// q[r] = sum of r's element contributions (element order); partial p.q.
// Four contributions of a row are loaded before they are added.
__global__ void __launch_bounds__(kVecThreads)
elem_pull_pq(int n, const int64_t *__restrict__ rptr, const int *__restrict__ ridx, const double *__restrict__ c,
             const double *__restrict__ p, double *__restrict__ q, double *__restrict__ part_pq) {
  __shared__ double sh[32];
  double spq = 0.0;
  for (int r = blockIdx.x * kVecThreads + threadIdx.x; r < n; r += gridDim.x * kVecThreads) {
    const int64_t t0 = rptr[r], t1 = rptr[r + 1];
    const double pr = p[r];
    double s = 0.0;
    int64_t t = t0;
    for (; t + 4 <= t1; t += 4) {
      const int i0 = ridx[t], i1 = ridx[t + 1], i2 = ridx[t + 2], i3 = ridx[t + 3];
      const double c0 = c[i0], c1 = c[i1], c2 = c[i2], c3 = c[i3];
      s = __dadd_rn(s, c0);
      s = __dadd_rn(s, c1);
      s = __dadd_rn(s, c2);
      s = __dadd_rn(s, c3);
    }
    for (; t < t1; t++) s = __dadd_rn(s, c[ridx[t]]);
    q[r] = s;
    spq += pr * s;
  }
  double b = block_sum<kVecThreads>(spq, sh);
  if (threadIdx.x == 0) part_pq[blockIdx.x] = b;
}

// ---------------------------------------------------------------------------
// Schwarz gather / pull sum and coarse transfer
// ---------------------------------------------------------------------------
// nrhs right-hand sides: vector k at r + k * rs, local vector k at xl + k * len
template <typename T>
__global__ void gather_subdomains(const double *__restrict__ r, const int *__restrict__ gidx,
                                  T *__restrict__ xl, int64_t len, int nrhs = 1, int64_t rs = 0) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < len;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int g = gidx[p];
    for (int k = 0; k < nrhs; k++) xl[k * len + p] = (T)r[k * rs + g];
  }
}

// crhs (in the coarse batch's local numbering) = R r
// nrhs right-hand sides: r_k at r + k * rs, the coarse vector k at xc + k * xcs.
// L lanes per coarse row (chosen for about 12 entries per lane), four loads
// in flight per lane, the lane sums added by a shuffle tree.
template <typename TR, int L>
__global__ void __launch_bounds__(kVecThreads)
restrict_to_coarse(const int64_t *__restrict__ Rp, const int *__restrict__ Rc, const TR *__restrict__ Rv,
                   const double *__restrict__ r, const int *__restrict__ cpos, double *__restrict__ xc, int nc,
                   int nrhs = 1, int64_t rs = 0, int64_t xcs = 0) {
  const int sub = threadIdx.x % L;
  const int rows_per_grid = gridDim.x * (kVecThreads / L);
  for (int a0 = blockIdx.x * (kVecThreads / L); a0 < nc; a0 += rows_per_grid) {
    const int a = a0 + threadIdx.x / L;
    const bool on = a < nc;
    const int64_t e0 = on ? Rp[a] : 0, e1 = on ? Rp[a + 1] : 0;
    for (int k = 0; k < nrhs; k++) {
      const double *rk = r + k * rs;
      double s = 0.0;
      int64_t e = e0 + sub;
      for (; e + 3 * L < e1; e += 4 * L) {
        const int c0 = Rc[e], c1 = Rc[e + L], c2 = Rc[e + 2 * L], c3 = Rc[e + 3 * L];
        const double v0 = (double)Rv[e], v1 = (double)Rv[e + L], v2 = (double)Rv[e + 2 * L], v3 = (double)Rv[e + 3 * L];
        const double x0 = rk[c0], x1 = rk[c1], x2 = rk[c2], x3 = rk[c3];
        s += v0 * x0;
        s += v1 * x1;
        s += v2 * x2;
        s += v3 * x3;
      }
      for (; e < e1; e += L) s += (double)Rv[e] * rk[Rc[e]];
#pragma unroll
      for (int o = L / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, L);
      if (on && sub == 0) xc[k * xcs + cpos[a]] = s;
    }
  }
}

// z_g = (sum of subdomain solutions at g, in subdomain order) + (P x_c)_g ;
// partial sums of r.z (and of r.z_old for the flexible variant).  One thread
// per node; Pcp holds coarse-vector positions (composed at setup).  The loads
// of a node are issued in three dependent rounds (row pointers, r and z_old;
// the first two pull positions and the first four P entries; the gathers),
// the rare longer rows finish in loops; the sums keep the entries' order.
template <typename T, typename TP>
__global__ void __launch_bounds__(kVecThreads)
pull_prolong_dot(int n, const int *__restrict__ pull_ptr, const int *__restrict__ pull_idx,
                 const T *__restrict__ xl, const int64_t *__restrict__ Pp, const int *__restrict__ Pcp,
                 const TP *__restrict__ Pv, const double *__restrict__ xc,
                 int mode, const double *__restrict__ r, double *__restrict__ z,
                 double *__restrict__ zold, double *__restrict__ part_rz, double *__restrict__ part_rzo,
                 const int *__restrict__ cb = nullptr, const int *__restrict__ csys = nullptr,
                 int64_t vs = 0, int64_t xls = 0, int64_t xcs = 0) {
  // mode bit 0: fine subdomains on; bit 1: coarse on; bit 2: identity fine (z=r);
  // bit 3: keep z_old and produce r.z_old.  cb (batched systems / right-hand
  // sides): CTA b owns the positions [cb[b], cb[b+1]) of the stacked vectors
  // and its partial sums are that chunk's; with csys, the chunk belongs to
  // right-hand side k = csys[b]: rows g - k*vs of the matrix and the local
  // vectors at k*xls (subdomains) and k*xcs (coarse).
  __shared__ double sh[32];
  double srz = 0.0, srzo = 0.0;
  const int g0 = cb ? cb[blockIdx.x] + threadIdx.x : blockIdx.x * kVecThreads + threadIdx.x;
  const int gend = cb ? cb[blockIdx.x + 1] : n;
  const int gstep = cb ? kVecThreads : gridDim.x * kVecThreads;
  const int64_t rk = csys ? csys[blockIdx.x] : 0;
  const int64_t voff = rk * vs;
  if (xl) xl += rk * xls;
  if (xc) xc += rk * xcs;
  const bool pull = (mode & 5) == 1, prol = (mode & 2) != 0, flex = (mode & 8) != 0;
  for (int gg = g0; gg < gend; gg += gstep) {
    const int64_t g = gg;              // position in the stacked vectors
    const int gl = (int)(g - voff);    // row of the matrix / pull lists
    // round 1
    const double rg = r[g];
    const double zo = flex ? zold[g] : 0.0;
    int q0 = 0, q1 = 0;
    int64_t e0 = 0, e1 = 0;
    if (pull) { q0 = pull_ptr[gl]; q1 = pull_ptr[gl + 1]; }
    if (prol) { e0 = Pp[gl]; e1 = Pp[gl + 1]; }
    // round 2
    const int i0 = q0 < q1 ? pull_idx[q0] : -1;
    const int i1 = q0 + 1 < q1 ? pull_idx[q0 + 1] : -1;
    int pc[4];
    TP pv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const bool on = e0 + u < e1;
      pc[u] = on ? Pcp[e0 + u] : -1;
      pv[u] = on ? Pv[e0 + u] : TP(0);
    }
    // round 3
    const T x0 = i0 >= 0 ? xl[i0] : T(0);
    const T x1 = i1 >= 0 ? xl[i1] : T(0);
    TP xv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) xv[u] = pc[u] >= 0 ? (TP)xc[pc[u]] : TP(0);
    double sv = 0.0;
    if (mode & 4) {
      sv = rg;
    } else if (pull) {
      if (i0 >= 0) sv = sv + (double)x0;
      if (i1 >= 0) sv = sv + (double)x1;
      for (int q = q0 + 2; q < q1; q++) sv = sv + (double)xl[pull_idx[q]];
    }
    if (prol) {
      TP t = TP(0);
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (pc[u] >= 0) t += pv[u] * xv[u];
      for (int64_t e = e0 + 4; e < e1; e++) t += Pv[e] * (TP)xc[Pcp[e]];
      sv = sv + (double)t;
    }
    if (flex) {
      srzo += rg * zo;
      zold[g] = sv;
    }
    z[g] = sv;
    srz += rg * sv;
  }
  double b = block_sum<kVecThreads>(srz, sh);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = b;
  if (flex) {
    b = block_sum<kVecThreads>(srzo, sh);
    if (threadIdx.x == 0) part_rzo[blockIdx.x] = b;
  }
}

// ---------------------------------------------------------------------------
// CG steps.  sc[] holds device scalars:
//   0 rho_prev, 1 rho, 2 alpha, 3 res_norm (r.r), 4 init_norm, 5 beta, 6 p.q
// ---------------------------------------------------------------------------
enum { SC_RHO_PREV = 0, SC_RHO = 1, SC_ALPHA = 2, SC_RES = 3, SC_INIT = 4, SC_BETA = 5, SC_PQ = 6 };

// beta of the iteration from the r.z partials: Fletcher-Reeves (DOUG) or
// flexible Polak-Ribiere
__device__ __forceinline__ double cg_beta(const double *part_rz, const double *part_rzo,
                                          const double *sc, int first, int flexible, double *rho_out) {
  const double rho = sum_partials(part_rz);
  *rho_out = rho;
  if (first) return 0.0;
  if (flexible) {
    const double rzo = sum_partials(part_rzo);
    return __ddiv_rn(__dsub_rn(rho, rzo), sc[SC_RHO_PREV]);
  }
  return __ddiv_rn(rho, sc[SC_RHO_PREV]);
}

// p = z + beta p (p = z on the first step); beta from the r.z partials
__global__ void __launch_bounds__(kVecThreads)
cg_direction(int n, const double *__restrict__ z, double *__restrict__ p,
             const double *__restrict__ part_rz, const double *__restrict__ part_rzo,
             double *__restrict__ sc, int first, int flexible) {
  __shared__ double s_beta;
  if (threadIdx.x < 32) {
    double rho;
    double beta = cg_beta(part_rz, part_rzo, sc, first, flexible, &rho);
    if (threadIdx.x == 0) {
      s_beta = beta;
      if (blockIdx.x == 0) { sc[SC_RHO] = rho; sc[SC_BETA] = beta; }
    }
  }
  __syncthreads();
  const double beta = s_beta;
  for (int i = blockIdx.x * kVecThreads + threadIdx.x; i < n; i += gridDim.x * kVecThreads)
    p[i] = first ? z[i] : __dadd_rn(z[i], __dmul_rn(beta, p[i]));
}

// q = A p with LANES lanes per row; partial sums of p.q
template <int LANES>
__global__ void __launch_bounds__(kVecThreads)
spmv_pq(int n, const int64_t *__restrict__ Ap, const int *__restrict__ Ac, const double *__restrict__ Av,
        const double *__restrict__ p, double *__restrict__ q, double *__restrict__ part_pq) {
  __shared__ double sh[32];
  const int sub = threadIdx.x % LANES;
  const int rows_per_block = kVecThreads / LANES;
  double spq = 0.0;
  for (int row0 = blockIdx.x * rows_per_block; row0 < n; row0 += gridDim.x * rows_per_block) {
    const int i = row0 + threadIdx.x / LANES;
    double s = 0.0;
    if (i < n) {
      int64_t e = Ap[i] + sub;
      const int64_t e1 = Ap[i + 1];
      // four entries of this lane's share loaded before they are summed
      for (; e + 3 * LANES < e1; e += 4 * LANES) {
        const int c0 = Ac[e], c1 = Ac[e + LANES], c2 = Ac[e + 2 * LANES], c3 = Ac[e + 3 * LANES];
        const double a0 = Av[e], a1 = Av[e + LANES], a2 = Av[e + 2 * LANES], a3 = Av[e + 3 * LANES];
        const double p0 = p[c0], p1 = p[c1], p2 = p[c2], p3 = p[c3];
        s = __fma_rn(a0, p0, s);
        s = __fma_rn(a1, p1, s);
        s = __fma_rn(a2, p2, s);
        s = __fma_rn(a3, p3, s);
      }
      for (; e < e1; e += LANES) s = __fma_rn(Av[e], p[Ac[e]], s);
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LANES);
    if (i < n && sub == 0) {
      q[i] = s;
      spq += p[i] * s;
    }
  }
  double b = block_sum<kVecThreads>(spq, sh);
  if (threadIdx.x == 0) part_pq[blockIdx.x] = b;
}

// x += alpha p; r -= alpha q; partial r.r  (alpha = rho / p.q)
__global__ void __launch_bounds__(kVecThreads)
cg_update(int n, const double *__restrict__ p, const double *__restrict__ q,
          double *__restrict__ x, double *__restrict__ r, double *__restrict__ sc,
          const double *__restrict__ part_pq, double *__restrict__ part_rr) {
  __shared__ double sh[32];
  __shared__ double s_alpha;
  if (threadIdx.x < 32) {
    const double pq = sum_partials(part_pq);
    if (threadIdx.x == 0) {
      const double alpha = __ddiv_rn(sc[SC_RHO], pq);
      s_alpha = alpha;
      if (blockIdx.x == 0) { sc[SC_ALPHA] = alpha; sc[SC_PQ] = pq; }
    }
  }
  __syncthreads();
  const double alpha = s_alpha;
  double srr = 0.0;
  for (int i = blockIdx.x * kVecThreads + threadIdx.x; i < n; i += gridDim.x * kVecThreads) {
    x[i] = __dadd_rn(x[i], __dmul_rn(alpha, p[i]));
    const double ri = __dsub_rn(r[i], __dmul_rn(alpha, q[i]));
    r[i] = ri;
    srr += ri * ri;
  }
  double b = block_sum<kVecThreads>(srr, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = b;
}

// r = b - A x (FP64 true residual), partial r.r
template <int LANES>
__global__ void __launch_bounds__(kVecThreads)
residual(int n, const int64_t *__restrict__ Ap, const int *__restrict__ Ac, const double *__restrict__ Av,
         const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ r,
         double *__restrict__ part_rr) {
  __shared__ double sh[32];
  const int sub = threadIdx.x % LANES;
  const int rows_per_block = kVecThreads / LANES;
  double srr = 0.0;
  for (int row0 = blockIdx.x * rows_per_block; row0 < n; row0 += gridDim.x * rows_per_block) {
    const int i = row0 + threadIdx.x / LANES;
    double s = 0.0;
    if (i < n)
      for (int64_t e = Ap[i] + sub; e < Ap[i + 1]; e += LANES) s = __fma_rn(Av[e], x[Ac[e]], s);
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LANES);
    if (i < n && sub == 0) {
      const double ri = __dsub_rn(b[i], s);
      r[i] = ri;
      srr += ri * ri;
    }
  }
  double t = block_sum<kVecThreads>(srr, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
}

// finish an iteration: res = sum(part_rr); rho_prev = rho; publish to host
__global__ void cg_finish(double *__restrict__ sc, const double *__restrict__ part_rr, int init,
                          volatile double *__restrict__ host_out, const int *__restrict__ status,
                          volatile int *__restrict__ host_status) {
  if (threadIdx.x < 32) {
    const double rr = sum_partials(part_rr);
    if (threadIdx.x == 0) {
      // init: 1 = initial residual, 0 = end of an iteration, 2 = report only
      if (init == 1) sc[SC_INIT] = rr;
      else if (init == 0) { sc[SC_RES] = rr; sc[SC_RHO_PREV] = sc[SC_RHO]; }
      host_out[0] = rr;
      host_out[1] = sc[SC_INIT];
      host_out[2] = sc[SC_ALPHA];
      host_out[3] = sc[SC_BETA];
      host_out[4] = sc[SC_RHO];
      host_out[5] = sc[SC_PQ];
      *host_status = *status;
    }
  }
}

// ---------------------------------------------------------------------------
// Batched independent systems (dg_set_systems).  The systems are the diagonal
// blocks of one matrix; every CTA of these vector kernels owns one chunk
// [cb[c], cb[c+1]) of the rows of system csys[c], so partial sums are per
// chunk and the CG scalars per system (bsc[k * BS_N + ...]).  A system leaves
// the iteration when its own residual test passes: its x, r and p are then
// frozen while the others go on, which makes each system's iterates those of
// its own PCG.
// ---------------------------------------------------------------------------
constexpr int kBatchChunk = 1024;  // rows per CTA of the batched vector kernels
enum { BS_RHO_PREV = 0, BS_RHO = 1, BS_ALPHA = 2, BS_RES = 3, BS_INIT = 4, BS_BETA = 5, BS_PQ = 6,
       BS_TRUE = 7, BS_N = 8 };
// per-system state
enum { BT_DONE = 0, BT_ACTIVE = 1, BT_CHECK = 2, BT_BREAKDOWN = 3 };
// bt_scalars steps
enum { BT_RHO = 0, BT_ALPHA = 1, BT_INIT = 2, BT_FINISH = 3, BT_CONFIRM = 4, BT_REPORT = 5 };

__global__ void __launch_bounds__(kVecThreads)
bt_direction(const int *__restrict__ cb, const int *__restrict__ csys, const int *__restrict__ state,
             const double *__restrict__ bsc, const double *__restrict__ z, double *__restrict__ p, int first) {
  const int k = csys[blockIdx.x];
  if (state[k] != BT_ACTIVE) return;
  const double beta = bsc[k * BS_N + BS_BETA];
  const int i1 = cb[blockIdx.x + 1];
  for (int i = cb[blockIdx.x] + threadIdx.x; i < i1; i += kVecThreads)
    p[i] = first ? z[i] : __dadd_rn(z[i], __dmul_rn(beta, p[i]));
}

// q = A p on the chunk's rows (LANES lanes per row), partial p.q
template <int LANES>
__global__ void __launch_bounds__(kVecThreads)
bt_spmv_pq(const int *__restrict__ cb, const int *__restrict__ csys, const int *__restrict__ state,
           const int64_t *__restrict__ Ap, const int *__restrict__ Ac, const double *__restrict__ Av,
           const double *__restrict__ p, double *__restrict__ q, double *__restrict__ part_pq, int64_t vs = 0) {
  // vs > 0 (right-hand sides of one matrix): position g of vector k is row g - k*vs
  __shared__ double sh[32];
  const int64_t voff = (int64_t)csys[blockIdx.x] * vs;
  const double *pc = p + voff;  // pc[c]: column c of this right-hand side
  if (state[csys[blockIdx.x]] != BT_ACTIVE) {
    if (threadIdx.x == 0) part_pq[blockIdx.x] = 0.0;
    return;
  }
  const int sub = threadIdx.x % LANES;
  const int rows_per_block = kVecThreads / LANES;
  const int i1 = cb[blockIdx.x + 1];
  double spq = 0.0;
  for (int row0 = cb[blockIdx.x]; row0 < i1; row0 += rows_per_block) {
    const int i = row0 + threadIdx.x / LANES;
    double s = 0.0;
    if (i < i1) {
      int64_t e = Ap[i - voff] + sub;
      const int64_t e1 = Ap[i - voff + 1];
      for (; e + 3 * LANES < e1; e += 4 * LANES) {
        const int c0 = Ac[e], c1 = Ac[e + LANES], c2 = Ac[e + 2 * LANES], c3 = Ac[e + 3 * LANES];
        const double a0 = Av[e], a1 = Av[e + LANES], a2 = Av[e + 2 * LANES], a3 = Av[e + 3 * LANES];
        const double p0 = pc[c0], p1 = pc[c1], p2 = pc[c2], p3 = pc[c3];
        s = __fma_rn(a0, p0, s);
        s = __fma_rn(a1, p1, s);
        s = __fma_rn(a2, p2, s);
        s = __fma_rn(a3, p3, s);
      }
      for (; e < e1; e += LANES) s = __fma_rn(Av[e], pc[Ac[e]], s);
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LANES);
    if (i < i1 && sub == 0) {
      q[i] = s;
      spq += p[i] * s;
    }
  }
  double b = block_sum<kVecThreads>(spq, sh);
  if (threadIdx.x == 0) part_pq[blockIdx.x] = b;
}

// x += alpha_k p; r -= alpha_k q; partial r.r
__global__ void __launch_bounds__(kVecThreads)
bt_update(const int *__restrict__ cb, const int *__restrict__ csys, const int *__restrict__ state,
          const double *__restrict__ bsc, const double *__restrict__ p, const double *__restrict__ q,
          double *__restrict__ x, double *__restrict__ r, double *__restrict__ part_rr) {
  __shared__ double sh[32];
  const int k = csys[blockIdx.x];
  if (state[k] != BT_ACTIVE) {
    if (threadIdx.x == 0) part_rr[blockIdx.x] = 0.0;
    return;
  }
  const double alpha = bsc[k * BS_N + BS_ALPHA];
  const int i1 = cb[blockIdx.x + 1];
  double srr = 0.0;
  for (int i = cb[blockIdx.x] + threadIdx.x; i < i1; i += kVecThreads) {
    x[i] = __dadd_rn(x[i], __dmul_rn(alpha, p[i]));
    const double ri = __dsub_rn(r[i], __dmul_rn(alpha, q[i]));
    r[i] = ri;
    srr += ri * ri;
  }
  double b = block_sum<kVecThreads>(srr, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = b;
}

// r = b - A x on the chunks of the systems in state `want` (all when want < 0)
template <int LANES>
__global__ void __launch_bounds__(kVecThreads)
bt_residual(const int *__restrict__ cb, const int *__restrict__ csys, const int *__restrict__ state, int want,
            const int64_t *__restrict__ Ap, const int *__restrict__ Ac, const double *__restrict__ Av,
            const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ r,
            double *__restrict__ part_rr, int64_t vs = 0) {
  __shared__ double sh[32];
  const int64_t voff = (int64_t)csys[blockIdx.x] * vs;
  const double *xc = x + voff;  // xc[c]: column c of this right-hand side
  if (want >= 0 && state[csys[blockIdx.x]] != want) {
    if (threadIdx.x == 0) part_rr[blockIdx.x] = 0.0;
    return;
  }
  const int sub = threadIdx.x % LANES;
  const int rows_per_block = kVecThreads / LANES;
  const int i1 = cb[blockIdx.x + 1];
  double srr = 0.0;
  for (int row0 = cb[blockIdx.x]; row0 < i1; row0 += rows_per_block) {
    const int i = row0 + threadIdx.x / LANES;
    double s = 0.0;
    if (i < i1)
      for (int64_t e = Ap[i - voff] + sub; e < Ap[i - voff + 1]; e += LANES) s = __fma_rn(Av[e], xc[Ac[e]], s);
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, LANES);
    if (i < i1 && sub == 0) {
      const double ri = __dsub_rn(b[i], s);
      r[i] = ri;
      srr += ri * ri;
    }
  }
  double t = block_sum<kVecThreads>(srr, sh);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
}

// Per-system CG scalars from the chunk partials (one warp per system, chunks
// summed in a fixed order), the state machine and the counts the host reads.
// One CTA of 1024 threads.  dit: the device iteration counter (incremented by
// BT_FINISH), so that a captured graph needs no per-iteration argument.
__global__ void __launch_bounds__(1024)
bt_scalars(int nsys, const int *__restrict__ sys_cptr, int step, int first, int flexible, int mixed, double tol2,
           const double *__restrict__ part_a, const double *__restrict__ part_b, double *__restrict__ bsc,
           int *__restrict__ state, int *__restrict__ iters, int *__restrict__ dit,
           volatile int *__restrict__ host_counts) {
  __shared__ int cnt[3];
  if (threadIdx.x < 3) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int it = *dit + (step == BT_FINISH ? 1 : 0);
  for (int k = wid; k < nsys; k += nw) {
    double *sc = bsc + (size_t)k * BS_N;
    const int c0 = sys_cptr[k], c1 = sys_cptr[k + 1];
    double a = 0.0, b = 0.0;
    for (int c = c0 + lane; c < c1; c += 32) a += part_a[c];
    a = __shfl_sync(0xffffffffu, warp_sum(a), 0);
    if (step == BT_RHO && flexible && !first) {
      for (int c = c0 + lane; c < c1; c += 32) b += part_b[c];
      b = __shfl_sync(0xffffffffu, warp_sum(b), 0);
    }
    int stt = state[k];
    if (lane == 0) {
      switch (step) {
        case BT_RHO:
          if (stt == BT_ACTIVE) {
            sc[BS_RHO] = a;
            sc[BS_BETA] = first ? 0.0 : flexible ? __ddiv_rn(__dsub_rn(a, b), sc[BS_RHO_PREV])
                                                 : __ddiv_rn(a, sc[BS_RHO_PREV]);
          }
          break;
        case BT_ALPHA:
          if (stt == BT_ACTIVE) {
            sc[BS_PQ] = a;
            sc[BS_ALPHA] = __ddiv_rn(sc[BS_RHO], a);
            if (!(a > 0.0)) { stt = BT_BREAKDOWN; iters[k] = *dit + 1; }
          }
          break;
        case BT_INIT:
          sc[BS_RES] = a;
          sc[BS_INIT] = a == 0.0 ? 1.0 : a;
          sc[BS_TRUE] = a;
          sc[BS_RHO_PREV] = 0.0;
          stt = BT_ACTIVE;
          iters[k] = 0;
          break;
        case BT_FINISH:
          if (stt == BT_ACTIVE) {
            sc[BS_RES] = a;
            sc[BS_RHO_PREV] = sc[BS_RHO];
            iters[k] = it;
            if (a != a) stt = BT_BREAKDOWN;
            else if (!(a / sc[BS_INIT] > tol2)) stt = mixed ? BT_CHECK : BT_DONE;
          }
          break;
        case BT_CONFIRM:  // the FP64 true residual decides; r now holds it
          if (stt == BT_CHECK) {
            sc[BS_RES] = a;
            stt = a / sc[BS_INIT] > tol2 ? BT_ACTIVE : BT_DONE;
          }
          break;
        default:  // BT_REPORT
          sc[BS_TRUE] = a;
          break;
      }
      state[k] = stt;
      if (stt == BT_ACTIVE) atomicAdd(&cnt[0], 1);
      else if (stt == BT_CHECK) atomicAdd(&cnt[1], 1);
      else if (stt == BT_BREAKDOWN) atomicAdd(&cnt[2], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (step == BT_FINISH) *dit = it;
    if (step == BT_INIT) *dit = 0;
    host_counts[0] = cnt[0];
    host_counts[1] = cnt[1];
    host_counts[2] = cnt[2];
  }
}

}  // namespace dg
