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
// All waits are __syncthreads barriers; no kernel spins on memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dg {

constexpr int kRedBlocks = 1024;   // partial-sum slots of every reduction
constexpr int kVecThreads = 256;

// device error word bits
enum : int { ERR_NOT_SPD = 1, ERR_NAN = 2, ERR_BREAKDOWN = 4 };

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
};

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

template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_factor_level(MfView v, const int *__restrict__ fronts, const double *__restrict__ vals,
                T *__restrict__ arena, int *__restrict__ status) {
  __shared__ T As[kNB][kTile];
  __shared__ T Bs[kNB][kTile];
  __shared__ T piv;
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  T *F = arena + v.f_off[f];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = kMfThreads / 32;
  // 1. zero the lower triangle
  for (int c = wid; c < m; c += nw)
    for (int i = c + lane; i < m; i += 32) F[(int64_t)c * m + i] = T(0);
  __syncthreads();
  // 2. original entries (each target appears once; duplicates summed in order)
  for (int64_t e = v.f_asm[f] + tid; e < v.f_asm[f + 1]; e += kMfThreads) {
    double s = 0.0;
    for (int64_t q = v.asm_sp[e]; q < v.asm_sp[e + 1]; q++) s += vals[v.asm_src[q]];
    arena[v.asm_tgt[e]] = (T)s;
  }
  __syncthreads();
  // 3. extend-add of the children's update matrices, children in order
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int mc = v.f_m[c], kc = v.f_k[c], rc = mc - kc;
    const T *U = arena + v.f_off[c] + (int64_t)kc * mc + kc;
    const int *rel = v.relmap + v.f_relmap[c];
    for (int b = wid; b < rc; b += nw) {
      const int pb = rel[b];
      for (int a = b + lane; a < rc; a += 32) F[(int64_t)pb * m + rel[a]] += U[(int64_t)b * mc + a];
    }
    __syncthreads();
  }
  // 4. partial Cholesky of the k pivot columns; the trailing (m-k) block
  //    becomes the update (Schur complement) matrix
  for (int j0 = 0; j0 < k; j0 += kNB) {
    const int jb = min(kNB, k - j0);
    for (int j = j0; j < j0 + jb; j++) {
      if (tid == 0) {
        T d = F[(int64_t)j * m + j];
        if (!(d > T(0))) { atomicOr(status, ERR_NOT_SPD); d = T(1); }
        piv = tsqrt<T>(d);
        F[(int64_t)j * m + j] = piv;
      }
      __syncthreads();
      const T p = piv;
      for (int i = j + 1 + tid; i < m; i += kMfThreads) F[(int64_t)j * m + i] /= p;
      __syncthreads();
      // remaining columns of the panel
      for (int c = j + 1 + wid; c < j0 + jb; c += nw) {
        const T lcj = F[(int64_t)j * m + c];
        for (int i = c + lane; i < m; i += 32) F[(int64_t)c * m + i] -= F[(int64_t)j * m + i] * lcj;
      }
      __syncthreads();
    }
    // trailing update of columns [j0+jb, m): F -= Lp Lp^T (lower part)
    const int c0 = j0 + jb;
    const int nt = (m - c0 + kTile - 1) / kTile;
    const int tx = tid & 15, ty = tid >> 4;
    for (int tj = 0; tj < nt; tj++) {
      for (int ti = tj; ti < nt; ti++) {
        const int r0 = c0 + ti * kTile, cc0 = c0 + tj * kTile;
        for (int q = tid; q < kNB * kTile; q += kMfThreads) {
          int t = q / kTile, r = q % kTile;
          T a = T(0), b = T(0);
          if (t < jb) {
            if (r0 + r < m) a = F[(int64_t)(j0 + t) * m + r0 + r];
            if (cc0 + r < m) b = F[(int64_t)(j0 + t) * m + cc0 + r];
          }
          As[t][r] = a;
          Bs[t][r] = b;
        }
        __syncthreads();
        T acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int b = 0; b < 4; b++) acc[a][b] = T(0);
        for (int t = 0; t < jb; t++) {
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
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const int col = cc0 + ty + 16 * b;
          if (col >= m) continue;
#pragma unroll
          for (int a = 0; a < 4; a++) {
            const int row = r0 + tx + 16 * a;
            if (row < m && row >= col) F[(int64_t)col * m + row] -= acc[a][b];
          }
        }
        __syncthreads();
      }
    }
  }
}

// Small fronts: the whole m x m front lives in shared memory while it is
// assembled and factored, then its lower part is written back.
constexpr int kSmallThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kSmallThreads)
mf_factor_small(MfView v, const int *__restrict__ fronts, const double *__restrict__ vals,
                T *__restrict__ arena, int *__restrict__ status) {
  extern __shared__ unsigned char smem_raw[];
  T *S = reinterpret_cast<T *>(smem_raw);
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  const int64_t off = v.f_off[f];
  const int tid = threadIdx.x, nt = kSmallThreads;
  for (int q = tid; q < m * m; q += nt) S[q] = T(0);
  __syncthreads();
  for (int64_t e = v.f_asm[f] + tid; e < v.f_asm[f + 1]; e += nt) {
    double sv = 0.0;
    for (int64_t q = v.asm_sp[e]; q < v.asm_sp[e + 1]; q++) sv += vals[v.asm_src[q]];
    S[v.asm_tgt[e] - off] = (T)sv;
  }
  __syncthreads();
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int mc = v.f_m[c], kc = v.f_k[c], rc = mc - kc;
    const T *U = arena + v.f_off[c] + (int64_t)kc * mc + kc;
    const int *rel = v.relmap + v.f_relmap[c];
    for (int q = tid; q < rc * rc; q += nt) {
      const int b = q / rc, a = q % rc;
      if (a >= b) S[rel[b] * m + rel[a]] += U[(int64_t)b * mc + a];
    }
    __syncthreads();
  }
  for (int j = 0; j < k; j++) {
    if (tid == 0) {
      T d = S[j * m + j];
      if (!(d > T(0))) { atomicOr(status, ERR_NOT_SPD); d = T(1); }
      S[j * m + j] = tsqrt<T>(d);
    }
    __syncthreads();
    const T p = S[j * m + j];
    for (int i = j + 1 + tid; i < m; i += nt) S[j * m + i] /= p;
    __syncthreads();
    const int r = m - j - 1;
    for (int q = tid; q < r * r; q += nt) {
      const int c = j + 1 + q / r, i = j + 1 + q % r;
      if (i >= c) S[c * m + i] -= S[j * m + i] * S[j * m + c];
    }
    __syncthreads();
  }
  T *F = arena + off;
  for (int q = tid; q < m * m; q += nt) {
    const int c = q / m, i = q % m;
    if (i >= c) F[q] = S[q];
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

// task = {front, first column of the chunk}
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_assemble_large(MfView v, const int2 *__restrict__ tasks, const double *__restrict__ vals,
                  T *__restrict__ arena) {
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
    for (int b = blo + wid; b < bhi; b += nw) {
      const int pb = rel[b];
      for (int a = b + lane; a < rc; a += 32) F[(int64_t)pb * m + rel[a]] += U[(int64_t)b * mc + a];
    }
    __syncthreads();
  }
}

// Panel at column j0 of a large front in two launches: mf_diag factors the
// jb x jb diagonal block of every listed front (one CTA each, in shared
// memory); mf_panel then solves L21 = A21 L11^-T for row chunks of kPanelRows
// rows (task = {front, first row of the chunk}), many CTAs per front.
constexpr int kPanelRows = 256;

template <typename T>
__device__ __forceinline__ void chol_small_smem(T (*D)[kNB + 1], int jb, int *status) {
  // right-looking Cholesky of D[0..jb)[0..jb) (lower, D[row][col]) by one CTA
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
    for (int q = tid; q < (jb - j - 1) * (jb - j - 1); q += blockDim.x) {
      int i = j + 1 + q / (jb - j - 1), c = j + 1 + q % (jb - j - 1);
      if (i >= c) D[i][c] -= D[i][j] * D[c][j];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_diag(MfView v, const int *__restrict__ fronts, int j0, T *__restrict__ arena, int *__restrict__ status) {
  __shared__ T D[kNB][kNB + 1];
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  const int jb = min(kNB, k - j0);
  T *F = arena + v.f_off[f];
  const int tid = threadIdx.x;
  for (int q = tid; q < jb * jb; q += kMfThreads) {
    int c = q / jb, i = q % jb;  // column-major walk: coalesced over i
    D[i][c] = i >= c ? F[(int64_t)(j0 + c) * m + j0 + i] : T(0);
  }
  __syncthreads();
  chol_small_smem<T>(D, jb, status);
  for (int q = tid; q < jb * jb; q += kMfThreads) {
    int c = q / jb, i = q % jb;
    if (i >= c) F[(int64_t)(j0 + c) * m + j0 + i] = D[i][c];
  }
}

template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_panel(MfView v, const int2 *__restrict__ tasks, int j0, T *__restrict__ arena) {
  __shared__ T D[kNB][kNB + 1];
  const int f = tasks[blockIdx.x].x, r0 = tasks[blockIdx.x].y;
  const int m = v.f_m[f], k = v.f_k[f];
  const int jb = min(kNB, k - j0);
  T *F = arena + v.f_off[f];
  const int tid = threadIdx.x;
  for (int q = tid; q < jb * jb; q += kMfThreads) {  // the factored diagonal block
    int c = q / jb, i = q % jb;
    D[i][c] = i >= c ? F[(int64_t)(j0 + c) * m + j0 + i] : T(0);
  }
  __syncthreads();
  const int rb = max(r0, j0 + jb), re = min(r0 + kPanelRows, m);
  for (int i = rb + tid; i < re; i += kMfThreads) {
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

// one 64x64 tile of the trailing update after the panel at j0;
// task = {front, (ti << 16) | tj}, tiles relative to column j0 + jb
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_update(MfView v, const int2 *__restrict__ tasks, int j0, T *__restrict__ arena) {
  __shared__ T As[kNB][kTile];
  __shared__ T Bs[kNB][kTile];
  const int f = tasks[blockIdx.x].x;
  const int ti = tasks[blockIdx.x].y >> 16, tj = tasks[blockIdx.x].y & 0xffff;
  const int m = v.f_m[f], k = v.f_k[f];
  const int jb = min(kNB, k - j0);
  T *F = arena + v.f_off[f];
  const int c0 = j0 + jb;
  const int r0 = c0 + ti * kTile, cc0 = c0 + tj * kTile;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int q = tid; q < kNB * kTile; q += kMfThreads) {
    int t = q / kTile, r = q % kTile;
    T a = T(0), b = T(0);
    if (t < jb) {
      if (r0 + r < m) a = F[(int64_t)(j0 + t) * m + r0 + r];
      if (cc0 + r < m) b = F[(int64_t)(j0 + t) * m + cc0 + r];
    }
    As[t][r] = a;
    Bs[t][r] = b;
  }
  __syncthreads();
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = T(0);
  for (int t = 0; t < jb; t++) {
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
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const int col = cc0 + ty + 16 * b;
    if (col >= m) continue;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int row = r0 + tx + 16 * a;
      if (row < m && row >= col) F[(int64_t)col * m + row] -= acc[a][b];
    }
  }
}

// ---------------------------------------------------------------------------
// multifrontal solves
// ---------------------------------------------------------------------------
// Solves keep the front's work vector w (length m) in shared memory when it
// fits (`wglob` otherwise) and walk the pivots in blocks of 32 columns: one
// warp solves the 32x32 triangle, all warps apply the block to the rest.
constexpr int kSB = 32;

// forward: w = [b_piv ; 0] + children's update vectors; y = L11^-1 w1;
// this front's update vector = w2 - L21 y
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_fwd_level(MfView v, const int *__restrict__ fronts, const T *__restrict__ arena,
             T *__restrict__ xl, T *__restrict__ uvec, T *__restrict__ wglob, int use_smem) {
  extern __shared__ unsigned char smem_raw[];
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  const T *F = arena + v.f_off[f];
  T *w = use_smem ? reinterpret_cast<T *>(smem_raw) : wglob + v.f_woff[f];
  T *x = xl + v.f_xoff[f] + v.f_p0[f];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < m; i += kMfThreads) w[i] = i < k ? x[i] : T(0);
  __syncthreads();
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int rc = v.f_m[c] - v.f_k[c];
    const int *rel = v.relmap + v.f_relmap[c];
    const T *u = uvec + v.f_uoff[c];
    for (int a = tid; a < rc; a += kMfThreads) w[rel[a]] += u[a];
    __syncthreads();
  }
  __shared__ T Dg[kSB][kSB + 1];
  for (int J0 = 0; J0 < k; J0 += kSB) {
    const int jb = min(kSB, k - J0);
    for (int q = tid; q < jb * jb; q += kMfThreads) {
      int c = q / jb, i = q % jb;
      Dg[i][c] = F[(int64_t)(J0 + c) * m + J0 + i];
    }
    __syncthreads();
    if (wid == 0) {
      T wl = lane < jb ? w[J0 + lane] : T(0);
      for (int j = 0; j < jb; j++) {
        const T yj = __shfl_sync(0xffffffffu, wl, j) / Dg[j][j];
        if (lane == j) wl = yj;
        if (lane > j && lane < jb) wl -= Dg[lane][j] * yj;
      }
      if (lane < jb) w[J0 + lane] = wl;
    }
    __syncthreads();
    for (int i = J0 + jb + tid; i < m; i += kMfThreads) {
      T s = T(0);
#pragma unroll 8
      for (int j = 0; j < jb; j++) s += F[(int64_t)(J0 + j) * m + i] * w[J0 + j];
      w[i] -= s;
    }
    __syncthreads();
  }
  for (int i = tid; i < k; i += kMfThreads) x[i] = w[i];
  T *u = uvec + v.f_uoff[f];
  for (int a = tid; a < m - k; a += kMfThreads) u[a] = w[k + a];
}

// backward: x_piv = L11^-T (y - L21^T x_rows)
template <typename T>
__global__ void __launch_bounds__(kMfThreads)
mf_bwd_level(MfView v, const int *__restrict__ fronts, const T *__restrict__ arena,
             T *__restrict__ xl, T *__restrict__ wglob, int use_smem) {
  extern __shared__ unsigned char smem_raw[];
  const int f = fronts[blockIdx.x];
  const int m = v.f_m[f], k = v.f_k[f];
  const T *F = arena + v.f_off[f];
  T *w = use_smem ? reinterpret_cast<T *>(smem_raw) : wglob + v.f_woff[f];
  T *xb = xl + v.f_xoff[f];
  const int *rows = v.rows + v.f_rows[f];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = kMfThreads / 32;
  for (int i = tid; i < m; i += kMfThreads) w[i] = xb[rows[i]];
  __syncthreads();
  // contributions of the already solved update rows
  for (int j = wid; j < k; j += nw) {
    T s = T(0);
    for (int i = k + lane; i < m; i += 32) s += F[(int64_t)j * m + i] * w[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) w[j] -= s;
  }
  __syncthreads();
  __shared__ T Dg[kSB][kSB + 1];
  for (int J1 = k; J1 > 0; J1 -= kSB) {
    const int J0 = max(0, J1 - kSB), jb = J1 - J0;
    for (int q = tid; q < jb * jb; q += kMfThreads) {
      int c = q / jb, i = q % jb;
      Dg[i][c] = F[(int64_t)(J0 + c) * m + J0 + i];
    }
    __syncthreads();
    if (wid == 0) {
      T wl = lane < jb ? w[J0 + lane] : T(0);
      for (int j = jb - 1; j >= 0; j--) {
        // x_j = (w_j - sum_{i>j in block} L(i,j) x_i) / L(j,j); the sum is
        // accumulated into wl of lane j by the lanes of the solved rows
        T contrib = (lane > j && lane < jb) ? Dg[lane][j] * wl : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) contrib += __shfl_down_sync(0xffffffffu, contrib, o);
        contrib = __shfl_sync(0xffffffffu, contrib, 0);
        if (lane == j) wl = (wl - contrib) / Dg[j][j];
      }
      if (lane < jb) w[J0 + lane] = wl;
    }
    __syncthreads();
    // columns left of the block: w_j -= sum_{i in block} L(i,j) x_i
    for (int j = wid; j < J0; j += nw) {
      T s = lane < jb ? F[(int64_t)j * m + J0 + lane] * w[J0 + lane] : T(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) w[j] -= s;
    }
    __syncthreads();
  }
  for (int i = tid; i < k; i += kMfThreads) xb[rows[i]] = w[i];
}

// ---------------------------------------------------------------------------
// Tiled solve layout of large fronts.  After the factorisation every 32-column
// block J of a large front (columns 32J .. 32J+jb) is stored as a contiguous
// run:
//   Dinv_J                        inverse of the jb x jb diagonal block (32 x 32)
//   run of rank 0, rank 1, ...    32x32 tiles tile(R, J), row-major, for the
//                                 row blocks R >= J owned by that cluster rank
//                                 (R % C == rank), ascending R
// Entries of the diagonal block (and rows past m) are zero in tile(J, J).
// The solves of one front are split over a thread-block cluster of C CTAs:
// CTA q owns the row blocks R with R % C == q, keeps their part of the work
// vector in shared memory and streams its own tile run with cp.async, G tiles
// per stage; the CTAs exchange the 32-value block solutions through
// distributed shared memory with one cluster barrier per column block.
// C = 1 is the plain one-CTA solve.
// ---------------------------------------------------------------------------
constexpr int kTileThreads = 256;
template <typename T> struct TilePipe;
template <> struct TilePipe<float> { static constexpr int G = 4, S = 4; };   // 16 KB stages, 64 KB ring
template <> struct TilePipe<double> { static constexpr int G = 2, S = 4; };  // 16 KB stages, 64 KB ring

struct PackView {
  const int *blk_front;        // block -> front
  const int *blk_j;            // block -> J
  const int *f_blk;            // front -> first block (large fronts), -1 otherwise
  const int64_t *blk_off;      // block -> element offset in the packed buffer
  const int *f_C;              // front -> cluster size of its solves
};

__host__ __device__ __forceinline__ int first_owned(int J, int C, int q) {  // smallest R >= J, R % C == q
  return J + ((q - J % C) % C + C) % C;
}
__host__ __device__ __forceinline__ int owned_count(int J, int nR, int C, int q) {
  const int f0 = first_owned(J, C, q);
  return f0 < nR ? (nR - f0 + C - 1) / C : 0;
}

// one CTA per column block: invert the diagonal block, copy the tiles
template <typename T>
__global__ void __launch_bounds__(256)
mf_pack(MfView v, PackView pk, const T *__restrict__ arena, T *__restrict__ packed) {
  __shared__ T L[32][33];
  __shared__ T X[32][33];
  const int b = blockIdx.x;
  const int f = pk.blk_front[b], J = pk.blk_j[b];
  const int m = v.f_m[f], k = v.f_k[f], C = pk.f_C[f];
  const int J0 = 32 * J, jb = min(32, k - J0);
  const T *F = arena + v.f_off[f];
  T *dst = packed + pk.blk_off[b];
  const int tid = threadIdx.x;
  for (int q = tid; q < 32 * 32; q += 256) {
    int c = q / 32, i = q % 32;
    L[i][c] = (i < jb && c < jb && i >= c) ? F[(int64_t)(J0 + c) * m + J0 + i] : T(0);
    X[i][c] = T(0);
  }
  __syncthreads();
  if (tid < jb) {  // column tid of the inverse of a lower triangular block
    const int c = tid;
    X[c][c] = T(1) / L[c][c];
    for (int i = c + 1; i < jb; i++) {
      T sum = T(0);
      for (int t = c; t < i; t++) sum += L[i][t] * X[t][c];
      X[i][c] = -sum / L[i][i];
    }
  }
  __syncthreads();
  for (int q = tid; q < 32 * 32; q += 256) dst[q] = X[q / 32][q % 32];
  const int nR = (m + 31) / 32;
  for (int R = J; R < nR; R++) {
    const int rank = R % C;
    int pos = 0;
    for (int r = 0; r < rank; r++) pos += owned_count(J, nR, C, r);
    pos += (R - first_owned(J, C, rank)) / C;
    T *td = dst + 1024 * (int64_t)(1 + pos);
    for (int q = tid; q < 32 * 32; q += 256) {
      const int rr = q / 32, c = q % 32;  // row-major tile
      const int row = 32 * R + rr;
      td[q] = (c < jb && row >= J0 + jb && row < m) ? F[(int64_t)(J0 + c) * m + row] : T(0);
    }
  }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <typename T>
__device__ __forceinline__ void issue_chunk(T *slot, const T *src, int elems) {
  const int n16 = elems * (int)sizeof(T) / 16;
  for (int q = threadIdx.x; q < n16; q += blockDim.x)
    cp_async16(reinterpret_cast<char *>(slot) + 16 * q, reinterpret_cast<const char *>(src) + 16 * q);
}

// distributed shared memory helpers (cluster rank of this CTA; remote loads)
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
template <typename T>
__device__ __forceinline__ T ld_dsmem(const T *local_addr, unsigned rank);
template <>
__device__ __forceinline__ double ld_dsmem<double>(const double *p, unsigned rank) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(p), ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(sa), "r"(rank));
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];\n" : "=d"(v) : "r"(ra) : "memory");
  return v;
}
template <>
__device__ __forceinline__ float ld_dsmem<float>(const float *p, unsigned rank) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(p), ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(sa), "r"(rank));
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];\n" : "=f"(v) : "r"(ra) : "memory");
  return v;
}

// The chunks one CTA consumes, in order.  Forward: for J ascending, Dinv_J
// (if the CTA owns row block J) then its tile run of block J in pieces of G
// tiles.  Backward: for J descending, the tile run, then Dinv_J if owned.
template <typename T>
struct ChunkCursor {
  const int64_t *blk_off;
  int fb, nb, nR, C, q;
  bool fwd;
  int J, t0, cnt;   // current block, first tile of the piece, tiles owned in block J
  bool dinv;        // current chunk is Dinv_J
  __device__ void setup_block() {
    cnt = owned_count(J, nR, C, q);
    t0 = 0;
    dinv = fwd ? (J % C == q) : false;
    if (!fwd && cnt == 0) dinv = (J % C == q);
  }
  __device__ void start(const int64_t *bo, int fb_, int nb_, int nR_, int C_, int q_, bool fwd_) {
    blk_off = bo; fb = fb_; nb = nb_; nR = nR_; C = C_; q = q_; fwd = fwd_;
    J = fwd ? 0 : nb - 1;
    setup_block();
    settle();
  }
  __device__ bool valid() const { return J >= 0 && J < nb; }
  __device__ bool has_chunk() const { return dinv || t0 < cnt; }
  __device__ void settle() {  // skip blocks without a chunk for this CTA
    while (valid() && !has_chunk()) {
      J += fwd ? 1 : -1;
      if (valid()) setup_block();
    }
  }
  __device__ void advance() {
    constexpr int G = TilePipe<T>::G;
    if (fwd) {
      if (dinv) dinv = false;
      else t0 += G;
    } else {
      if (t0 < cnt) {
        t0 += G;
        if (t0 >= cnt) dinv = (J % C == q);
      } else {
        dinv = false;
      }
    }
    if (!has_chunk()) {
      J += fwd ? 1 : -1;
      if (valid()) setup_block();
    }
    settle();
  }
  __device__ int ntiles() const { return min(TilePipe<T>::G, cnt - t0); }
  __device__ const T *src(const T *packed, int &elems) const {
    const T *base = packed + blk_off[fb + J];
    if (dinv) { elems = 1024; return base; }
    int pre = 0;
    for (int r = 0; r < q; r++) pre += owned_count(J, nR, C, r);
    elems = 1024 * ntiles();
    return base + 1024 * (int64_t)(1 + pre + t0);
  }
};

// forward solve, grid = nfronts * C, cluster (C,1,1)
template <typename T, int C>
__global__ void __launch_bounds__(kTileThreads)
mf_fwd_tiles(MfView v, PackView pk, const int *__restrict__ fronts, const T *__restrict__ packed,
             T *__restrict__ xl, T *__restrict__ uvec) {
  constexpr int G = TilePipe<T>::G, S = TilePipe<T>::S, SLOT = G * 1024;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *ring = reinterpret_cast<T *>(smem_raw);            // S slots of G tiles
  T *wloc = ring + S * SLOT;                            // owned row blocks x 32
  __shared__ T ybuf[2][32];
  __shared__ T yJ[32];
  const unsigned q = C > 1 ? cluster_rank() : 0;
  const int f = fronts[blockIdx.x / C];
  const int m = v.f_m[f], k = v.f_k[f];
  const int fb = pk.f_blk[f], nb = (k + 31) / 32, nR = (m + 31) / 32;
  const int tid = threadIdx.x;
  T *x = xl + v.f_xoff[f] + v.f_p0[f];
  auto loc = [&](int row) -> T & { return wloc[(row / 32) / C * 32 + row % 32]; };
  auto owned = [&](int row) { return (row / 32) % C == (int)q; };
  ChunkCursor<T> cur;
  cur.start(pk.blk_off, fb, nb, nR, C, (int)q, true);
  for (int st = 0; st < S; st++) {
    if (cur.valid()) {
      int el;
      const T *sp = cur.src(packed, el);
      issue_chunk<T>(ring + st * SLOT, sp, el);
      cur.advance();
    }
    cp_async_commit();
  }
  const int nown = (nR - (int)q + C - 1) / C;
  for (int i = tid; i < nown * 32; i += kTileThreads) {
    const int row = ((i / 32) * C + (int)q) * 32 + i % 32;
    wloc[i] = row < k ? x[row] : T(0);
  }
  __syncthreads();
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int rc = v.f_m[c] - v.f_k[c];
    const int *rel = v.relmap + v.f_relmap[c];
    const T *u = uvec + v.f_uoff[c];
    for (int a = tid; a < rc; a += kTileThreads) {
      const int row = rel[a];
      if (owned(row)) loc(row) += u[a];
    }
    __syncthreads();
  }
  int slot = 0;
  auto refill = [&]() {
    if (cur.valid()) {
      int el;
      const T *sp = cur.src(packed, el);
      issue_chunk<T>(ring + slot * SLOT, sp, el);
      cur.advance();
    }
    cp_async_commit();
    slot = (slot + 1) % S;
  };
  for (int J = 0; J < nb; J++) {
    const int J0 = 32 * J, jb = min(32, k - J0);
    if (J % C == (int)q) {  // owner: y_J = Dinv_J w_J (its Dinv is the next chunk)
      cp_async_wait<S - 1>();
      __syncthreads();
      const T *Sm = ring + slot * SLOT;
      if (tid < 32) {
        T sum = T(0);
        if (tid < jb)
          for (int sidx = 0; sidx <= tid; sidx++) sum += Sm[tid * 32 + sidx] * loc(J0 + sidx);
        ybuf[J & 1][tid] = sum;  // zero past jb: the padded tile columns multiply it
      }
      __syncthreads();
      if (tid < jb) loc(J0 + tid) = ybuf[J & 1][tid];
      __syncthreads();
      refill();
    }
    if (C > 1) cluster_sync();
    if (tid < 32) yJ[tid] = C > 1 ? ld_dsmem<T>(&ybuf[J & 1][tid], (unsigned)(J % C)) : ybuf[J & 1][tid];
    __syncthreads();
    const int cnt = owned_count(J, nR, C, (int)q);
    const int f0 = first_owned(J, C, (int)q);
    for (int t0 = 0; t0 < cnt; t0 += G) {
      cp_async_wait<S - 1>();
      __syncthreads();
      const T *Sm = ring + slot * SLOT;
      const int nt = min(G, cnt - t0);
      const int rr = tid >> 3, c4 = (tid & 7) * 4;  // 8 threads per tile row
      for (int t = 0; t < nt; t++) {
        const T *tl = Sm + t * 1024;
        T part = tl[rr * 32 + c4] * yJ[c4] + tl[rr * 32 + c4 + 1] * yJ[c4 + 1] +
                 tl[rr * 32 + c4 + 2] * yJ[c4 + 2] + tl[rr * 32 + c4 + 3] * yJ[c4 + 3];
        part += __shfl_down_sync(0xffffffffu, part, 4, 8);
        part += __shfl_down_sync(0xffffffffu, part, 2, 8);
        part += __shfl_down_sync(0xffffffffu, part, 1, 8);
        const int row = 32 * (f0 + (t0 + t) * C) + rr;
        if ((tid & 7) == 0 && row < m) loc(row) -= part;
      }
      __syncthreads();
      refill();
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  for (int i = tid; i < nown * 32; i += kTileThreads) {
    const int row = ((i / 32) * C + (int)q) * 32 + i % 32;
    if (row < k) x[row] = wloc[i];
    else if (row < m) uvec[v.f_uoff[f] + row - k] = wloc[i];
  }
  if (C > 1) cluster_sync();  // no CTA leaves while its shared memory may still be read
}

// backward solve, grid = nfronts * C, cluster (C,1,1)
template <typename T, int C>
__global__ void __launch_bounds__(kTileThreads)
mf_bwd_tiles(MfView v, PackView pk, const int *__restrict__ fronts, const T *__restrict__ packed,
             T *__restrict__ xl) {
  constexpr int G = TilePipe<T>::G, S = TilePipe<T>::S, SLOT = G * 1024;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *ring = reinterpret_cast<T *>(smem_raw);
  T *wloc = ring + S * SLOT;
  __shared__ T part[2][32];
  __shared__ T red[8][32];
  __shared__ T tJ[32];
  const unsigned q = C > 1 ? cluster_rank() : 0;
  const int f = fronts[blockIdx.x / C];
  const int m = v.f_m[f], k = v.f_k[f];
  const int fb = pk.f_blk[f], nb = (k + 31) / 32, nR = (m + 31) / 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  T *xb = xl + v.f_xoff[f];
  const int *rows = v.rows + v.f_rows[f];
  auto loc = [&](int row) -> T & { return wloc[(row / 32) / C * 32 + row % 32]; };
  ChunkCursor<T> cur;
  cur.start(pk.blk_off, fb, nb, nR, C, (int)q, false);
  for (int st = 0; st < S; st++) {
    if (cur.valid()) {
      int el;
      const T *sp = cur.src(packed, el);
      issue_chunk<T>(ring + st * SLOT, sp, el);
      cur.advance();
    }
    cp_async_commit();
  }
  const int nown = (nR - (int)q + C - 1) / C;
  for (int i = tid; i < nown * 32; i += kTileThreads) {
    const int row = ((i / 32) * C + (int)q) * 32 + i % 32;
    wloc[i] = row < m ? xb[rows[row]] : T(0);
  }
  __syncthreads();
  int slot = 0;
  auto refill = [&]() {
    if (cur.valid()) {
      int el;
      const T *sp = cur.src(packed, el);
      issue_chunk<T>(ring + slot * SLOT, sp, el);
      cur.advance();
    }
    cp_async_commit();
    slot = (slot + 1) % S;
  };
  for (int J = nb - 1; J >= 0; J--) {
    const int J0 = 32 * J, jb = min(32, k - J0);
    // partial t_J = sum over owned R >= J of tile(R,J)^T x_R
    T acc = T(0);  // thread (wid, lane): column lane, rows wid*4 .. wid*4+3 of each tile
    const int cnt = owned_count(J, nR, C, (int)q);
    const int f0 = first_owned(J, C, (int)q);
    for (int t0 = 0; t0 < cnt; t0 += G) {
      cp_async_wait<S - 1>();
      __syncthreads();
      const T *Sm = ring + slot * SLOT;
      const int nt = min(G, cnt - t0);
      for (int t = 0; t < nt; t++) {
        const T *tl = Sm + t * 1024;
        const int R = f0 + (t0 + t) * C;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int rr = wid * 4 + u;
          const int row = 32 * R + rr;
          if (row < m) acc += tl[rr * 32 + lane] * loc(row);
        }
      }
      __syncthreads();
      refill();
    }
    red[wid][lane] = acc;
    __syncthreads();
    if (tid < 32) {
      T s = T(0);
#pragma unroll
      for (int w = 0; w < 8; w++) s += red[w][tid];
      part[J & 1][tid] = s;
    }
    __syncthreads();
    if (C > 1) cluster_sync();
    if (J % C == (int)q) {  // owner: t_J = y_J - sum of partials; x_J = Dinv_J^T t_J
      if (tid < 32) {
        T s = T(0);
        for (int r = 0; r < C; r++) s += C > 1 ? ld_dsmem<T>(&part[J & 1][tid], (unsigned)r) : part[J & 1][tid];
        tJ[tid] = tid < jb ? loc(J0 + tid) - s : T(0);
      }
      cp_async_wait<S - 1>();
      __syncthreads();
      const T *Sm = ring + slot * SLOT;
      if (tid < jb) {
        T sum = T(0);
        for (int sidx = tid; sidx < jb; sidx++) sum += Sm[sidx * 32 + tid] * tJ[sidx];
        loc(J0 + tid) = sum;
      }
      __syncthreads();
      refill();
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  for (int i = tid; i < nown * 32; i += kTileThreads) {
    const int row = ((i / 32) * C + (int)q) * 32 + i % 32;
    if (row < k) xb[rows[row]] = wloc[i];
  }
  if (C > 1) cluster_sync();
}

// ---------------------------------------------------------------------------
// Small fronts (m <= 128): one warp per front.  The front's factor columns
// (m x k, contiguous in the arena) are staged in shared memory with cp.async,
// then the pivots are eliminated from shared memory.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int round4(int x) { return (x + 3) & ~3; }

template <typename T>
__device__ __forceinline__ void stage_factor_warp(T *Ls, const T *src, int elems) {
  const int lane = threadIdx.x & 31;
  const int n16 = (elems * (int)sizeof(T) + 15) / 16;
  for (int q = lane; q < n16; q += 32)
    cp_async16(reinterpret_cast<char *>(Ls) + 16 * q, reinterpret_cast<const char *>(src) + 16 * q);
  cp_async_commit();
}

template <typename T>
__global__ void __launch_bounds__(256)
mf_fwd_warp(MfView v, const int *__restrict__ fronts, int nf, const T *__restrict__ arena,
            T *__restrict__ xl, T *__restrict__ uvec, int per_warp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int gw = blockIdx.x * nw + wid;
  if (gw >= nf) return;  // warp-level kernel: no block barriers below
  T *Ls = reinterpret_cast<T *>(smem_raw) + (size_t)wid * per_warp;
  const int f = fronts[gw];
  const int m = v.f_m[f], k = v.f_k[f];
  T *w = Ls + round4(m * k);
  stage_factor_warp<T>(Ls, arena + v.f_off[f], m * k);
  T *x = xl + v.f_xoff[f] + v.f_p0[f];
  for (int i = lane; i < m; i += 32) w[i] = i < k ? x[i] : T(0);
  __syncwarp();
  for (int ci = v.f_child_ptr[f]; ci < v.f_child_ptr[f + 1]; ci++) {
    const int c = v.f_children[ci];
    const int rc = v.f_m[c] - v.f_k[c];
    const int *rel = v.relmap + v.f_relmap[c];
    const T *u = uvec + v.f_uoff[c];
    for (int a = lane; a < rc; a += 32) w[rel[a]] += u[a];
    __syncwarp();
  }
  cp_async_wait<0>();
  __syncwarp();
  for (int j = 0; j < k; j++) {
    const T yj = w[j] / Ls[j * m + j];
    __syncwarp();
    for (int i = j + 1 + lane; i < m; i += 32) w[i] -= Ls[j * m + i] * yj;
    if (lane == 0) w[j] = yj;
    __syncwarp();
  }
  for (int i = lane; i < k; i += 32) x[i] = w[i];
  T *u = uvec + v.f_uoff[f];
  for (int a = lane; a < m - k; a += 32) u[a] = w[k + a];
}

template <typename T>
__global__ void __launch_bounds__(256)
mf_bwd_warp(MfView v, const int *__restrict__ fronts, int nf, const T *__restrict__ arena,
            T *__restrict__ xl, int per_warp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int gw = blockIdx.x * nw + wid;
  if (gw >= nf) return;
  T *Ls = reinterpret_cast<T *>(smem_raw) + (size_t)wid * per_warp;
  const int f = fronts[gw];
  const int m = v.f_m[f], k = v.f_k[f];
  T *w = Ls + round4(m * k);
  stage_factor_warp<T>(Ls, arena + v.f_off[f], m * k);
  T *xb = xl + v.f_xoff[f];
  const int *rows = v.rows + v.f_rows[f];
  for (int i = lane; i < m; i += 32) w[i] = xb[rows[i]];
  cp_async_wait<0>();
  __syncwarp();
  for (int j = k - 1; j >= 0; j--) {
    T sum = T(0);
    for (int i = j + 1 + lane; i < m; i += 32) sum += Ls[j * m + i] * w[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane == 0) w[j] = (w[j] - sum) / Ls[j * m + j];
    __syncwarp();
  }
  for (int i = lane; i < k; i += 32) xb[rows[i]] = w[i];
}

// ---------------------------------------------------------------------------
// Schwarz gather / pull sum and coarse transfer
// ---------------------------------------------------------------------------
template <typename T>
__global__ void gather_subdomains(const double *__restrict__ r, const int *__restrict__ gidx,
                                  T *__restrict__ xl, int64_t len) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < len;
       p += (int64_t)gridDim.x * blockDim.x)
    xl[p] = (T)r[gidx[p]];
}

// crhs (in the coarse batch's local numbering) = R r
template <typename TR>
__global__ void restrict_to_coarse(const int64_t *__restrict__ Rp, const int *__restrict__ Rc,
                                   const TR *__restrict__ Rv, const double *__restrict__ r,
                                   const int *__restrict__ cpos, double *__restrict__ xc, int nc) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < nc; a += warps) {
    double s = 0.0;
    for (int64_t e = Rp[a] + lane; e < Rp[a + 1]; e += 32) s += (double)Rv[e] * r[Rc[e]];
    s = warp_sum(s);
    if (lane == 0) xc[cpos[a]] = s;
  }
}

// z_g = (sum of subdomain solutions at g, in subdomain order) + (P x_c)_g ;
// partial sums of r.z (and of r.z_old for the flexible variant).  One thread
// per node; Pcp holds coarse-vector positions (composed at setup).
template <typename T, typename TP>
__global__ void __launch_bounds__(kVecThreads)
pull_prolong_dot(int n, const int64_t *__restrict__ pull_ptr, const int64_t *__restrict__ pull_idx,
                 const T *__restrict__ xl, const int64_t *__restrict__ Pp, const int *__restrict__ Pcp,
                 const TP *__restrict__ Pv, const double *__restrict__ xc,
                 int mode, const double *__restrict__ r, double *__restrict__ z,
                 double *__restrict__ zold, double *__restrict__ part_rz, double *__restrict__ part_rzo) {
  // mode bit 0: fine subdomains on; bit 1: coarse on; bit 2: identity fine (z=r);
  // bit 3: keep z_old and produce r.z_old
  __shared__ double sh[32];
  double srz = 0.0, srzo = 0.0;
  for (int g = blockIdx.x * kVecThreads + threadIdx.x; g < n; g += gridDim.x * kVecThreads) {
    double sv = 0.0;
    if (mode & 4) {
      sv = r[g];
    } else if (mode & 1) {
      const int64_t q0 = pull_ptr[g], q1 = pull_ptr[g + 1];
      for (int64_t q = q0; q < q1; q++) sv = sv + (double)xl[pull_idx[q]];
    }
    if (mode & 2) {
      const int64_t e0 = Pp[g], e1 = Pp[g + 1];
      TP t = TP(0);
      int64_t e = e0;
      for (; e + 4 <= e1; e += 4) {  // independent loads in flight
        const int c0 = Pcp[e], c1 = Pcp[e + 1], c2 = Pcp[e + 2], c3 = Pcp[e + 3];
        const TP v0 = Pv[e], v1 = Pv[e + 1], v2 = Pv[e + 2], v3 = Pv[e + 3];
        const TP x0 = (TP)xc[c0], x1 = (TP)xc[c1], x2 = (TP)xc[c2], x3 = (TP)xc[c3];
        t += v0 * x0;
        t += v1 * x1;
        t += v2 * x2;
        t += v3 * x3;
      }
      for (; e < e1; e++) t += Pv[e] * (TP)xc[Pcp[e]];
      sv = sv + (double)t;
    }
    const double rg = r[g];
    if (mode & 8) {
      srzo += rg * zold[g];
      zold[g] = sv;
    }
    z[g] = sv;
    srz += rg * sv;
  }
  double b = block_sum<kVecThreads>(srz, sh);
  if (threadIdx.x == 0) part_rz[blockIdx.x] = b;
  if (mode & 8) {
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
      if (LANES == 1) {  // short rows: all loads of a row issued before the sums
        for (; e + 4 <= e1; e += 4) {
          const int c0 = Ac[e], c1 = Ac[e + 1], c2 = Ac[e + 2], c3 = Ac[e + 3];
          const double a0 = Av[e], a1 = Av[e + 1], a2 = Av[e + 2], a3 = Av[e + 3];
          const double p0 = p[c0], p1 = p[c1], p2 = p[c2], p3 = p[c3];
          s = __fma_rn(a0, p0, s);
          s = __fma_rn(a1, p1, s);
          s = __fma_rn(a2, p2, s);
          s = __fma_rn(a3, p3, s);
        }
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

}  // namespace dg
