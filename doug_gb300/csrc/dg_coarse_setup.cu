// Coarse-level setup on the GPU: prolongator smoothing (IntRestBuild,
// src/coarse/CoarseMtx.F90:128-233, 418-427), the Galerkin product
// (CoarseMtxBuild, CoarseMtx.F90:476-516) through the reference's
// first-touch SpGEMM (SpMtx_AB, src/datatypes/SpMtx/SpMtx_op_AB.f90:39-200),
// and the stable re-bucketings between them (SpMtx_arrange,
// src/datatypes/SpMtx/SpMtx_arrangement.F90:58-292).
//
// The outputs are bit-for-bit those of the host setup (and of the oracle):
//   * SpGEMM: row i of C lists its columns in first-touch order (A's row
//     entries in order, then B's row entries in order); each value is
//     the running sum c = c + a*b in that order, every product and sum
//     rounded on its own (__dmul_rn, __dadd_rn: no fused multiply-add);
//     explicit zeros stay.  One warp per row: the lanes take 32 entries of
//     B's row at a time, look their columns up in a hash table of the row
//     (shared memory, or global memory for very long rows), and new columns
//     get the next positions in lane order (ballot + prefix count), which is
//     the sequential order because a row of B holds every column at most
//     once.  Rows of B with repeated columns switch the product to one lane
//     per row.  A symbolic pass counts each row, a scan places the rows,
//     the numeric pass repeats the walk and writes.
//   * transposes keep the stable order of the bucketing: every column's
//     entries are sorted by their position in the row-major input.
//   * the smoother S = I(1 - omega) - omega D^-1 A_strong with d_i = a_ii +
//     sum of i's weak entries, weak entries kept as explicit zeros.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "host/setup.hpp"

namespace dg {
namespace cs {

struct Err {
  cudaError_t e;
  const char *what;
};
#define CSK(call)                                         \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) throw Err{_e, #call};          \
  } while (0)

template <typename T>
struct Buf {
  T *p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf &) = delete;
  Buf &operator=(const Buf &) = delete;
  Buf(Buf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  Buf &operator=(Buf &&o) noexcept {
    if (p) cudaFree(p);
    p = o.p; n = o.n; o.p = nullptr; o.n = 0;
    return *this;
  }
  ~Buf() { if (p) cudaFree(p); }
  void alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; }
    n = count;
    CSK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
  }
  void upload(const T *src, size_t count) {
    alloc(count);
    if (count) CSK(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
  }
  void download(std::vector<T> &dst, size_t count) const {
    dst.resize(count);
    if (count) CSK(cudaMemcpy(dst.data(), p, count * sizeof(T), cudaMemcpyDeviceToHost));
  }
};

// CSR on the device (int64 row pointers, int32 columns, FP64 values)
struct DCsr {
  int nrows = 0, ncols = 0;
  int64_t nnz = 0;
  Buf<int64_t> ptr;
  Buf<int> col;
  Buf<double> val;
};

constexpr int kThreads = 256;

inline int nblocks(int64_t n, int per = kThreads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + per - 1) / per, 1 << 30));
}

// ---------------------------------------------------------------------------
// exclusive scan of int64 counts: out[0] = 0, out[i+1] = out[i] + in[i]
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;

__global__ void scan_block_sums(const int64_t *__restrict__ in, int64_t n, int64_t *__restrict__ sums) {
  __shared__ int64_t sh[kThreads];
  const int64_t b0 = (int64_t)blockIdx.x * kScanBlock;
  int64_t s = 0;
  for (int64_t i = b0 + threadIdx.x; i < min(n, b0 + kScanBlock); i += kThreads) s += in[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = sh[0];
}

// one block scans the block sums sequentially (a few thousand at most)
__global__ void scan_sums_serial(int64_t *sums, int nb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t run = 0;
  for (int b = 0; b < nb; b++) {
    const int64_t t = sums[b];
    sums[b] = run;
    run += t;
  }
  sums[nb] = run;
}

// within a block of kScanBlock entries: 4 entries per thread, a warp scan of
// the thread totals and a scan of the warp totals
__global__ void scan_apply(const int64_t *__restrict__ in, int64_t n, const int64_t *__restrict__ sums,
                           int64_t *__restrict__ out) {
  __shared__ int64_t warp_tot[kThreads / 32];
  const int64_t b0 = (int64_t)blockIdx.x * kScanBlock;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  int64_t v[4], tot = 0;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int64_t i = b0 + 4 * t + q;
    v[q] = i < n ? in[i] : 0;
    tot += v[q];
  }
  int64_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  int64_t wbase = 0;
  for (int w = 0; w < wid; w++) wbase += warp_tot[w];
  int64_t run = sums[blockIdx.x] + wbase + inc - tot;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int64_t i = b0 + 4 * t + q;
    if (i < n) out[i + 1] = run + v[q];
    run += v[q];
  }
  if (blockIdx.x == 0 && t == 0) out[0] = 0;
}

// out has n+1 entries
void exclusive_scan(const int64_t *in, int64_t n, int64_t *out, cudaStream_t s) {
  static_assert(kScanBlock == 4 * kThreads, "four entries per thread");
  const int nb = (int)std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  Buf<int64_t> sums;
  sums.alloc((size_t)nb + 1);
  scan_block_sums<<<nb, kThreads, 0, s>>>(in, n, sums.p);
  scan_sums_serial<<<1, 32, 0, s>>>(sums.p, nb);
  scan_apply<<<nb, kThreads, 0, s>>>(in, n, sums.p, out);
  CSK(cudaGetLastError());
  CSK(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// smoother S (same pattern as A): CoarseMtx.F90:154-233
// ---------------------------------------------------------------------------
__global__ void smoother_rows(int n, const int64_t *__restrict__ ptr, const int *__restrict__ col,
                              const double *__restrict__ val, const unsigned char *__restrict__ strong,
                              double omega, double *__restrict__ sval) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int64_t k = ptr[r]; k < ptr[r + 1]; k++)
    if (col[k] == r || !strong[k]) d = __dadd_rn(d, val[k]);
  const double diag = __dsub_rn(1.0, omega);
  const double w = __ddiv_rn(omega, d);
  for (int64_t k = ptr[r]; k < ptr[r + 1]; k++) {
    double v;
    if (col[k] == r) v = diag;
    else if (strong[k]) v = -__dmul_rn(w, val[k]);
    else v = 0.0;
    sval[k] = v;
  }
}

// ---------------------------------------------------------------------------
// stable transpose
// ---------------------------------------------------------------------------
__global__ void row_ids(int n, const int64_t *__restrict__ ptr, int *__restrict__ rid) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int64_t k = ptr[r]; k < ptr[r + 1]; k++) rid[k] = r;
}

__global__ void count_cols(int64_t nnz, const int *__restrict__ col, int64_t *__restrict__ cnt) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(reinterpret_cast<unsigned long long *>(&cnt[col[e]]), 1ull);
}

__global__ void place_cols(int64_t nnz, const int *__restrict__ col, const int64_t *__restrict__ tptr,
                           int64_t *__restrict__ fill, int64_t *__restrict__ slot) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = col[e];
    const unsigned long long q = atomicAdd(reinterpret_cast<unsigned long long *>(&fill[c]), 1ull);
    slot[tptr[c] + (int64_t)q] = e;
  }
}

// every column's entries in input order (insertion sort of their positions),
// then the transposed row ids and values
__global__ void order_cols(int nc, const int64_t *__restrict__ tptr, int64_t *__restrict__ slot,
                           const int *__restrict__ rid, const double *__restrict__ val, int *__restrict__ tcol,
                           double *__restrict__ tval) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int64_t a = tptr[c], b = tptr[c + 1];
  for (int64_t i = a + 1; i < b; i++) {
    const int64_t x = slot[i];
    int64_t j = i - 1;
    while (j >= a && slot[j] > x) { slot[j + 1] = slot[j]; j--; }
    slot[j + 1] = x;
  }
  for (int64_t i = a; i < b; i++) {
    const int64_t e = slot[i];
    tcol[i] = rid[e];
    tval[i] = val[e];
  }
}

// T = M^T with M's rows (nrows) becoming columns; the entries of every row
// of T come in the row-major order of M (stable bucketing by column)
void transpose(const DCsr &M, DCsr &T, cudaStream_t s) {
  T.nrows = M.ncols;
  T.ncols = M.nrows;
  T.nnz = M.nnz;
  Buf<int> rid;
  rid.alloc((size_t)M.nnz);
  row_ids<<<nblocks(M.nrows), kThreads, 0, s>>>(M.nrows, M.ptr.p, rid.p);
  Buf<int64_t> cnt, fill, slot;
  cnt.alloc((size_t)T.nrows);
  fill.alloc((size_t)T.nrows);
  CSK(cudaMemsetAsync(cnt.p, 0, sizeof(int64_t) * std::max<size_t>(1, (size_t)T.nrows), s));
  CSK(cudaMemsetAsync(fill.p, 0, sizeof(int64_t) * std::max<size_t>(1, (size_t)T.nrows), s));
  const int gs = nblocks(M.nnz);
  count_cols<<<std::min(gs, 4096), kThreads, 0, s>>>(M.nnz, M.col.p, cnt.p);
  CSK(cudaGetLastError());
  T.ptr.alloc((size_t)T.nrows + 1);
  exclusive_scan(cnt.p, T.nrows, T.ptr.p, s);
  slot.alloc((size_t)M.nnz);
  place_cols<<<std::min(gs, 4096), kThreads, 0, s>>>(M.nnz, M.col.p, T.ptr.p, fill.p, slot.p);
  T.col.alloc((size_t)M.nnz);
  T.val.alloc((size_t)M.nnz);
  order_cols<<<nblocks(T.nrows, 128), 128, 0, s>>>(T.nrows, T.ptr.p, slot.p, rid.p, M.val.p, T.col.p, T.val.p);
  CSK(cudaGetLastError());
  CSK(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// first-touch SpGEMM
// ---------------------------------------------------------------------------
// candidate count of row i: sum of the lengths of B's rows that A's row names
__global__ void row_bounds(int n, const int64_t *__restrict__ ap, const int *__restrict__ ac,
                           const int64_t *__restrict__ bp, int64_t *__restrict__ bound) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t s = 0;
  for (int64_t k = ap[i]; k < ap[i + 1]; k++) s += bp[ac[k] + 1] - bp[ac[k]];
  bound[i] = s;
}

__device__ __forceinline__ unsigned hash_col(int j, unsigned mask) { return ((unsigned)j * 2654435761u) & mask; }

// The walk over row i shared by the symbolic (NUMERIC false: count) and the
// numeric pass (write columns and values from out position base).  key /
// pos: the row's hash table, H slots (a power of two, at least twice the
// row's candidate count).  SERIAL: lane 0 alone walks (rows of B that may
// repeat a column).
template <bool NUMERIC, bool SERIAL>
__device__ __forceinline__ int64_t row_walk(int i, const int64_t *__restrict__ ap, const int *__restrict__ ac,
                                            const double *__restrict__ av, const int64_t *__restrict__ bp,
                                            const int *__restrict__ bc, const double *__restrict__ bv, int *key,
                                            int *pos, unsigned H, int64_t base, int *__restrict__ cc,
                                            double *__restrict__ cv) {
  const int lane = threadIdx.x & 31;
  for (unsigned t = lane; t < H; t += 32) key[t] = -1;
  __syncwarp();
  const unsigned mask = H - 1;
  int count = 0;
  if constexpr (SERIAL) {
    if (lane == 0) {
      for (int64_t k = ap[i]; k < ap[i + 1]; k++) {
        const int kk = ac[k];
        const double a = NUMERIC ? av[k] : 0.0;
        for (int64_t p = bp[kk]; p < bp[kk + 1]; p++) {
          const int j = bc[p];
          unsigned h = hash_col(j, mask);
          while (key[h] != -1 && key[h] != j) h = (h + 1) & mask;
          if (key[h] == -1) {
            key[h] = j;
            pos[h] = count;
            if (NUMERIC) { cc[base + count] = j; cv[base + count] = __dmul_rn(a, bv[p]); }
            count++;
          } else if (NUMERIC) {
            const int64_t q = base + pos[h];
            cv[q] = __dadd_rn(cv[q], __dmul_rn(a, bv[p]));
          }
        }
      }
    }
    count = __shfl_sync(0xffffffffu, count, 0);
    return count;
  } else {
  for (int64_t k = ap[i]; k < ap[i + 1]; k++) {
    const int kk = ac[k];
    const double a = NUMERIC ? av[k] : 0.0;
    const int64_t p1 = bp[kk + 1];
    for (int64_t p0 = bp[kk]; p0 < p1; p0 += 32) {
      const int64_t p = p0 + lane;
      const bool valid = p < p1;
      int j = -1, slot = -1;
      bool isnew = false;
      if (valid) {
        j = bc[p];
        unsigned h = hash_col(j, mask);
        for (;;) {
          const int cur = key[h];
          if (cur == j) { slot = (int)h; break; }
          if (cur == -1) {
            const int prev = atomicCAS(&key[h], -1, j);
            if (prev == -1) { slot = (int)h; isnew = true; break; }
            if (prev == j) { slot = (int)h; break; }
          }
          h = (h + 1) & mask;
        }
      }
      const unsigned nm = __ballot_sync(0xffffffffu, isnew);
      const int mine = count + __popc(nm & ((1u << lane) - 1u));
      if (isnew) pos[slot] = mine;
      __syncwarp();
      if (NUMERIC && valid) {
        const double prod = __dmul_rn(a, bv[p]);
        if (isnew) {
          cc[base + mine] = j;
          cv[base + mine] = prod;
        } else {
          const int64_t q = base + pos[slot];
          cv[q] = __dadd_rn(cv[q], prod);
        }
      }
      count += __popc(nm);
      __syncwarp();
    }
  }
  return count;
  }
}

// rows[] with H-slot tables in shared memory, WPB warps per block
template <bool NUMERIC, bool SERIAL, int H, int WPB>
__global__ void __launch_bounds__(32 * WPB)
spgemm_smem(int nrows_list, const int *__restrict__ rows, const int64_t *__restrict__ ap,
            const int *__restrict__ ac, const double *__restrict__ av, const int64_t *__restrict__ bp,
            const int *__restrict__ bc, const double *__restrict__ bv, const int64_t *__restrict__ cp,
            int64_t *__restrict__ cnt, int *__restrict__ cc, double *__restrict__ cv) {
  extern __shared__ int smem_tab[];
  const int wid = threadIdx.x >> 5;
  int *key = smem_tab + (size_t)wid * 2 * H, *pos = key + H;
  for (int q = blockIdx.x * WPB + wid; q < nrows_list; q += gridDim.x * WPB) {
    const int i = rows[q];
    const int64_t base = NUMERIC ? cp[i] : 0;
    const int c = (int)row_walk<NUMERIC, SERIAL>(i, ap, ac, av, bp, bc, bv, key, pos, (unsigned)H, base, cc, cv);
    if (!NUMERIC && (threadIdx.x & 31) == 0) cnt[i] = c;
    __syncwarp();
  }
}

// rows[] whose tables live in global memory: row q of the list owns slots
// [toff[q], toff[q] + tsize[q]) of gkey / gpos
template <bool NUMERIC, bool SERIAL>
__global__ void spgemm_gmem(int nrows_list, const int *__restrict__ rows, const int64_t *__restrict__ toff,
                            const int *__restrict__ tsize, int *gkey, int *gpos, const int64_t *__restrict__ ap,
                            const int *__restrict__ ac, const double *__restrict__ av, const int64_t *__restrict__ bp,
                            const int *__restrict__ bc, const double *__restrict__ bv, const int64_t *__restrict__ cp,
                            int64_t *__restrict__ cnt, int *__restrict__ cc, double *__restrict__ cv) {
  const int wid = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  for (int q = blockIdx.x * wpb + wid; q < nrows_list; q += gridDim.x * wpb) {
    const int i = rows[q];
    const int64_t base = NUMERIC ? cp[i] : 0;
    const int c = (int)row_walk<NUMERIC, SERIAL>(i, ap, ac, av, bp, bc, bv, gkey + toff[q], gpos + toff[q],
                                                 (unsigned)tsize[q], base, cc, cv);
    if (!NUMERIC && (threadIdx.x & 31) == 0) cnt[i] = c;
    __syncwarp();
  }
}

constexpr int kSmallH = 1024, kSmallWPB = 4;     // 32 KB of tables per block
constexpr int kLargeH = 8192, kLargeWPB = 2;     // 128 KB of tables per block

struct RowClasses {
  std::vector<int> small, large, huge;
  std::vector<int64_t> huge_off;
  std::vector<int> huge_size;
};

template <bool NUMERIC, bool SERIAL>
void spgemm_pass(const DCsr &A, const DCsr &B, const RowClasses &rc, const Buf<int> &ds, const Buf<int> &dl,
                 const Buf<int> &dh, const Buf<int64_t> &dhoff, const Buf<int> &dhsz, Buf<int> &gkey, Buf<int> &gpos,
                 const int64_t *cp, int64_t *cnt, int *cc, double *cv, cudaStream_t s) {
  if (!rc.small.empty()) {
    const size_t sm = (size_t)kSmallWPB * 2 * kSmallH * sizeof(int);
    auto k = spgemm_smem<NUMERIC, SERIAL, kSmallH, kSmallWPB>;
    CSK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const int g = (int)std::min<size_t>((rc.small.size() + kSmallWPB - 1) / kSmallWPB, 152 * 8);
    k<<<g, 32 * kSmallWPB, sm, s>>>((int)rc.small.size(), ds.p, A.ptr.p, A.col.p, A.val.p, B.ptr.p, B.col.p,
                                      B.val.p, cp, cnt, cc, cv);
    CSK(cudaGetLastError());
  }
  if (!rc.large.empty()) {
    const size_t sm = (size_t)kLargeWPB * 2 * kLargeH * sizeof(int);
    auto k = spgemm_smem<NUMERIC, SERIAL, kLargeH, kLargeWPB>;
    CSK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const int g = (int)std::min<size_t>((rc.large.size() + kLargeWPB - 1) / kLargeWPB, 152);
    k<<<g, 32 * kLargeWPB, sm, s>>>((int)rc.large.size(), dl.p, A.ptr.p, A.col.p, A.val.p, B.ptr.p, B.col.p,
                                      B.val.p, cp, cnt, cc, cv);
    CSK(cudaGetLastError());
  }
  if (!rc.huge.empty()) {
    const int g = (int)std::min<size_t>((rc.huge.size() + 3) / 4, 152 * 4);
    spgemm_gmem<NUMERIC, SERIAL><<<g, 128, 0, s>>>((int)rc.huge.size(), dh.p, dhoff.p, dhsz.p, gkey.p, gpos.p,
                                                     A.ptr.p, A.col.p, A.val.p, B.ptr.p, B.col.p, B.val.p, cp, cnt,
                                                     cc, cv);
    CSK(cudaGetLastError());
  }
  CSK(cudaStreamSynchronize(s));
}

// C = A B with the reference's first-touch order; b_repeats: some row of B
// may list a column twice
void spgemm(const DCsr &A, const DCsr &B, bool b_repeats, DCsr &C, cudaStream_t s) {
  C.nrows = A.nrows;
  C.ncols = B.ncols;
  Buf<int64_t> bound;
  bound.alloc((size_t)A.nrows);
  row_bounds<<<nblocks(A.nrows), kThreads, 0, s>>>(A.nrows, A.ptr.p, A.col.p, B.ptr.p, bound.p);
  CSK(cudaGetLastError());
  CSK(cudaStreamSynchronize(s));
  std::vector<int64_t> hb;
  bound.download(hb, (size_t)A.nrows);
  RowClasses rc;
  int64_t hoff = 0;
  for (int i = 0; i < A.nrows; i++) {
    const int64_t b = hb[(size_t)i];
    if (2 * b <= kSmallH) rc.small.push_back(i);
    else if (2 * b <= kLargeH) rc.large.push_back(i);
    else {
      int64_t h = 1;
      while (h < 2 * b) h <<= 1;
      if (h > ((int64_t)1 << 30)) throw std::runtime_error("a product row has more than 2^29 candidates");
      rc.huge.push_back(i);
      rc.huge_off.push_back(hoff);
      rc.huge_size.push_back((int)h);
      hoff += h;
    }
  }
  Buf<int> ds, dl, dh, dhsz, gkey, gpos;
  Buf<int64_t> dhoff;
  ds.upload(rc.small.data(), rc.small.size());
  dl.upload(rc.large.data(), rc.large.size());
  dh.upload(rc.huge.data(), rc.huge.size());
  dhoff.upload(rc.huge_off.data(), rc.huge_off.size());
  dhsz.upload(rc.huge_size.data(), rc.huge_size.size());
  gkey.alloc((size_t)std::max<int64_t>(hoff, 1));
  gpos.alloc((size_t)std::max<int64_t>(hoff, 1));
  Buf<int64_t> cnt;
  cnt.alloc((size_t)A.nrows);
  if (b_repeats)
    spgemm_pass<false, true>(A, B, rc, ds, dl, dh, dhoff, dhsz, gkey, gpos, nullptr, cnt.p, nullptr, nullptr, s);
  else
    spgemm_pass<false, false>(A, B, rc, ds, dl, dh, dhoff, dhsz, gkey, gpos, nullptr, cnt.p, nullptr, nullptr, s);
  C.ptr.alloc((size_t)A.nrows + 1);
  exclusive_scan(cnt.p, A.nrows, C.ptr.p, s);
  int64_t total = 0;
  CSK(cudaMemcpy(&total, C.ptr.p + A.nrows, sizeof(int64_t), cudaMemcpyDeviceToHost));
  C.nnz = total;
  C.col.alloc((size_t)total);
  C.val.alloc((size_t)total);
  if (b_repeats)
    spgemm_pass<true, true>(A, B, rc, ds, dl, dh, dhoff, dhsz, gkey, gpos, C.ptr.p, cnt.p, C.col.p, C.val.p, s);
  else
    spgemm_pass<true, false>(A, B, rc, ds, dl, dh, dhoff, dhsz, gkey, gpos, C.ptr.p, cnt.p, C.col.p, C.val.p, s);
}

void upload(const Csr &h, DCsr &d) {
  d.nrows = h.nrows;
  d.ncols = h.ncols;
  d.nnz = (int64_t)h.col.size();
  d.ptr.upload(h.ptr.data(), h.ptr.size());
  d.col.upload(h.col.data(), h.col.size());
  d.val.upload(h.val.data(), h.val.size());
}

void download(const DCsr &d, Csr &h) {
  h.nrows = d.nrows;
  h.ncols = d.ncols;
  d.ptr.download(h.ptr, (size_t)d.nrows + 1);
  d.col.download(h.col, (size_t)d.nnz);
  d.val.download(h.val, (size_t)d.nnz);
}

// some row of M lists a column twice
bool has_repeats(const Csr &M) {
  std::vector<int> mark((size_t)std::max(M.ncols, 1), -1);
  for (int r = 0; r < M.nrows; r++)
    for (int64_t k = M.ptr[(size_t)r]; k < M.ptr[(size_t)r + 1]; k++) {
      const int c = M.col[(size_t)k];
      if (mark[(size_t)c] == r) return true;
      mark[(size_t)c] = r;
    }
  return false;
}

}  // namespace cs

// IntRestBuild with smoothers 0 or 1 and CoarseMtxBuild on the GPU; see
// setup.hpp (DeviceGalerkin).
bool device_restriction_galerkin(const Csr &A, const std::vector<char> &strong, const Aggregates &fine, int smoothers,
                                 double omega, SetupResult &out, Csr &AC, double &seconds, std::string &err) {
  using namespace cs;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    err = "no CUDA device";
    return false;
  }
  cudaStream_t s = nullptr;
  try {
    // a blocking stream: the synchronous copies (legacy default stream) of
    // the helpers above are ordered with the kernels launched on it
    CSK(cudaStreamCreate(&s));
    cudaEvent_t e0, e1;
    CSK(cudaEventCreate(&e0));
    CSK(cudaEventCreate(&e1));
    CSK(cudaEventRecord(e0, s));
    const int n = A.nrows;
    DCsr dA;
    upload(A, dA);
    const bool a_repeats = has_repeats(A);
    // tentative prolongator T as restriction rows (aggregate -> its nodes)
    Csr Th;
    Th.nrows = fine.nagr;
    Th.ncols = n;
    Th.ptr.assign((size_t)fine.nagr + 1, 0);
    for (int a = 0; a < fine.nagr; a++) Th.ptr[(size_t)a + 1] = fine.starts[(size_t)a + 1];
    Th.col.resize((size_t)fine.starts[(size_t)fine.nagr]);
    for (size_t q = 0; q < Th.col.size(); q++) Th.col[q] = fine.nodes[q] - 1;
    Th.val.assign(Th.col.size(), 1.0);
    DCsr dT, dR;
    upload(Th, dT);
    if (smoothers == 0) {
      dR = std::move(dT);
    } else {
      // S on A's pattern, then R = T S^T through the column view of S
      DCsr dS;
      dS.nrows = dA.nrows; dS.ncols = dA.ncols; dS.nnz = dA.nnz;
      dS.ptr.upload(A.ptr.data(), A.ptr.size());
      dS.col.upload(A.col.data(), A.col.size());
      dS.val.alloc((size_t)dA.nnz);
      Buf<unsigned char> dstrong;
      std::vector<unsigned char> st8(strong.begin(), strong.end());
      dstrong.upload(st8.data(), st8.size());
      smoother_rows<<<nblocks(n), kThreads, 0, s>>>(n, dS.ptr.p, dS.col.p, dA.val.p, dstrong.p, omega, dS.val.p);
      CSK(cudaGetLastError());
      DCsr dSt;
      transpose(dS, dSt, s);
      spgemm(dT, dSt, a_repeats, dR, s);
    }
    // CoarseMtxBuild: P = R by columns, T = A P, R by rows (columns
    // ascending), AC = R T
    DCsr dP, dTm, dRs, dAC;
    transpose(dR, dP, s);
    spgemm(dA, dP, false, dTm, s);
    transpose(dP, dRs, s);
    spgemm(dRs, dTm, false, dAC, s);
    CSK(cudaEventRecord(e1, s));
    CSK(cudaEventSynchronize(e1));
    CSK(cudaStreamSynchronize(s));
    float ms = 0;
    CSK(cudaEventElapsedTime(&ms, e0, e1));
    seconds = ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    download(dP, out.P);
    out.P.nrows = n;
    out.P.ncols = fine.nagr;
    download(dRs, out.R);
    download(dAC, AC);
    // R's entries in the column-arranged order of the reference (its final
    // entry order): fine node after fine node, coarse freedoms ascending
    out.R_i.clear(); out.R_j.clear(); out.R_v.clear();
    out.R_i.reserve(out.P.col.size()); out.R_j.reserve(out.P.col.size()); out.R_v.reserve(out.P.col.size());
    for (int col = 0; col < n; col++)
      for (int64_t k = out.P.ptr[(size_t)col]; k < out.P.ptr[(size_t)col + 1]; k++) {
        out.R_i.push_back(out.P.col[(size_t)k] + 1);
        out.R_j.push_back(col + 1);
        out.R_v.push_back(out.P.val[(size_t)k]);
      }
    cudaStreamDestroy(s);
    return true;
  } catch (const Err &e) {
    err = std::string("coarse setup on the GPU: ") + e.what + ": " + cudaGetErrorString(e.e);
  } catch (const std::exception &ex) {
    err = std::string("coarse setup on the GPU: ") + ex.what();
  }
  if (s) cudaStreamDestroy(s);
  return false;
}

}  // namespace dg
