// FP64 true residual r = b - A x and ||r||_2^2 for a CSR matrix on the GPU.
//
// The reference computes this residual before the PCG loop
// (src/solvers/pcg.F90:364-367) and, in doug_geom, after it
// (src/main/geom.F90:135-142).  The solver uses the same arithmetic
// internally; this file exposes it to callers that hold their own device
// CSR matrix (for example to check a solution written by dg_solve_device).
//
// The norm is reduced deterministically: each block of kResidRowsPerBlock
// rows writes one partial sum, and one block adds the partials in order.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/doug_gpu.h"

namespace dg {
namespace resid {

constexpr int kThreads = 256;
constexpr int kLanes = 8;                         // lanes per row
constexpr int kRowsPerBlock = 1024;               // rows per partial sum

// r = b - A x for rows [blk*1024, (blk+1)*1024); partial[blk] = sum r_i^2
__global__ void __launch_bounds__(kThreads)
residual_partials(int n, const long long *__restrict__ rp, const int *__restrict__ col,
                  const double *__restrict__ val, const double *__restrict__ x,
                  const double *__restrict__ b, double *__restrict__ r, double *__restrict__ partial) {
  __shared__ double sh[kThreads / 32];
  const int sub = threadIdx.x % kLanes;
  const int row_in_pass = threadIdx.x / kLanes;   // 32 rows per pass
  const int r0 = blockIdx.x * kRowsPerBlock;
  double acc = 0.0;
  for (int pass = 0; pass < kRowsPerBlock / (kThreads / kLanes); pass++) {
    const int i = r0 + pass * (kThreads / kLanes) + row_in_pass;
    double s = 0.0;
    if (i < n)
      for (long long e = rp[i] + sub; e < rp[i + 1]; e += kLanes) s = __fma_rn(val[e], x[col[e]], s);
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, kLanes);
    if (i < n && sub == 0) {
      const double ri = __dsub_rn(b[i], s);
      r[i] = ri;
      acc += ri * ri;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; w++) t += sh[w];
    partial[blockIdx.x] = t;
  }
}

// out = sum of partial[0..np) in a fixed order (one block)
__global__ void __launch_bounds__(kThreads)
sum_partials_ordered(int np, const double *__restrict__ partial, double *__restrict__ out) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int q = threadIdx.x; q < np; q += kThreads) s += partial[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

int blocks_for(int n) { return (n + kRowsPerBlock - 1) / kRowsPerBlock; }

}  // namespace resid
}  // namespace dg

extern "C" dg_status dg_residual_csr(int n, const long long *d_rowptr, const int *d_col,
                                     const double *d_val, const double *d_x, const double *d_b,
                                     double *d_r, double *d_norm2, void *cuda_stream) {
  using namespace dg::resid;
  if (n <= 0 || !d_rowptr || !d_col || !d_val || !d_x || !d_b || !d_r || !d_norm2) return DG_BAD_INPUT;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const int nb = blocks_for(n);
  double *partial = nullptr;
  if (cudaMallocAsync(&partial, (size_t)nb * sizeof(double), s) != cudaSuccess) return DG_CUDA_ERROR;
  residual_partials<<<nb, kThreads, 0, s>>>(n, d_rowptr, d_col, d_val, d_x, d_b, d_r, partial);
  sum_partials_ordered<<<1, kThreads, 0, s>>>(nb, partial, d_norm2);
  cudaError_t e = cudaGetLastError();
  cudaFreeAsync(partial, s);
  return e == cudaSuccess ? DG_OK : DG_CUDA_ERROR;
}

// ---------------------------------------------------------------------------
// Allocation-free variant.
//
// Some callers cannot allocate device memory at the point where they need
// the residual: an application that hands all device memory to its own pool
// and forbids other allocations, code that runs while another component is
// capturing the stream into a CUDA graph (where cudaMalloc is not allowed),
// or a latency-critical loop that must not pay for an allocation's implicit
// synchronisation.  dg_residual_csr_noalloc gives them the same result as
// dg_residual_csr without calling cudaMalloc, cudaFree or any allocating
// routine: its partial sums live in the fixed array below, which is part of
// the library image and stays resident on every GPU that loads the library
// until the process exits.
// ---------------------------------------------------------------------------
namespace dg {
namespace resid {

constexpr int kNoAllocMaxPartials = 65536;  // 512 KiB of doubles
constexpr long long kNoAllocMaxRows = (long long)kNoAllocMaxPartials * kRowsPerBlock;  // 67,108,864

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxPartials];

// Host code may not use g_noalloc_partials as an address: on the host the
// name refers to a stand-in variable, not to device memory.  The device
// address is looked up with the device current and cached per device,
// together with the id of the CUDA context it belongs to: after a
// cudaDeviceReset the device gets a new primary context, into which the
// library's module (and the array) is loaded again, possibly elsewhere, so a
// changed context id makes the next call look the address up again.
constexpr int kMaxDevices = 128;
static double *g_noalloc_ptr[kMaxDevices];
static unsigned long long g_noalloc_ctx[kMaxDevices];
static std::mutex g_noalloc_mu;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points,
// so that the library does not link the driver library itself.
typedef int (*ctx_get_current_fn)(void **ctx);
typedef int (*ctx_get_id_fn)(void *ctx, unsigned long long *id);
static ctx_get_current_fn g_ctx_get_current;
static ctx_get_id_fn g_ctx_get_id;

// The id of the calling thread's current context (0: none yet).
static cudaError_t current_context_id(unsigned long long *id) {
  *id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess) return e != cudaSuccess ? e : cudaErrorNotSupported;
    e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess || q2 != cudaDriverEntryPointSuccess) return e != cudaSuccess ? e : cudaErrorNotSupported;
    g_ctx_get_current = reinterpret_cast<ctx_get_current_fn>(f1);
    g_ctx_get_id = reinterpret_cast<ctx_get_id_fn>(f2);
  }
  void *ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0) return cudaErrorUnknown;
  if (!ctx) return cudaSuccess;
  if (g_ctx_get_id(ctx, id) != 0) return cudaErrorUnknown;
  return cudaSuccess;
}

static cudaError_t noalloc_scratch(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  unsigned long long ctx = 0;
  e = current_context_id(&ctx);
  if (e != cudaSuccess) return e;
  if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    double *p = nullptr;
    // loads the module into the device's primary context if it is not yet
    e = cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_noalloc_partials);
    if (e != cudaSuccess) return e;
    e = current_context_id(&ctx);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = ctx;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace resid
}  // namespace dg

extern "C" dg_status dg_residual_csr_noalloc(int n, const long long *d_rowptr, const int *d_col,
                                             const double *d_val, const double *d_x, const double *d_b,
                                             double *d_r, double *d_norm2, void *cuda_stream) {
  using namespace dg::resid;
  if (n <= 0 || !d_rowptr || !d_col || !d_val || !d_x || !d_b || !d_r || !d_norm2) return DG_BAD_INPUT;
  if ((long long)n > kNoAllocMaxRows) return DG_BAD_INPUT;  // the fixed scratch holds 65,536 partials
  double *partial = nullptr;
  if (noalloc_scratch(&partial) != cudaSuccess) return DG_CUDA_ERROR;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const int nb = blocks_for(n);
  // every partial of [0, nb) is written before it is read, so the contents
  // left by an earlier call need no clearing
  residual_partials<<<nb, kThreads, 0, s>>>(n, d_rowptr, d_col, d_val, d_x, d_b, d_r, partial);
  sum_partials_ordered<<<1, kThreads, 0, s>>>(nb, partial, d_norm2);
  return cudaGetLastError() == cudaSuccess ? DG_OK : DG_CUDA_ERROR;
}
