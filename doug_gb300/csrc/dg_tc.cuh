// Fifth-generation tensor-core helpers (sm_100a / sm_103a): tcgen05 MMAs
// with the accumulator in tensor memory (TMEM), operands staged in shared
// memory in the 128-byte-swizzled K-major layout, completion tracked with
// an mbarrier.  Used by the 3xTF32 trailing update of the large fronts.
//
// Shared-memory operand layout (SWIZZLE_128B, K-major): a tile of R rows x
// 32 FP32 values of K; row r takes 128 bytes, eight rows form a 1024-byte
// atom, and the 16-byte chunk c of row r sits at chunk c ^ (r % 8) of the
// row.  Tiles start on 1024-byte boundaries.  The matrix descriptor of such
// a tile: start address >> 4 (bits 0-13), leading byte offset 16 B
// (unused for this layout, bits 16-29), stride byte offset 1024 B between
// 8-row groups (bits 32-45), descriptor version 1 (bits 46-47), swizzle mode
// 128B (value 2, bits 61-63).  A K step of 8 TF32 values moves the start
// address by 32 bytes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, kk), kk < 32, in a SWIZZLE_128B K-major tile
__device__ __forceinline__ uint32_t sw128_offset(int r, int kk) {
  const uint32_t chunk = (uint32_t)(kk >> 2) ^ (uint32_t)(r & 7);
  return (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u + chunk * 16u + (uint32_t)(kk & 3) * 4u;
}

__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);   // start address
  d |= (uint64_t)1u << 16;                      // leading byte offset (16 B)
  d |= (uint64_t)(1024u >> 4) << 32;            // stride byte offset
  d |= (uint64_t)1u << 46;                      // descriptor version
  d |= (uint64_t)2u << 61;                      // SWIZZLE_128B
  return d;
}

// instruction descriptor of kind::tf32: D F32, A and B TF32, both K-major,
// M x N (M = 128, N a multiple of 16 up to 256)
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A B^T for one K step; accumulate = 0 overwrites D
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
#endif
}

// the mbarrier at bar is arrived on once every MMA issued so far is done
__device__ __forceinline__ void mma_commit(uint32_t bar) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
#endif
}

__device__ __forceinline__ void fence_before_sync() {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
#endif
}
__device__ __forceinline__ void fence_after_sync() {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#endif
}
// generic-proxy shared-memory writes become visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one warp allocates / frees ncols TMEM columns; the address lands in *dst
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
#endif
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
#endif
}

// 32 consecutive FP32 columns of this thread's TMEM lane (warp w of a
// warpgroup reads lanes 32 (w % 4) ..)
__device__ __forceinline__ void tmem_load32(uint32_t taddr, float (&v)[32]) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
#else
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = 0.f;
#endif
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_load16(uint32_t taddr, float (&v)[16]) {
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
#else
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = 0.f;
#endif
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// waits for the phase with the given parity to complete, at most max_polls
// polls; false when it gave up
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long max_polls) {
  const uint32_t a = smem_u32(bar);
  for (long long i = 0; i < max_polls; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

}  // namespace tc
}  // namespace dg
