// Minimal tcgen05 (5th-generation tensor core) helpers for sm_100-family
// GPUs, in inline PTX (internal header).
//
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte "core matrices"; element (r, k) of a 16-bit
// operand with K columns sits at
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 bytes (next core matrix along K) and SBO = K / 8 * 128
// (next 8-row group).  Accumulators live in tensor memory (TMEM): for
// M = 128 and one CTA, row i of D is TMEM lane i and column j is column j.
// Every wait is bounded: on timeout a flag is set and false is returned.
#pragma once
#include <cstdint>

namespace imodel {
namespace tc05 {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in a K-major operand with k_cols columns
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int k_cols) {
  return static_cast<uint32_t>((r >> 3) * (k_cols * 16) + (k >> 3) * 128 + (r & 7) * 16 +
                               (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16;
  d |= static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// instruction descriptor, kind::f16: BF16 A and B (both K-major), FP32 D
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4)                                   // D: F32
         | (1u << 7)                                 // A: BF16
         | (1u << 10)                                // B: BF16
         | (static_cast<uint32_t>(n >> 3) << 17)     // N / 8
         | (static_cast<uint32_t>(m >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// D(tmem) (+)= A(smem) * B(smem)^T, one instruction (K = 16), issued by one thread
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// the mbarrier receives one arrival when all previously issued MMAs are done
__device__ __forceinline__ void commit(uint64_t *mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for phase `parity` of the mbarrier; false (and *err |= flag)
// if it did not complete
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, int *err, int flag) {
  for (int it = 0; it < (1 << 20); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  atomicOr(err, flag);
  return false;
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes become visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// CTA-wide barrier ordering tcgen05 operations around it
__device__ __forceinline__ void sync_cta() {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape)
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace tc05
}  // namespace imodel
