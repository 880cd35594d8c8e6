// tcgen05 (fifth-generation tensor core) building blocks for sm_103a as inline
// PTX: tensor-memory allocation, shared-memory matrix descriptors, the TF32
// MMA with an FP32 accumulator in tensor memory, its completion through an
// mbarrier, and the tensor-memory load of the accumulator.
//
// Operands are K-major without swizzle: an M x K (or N x K) matrix is a grid
// of core matrices of 8 rows x 16 bytes (4 TF32 values), each stored as 128
// contiguous bytes (row i at 16 i); core matrices adjacent along K are `lbo`
// bytes apart and those adjacent along M / N `sbo` bytes apart.  One
// kind::tf32 MMA consumes K = 8 (two core matrices along K).
#pragma once

#include <cstdint>

namespace rkdg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M / N) byte offsets in 16-byte units, descriptor version 1 (sm_100 family),
// base offset 0, no swizzle.
__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D in FP32 (bits 4-5 = 1), A and B
// TF32 (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N / 8 in
// bits 17-22, M / 16 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Whole warp: allocate ncols (a power of two >= 32) tensor-memory columns;
// the address is written to *dst (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// Whole warp (the allocating one).
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// Ordering of tensor-core operations around thread synchronisation.
__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes made visible to the tensor core.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One thread: D[tmem] (+)= A[smem] x B[smem]^T (accumulate when accum != 0).
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t"
      ".reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t"
      "}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accum)
      : "memory");
}
// One thread: arrive on the mbarrier once every MMA it issued has completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Bounded wait for the phase of the given parity to complete; false when it
// did not within max_tries polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, int max_tries) {
  const uint32_t a = smem_u32(mbar);
  for (int i = 0; i < max_tries; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t"
        ".reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t"
        "}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Whole warp: 32 consecutive FP32 columns of the warp's 32 tensor-memory
// lanes (lane 32 (warp % 4) + thread), one lane per thread; then wait.
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// TF32 split of an FP32 value: hi keeps the 10 explicit mantissa bits a TF32
// operand carries (rounded to nearest), lo = x - hi exactly (its own TF32
// rounding happens in the MMA).  hi * b_hi + hi * b_lo + lo * b_hi carries
// the product to about 2^-21 relative.
__host__ __device__ inline float tf32_hi(float x) {
#ifdef __CUDA_ARCH__
  const uint32_t b = __float_as_uint(x);
  return __uint_as_float((b + 0x1000u) & 0xFFFFE000u);
#else
  uint32_t b;
  __builtin_memcpy(&b, &x, 4);
  b = (b + 0x1000u) & 0xFFFFE000u;
  float y;
  __builtin_memcpy(&y, &b, 4);
  return y;
#endif
}

}  // namespace tc
}  // namespace rkdg
