// tc.cuh - exact integer arithmetic on the fp16 tensor cores: 8-bit limbs of
// the packed Q1.15 samples as fp16 pairs, and the mma.sync m16n8k16
// f16 x f16 -> f32 instruction. A limb (and its negation) is an integer of
// magnitude <= 256, exact in fp16; a product of two limbs is below 2^16, exact
// in fp32; and a kernel that keeps every accumulated sum below 2^24 in
// magnitude gets exact integers out of the fp32 accumulators.
#pragma once

#include <stdint.h>

namespace rd {

__device__ __forceinline__ uint32_t hsub2(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// fp16x2 limb words of a packed sample v = {im, re}: hi = (re >> 8, im >> 8),
// lo = (re & 255, im & 255), the real part in the low half. The fp16 number
// with bits 0x6400 | u is 1024 + u for u < 1024, so placing a byte under that
// exponent and subtracting the bias gives the byte's value exactly; the high
// byte is made unsigned by flipping the sign bit first (bias 1024 + 128).
__device__ __forceinline__ void limb_words(uint32_t v, uint32_t& hi, uint32_t& lo) {
  hi = hsub2((((v ^ 0x80008000u) >> 8) & 0x00FF00FFu) | 0x64006400u, 0x64806480u);
  lo = hsub2((v & 0x00FF00FFu) | 0x64006400u, 0x64006400u);
}

// (-b, a) from the fp16 pair (a, b): the halves swapped, the new low half negated
__device__ __forceinline__ uint32_t negswap(uint32_t w) {
  return __byte_perm(w, 0u, 0x1032) ^ 0x00008000u;
}

__device__ __forceinline__ void mma_f16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                        uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// 2^16 c16 + 2^8 c8 + c0 from three fp32 accumulators holding exact integers
__device__ __forceinline__ long long fold3(float c16, float c8, float c0) {
  return (long long)__float2int_rn(c16) * 65536 + (long long)__float2int_rn(c8) * 256 +
         (long long)__float2int_rn(c0);
}

}  // namespace rd

// ---- tcgen05 (5th-generation tensor cores, TMEM accumulators) -------------
namespace rd {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, `lbo` bytes between core matrices adjacent
// along K, `sbo` bytes between adjacent 8-row groups.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  return d;
}

// Instruction descriptor of kind::f16: f16 x f16 -> f32, both operands
// K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_f16(uint32_t m, uint32_t n) {
  return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(const uint64_t* mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
}

// Bounded wait for phase `parity` of an mbarrier; false when it gave up.
__device__ __forceinline__ bool mbar_wait(const uint64_t* mbar, uint32_t parity,
                                          uint32_t max_iter = (1u << 24)) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < max_iter && !done; ++it)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
  return done != 0;
}

// 1D bulk copy global -> shared (the TMA engine), completion counted in bytes
// on `mbar`; size and both addresses are multiples of 16 bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor core / TMA
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16 consecutive 32-bit TMEM columns of this thread's lane (warp quadrant).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

}  // namespace rd
