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

// Balanced 8-bit limbs of v = {im, re}: x = 256 xh + xl with xl the
// sign-extended low byte of x, in [-128, 127], and xh = (x >> 8) + bit 7 of
// x, in [-128, 128]; every limb and limb product is then at most 2^7 and 2^14
// in magnitude. As fp16 pairs, the real part in the low half: xl + 128 is the
// low byte with bit 7 flipped, xh + 128 is the high byte with bit 7 flipped
// plus bit 7 of x (at most 256, so no carry crosses into the other half);
// placed under the exponent of 1024 and the bias 1024 + 128 subtracted.
__device__ __forceinline__ void limb_words_bal(uint32_t v, uint32_t& hi, uint32_t& lo) {
  const uint32_t t = (((v >> 8) & 0x00FF00FFu) ^ 0x00800080u) + ((v >> 7) & 0x00010001u);
  hi = hsub2(t | 0x64006400u, 0x64806480u);
  lo = hsub2(((v ^ 0x00800080u) & 0x00FF00FFu) | 0x64006400u, 0x64806480u);
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

// The integer held exactly by an fp32 value v with |v| <= 2^24, with adds
// only (no float-to-int conversion instruction): v + 1.5 2^25 lies in
// [2^25, 2^26], where fp32 values are the multiples of 4, so it rounds v to
// a multiple of 4 whose quarter is the difference of the bit patterns; the
// rest, v minus that multiple (exact, |r| <= 2), is read the same way off
// r + 1.5 2^23, where the values are the integers.
__device__ __forceinline__ int exact_int24(float v) {
  const float m25 = 50331648.0f, m23 = 12582912.0f;
  const float t = __fadd_rn(v, m25);
  const int q = __float_as_int(t) - __float_as_int(m25);
  const float r = __fsub_rn(v, __fsub_rn(t, m25));
  return q * 4 + (__float_as_int(__fadd_rn(r, m23)) - __float_as_int(m23));
}

// fold3 for accumulators of magnitude <= 2^24
__device__ __forceinline__ long long fold3_24(float c16, float c8, float c0) {
  return (long long)exact_int24(c16) * 65536 + (long long)exact_int24(c8) * 256 +
         (long long)exact_int24(c0);
}

}  // namespace rd
