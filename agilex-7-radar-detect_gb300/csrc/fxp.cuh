// fxp.cuh - fixed-point primitives of the chain, for device and host code.
//
// The numeric contract of the reference model (model/cpp/fxp/fxp.hpp): Q1.15
// samples, exact products, round-to-nearest-even then saturate, flags of the
// ROUNDED value packed {sat_pos<<1 | sat_neg}. These are this project's own
// formulations for sm_103a: 32-bit where the value range provably fits, 64-bit
// only where it does not. Every function states the reference lines it
// reproduces; tests check them against the reference's fxp_ops.vec and
// cmult.vec on the GPU.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define RD_HD __host__ __device__ __forceinline__
#else
#define RD_HD inline
#endif

namespace rd {

struct cplx {
  int16_t re, im;
};

RD_HD cplx unpack(uint32_t p) {
  cplx c;
  c.re = (int16_t)(uint16_t)(p & 0xFFFFu);
  c.im = (int16_t)(uint16_t)(p >> 16);
  return c;
}
RD_HD uint32_t pack(cplx c) {
  return ((uint32_t)(uint16_t)c.im << 16) | (uint32_t)(uint16_t)c.re;
}
RD_HD uint32_t pack2(int32_t re, int32_t im) {
  return ((uint32_t)(uint16_t)im << 16) | (uint32_t)(uint16_t)re;
}

// ---- 64-bit, wrap-safe (fxp.hpp:87-126) ----------------------------------
RD_HD int64_t add_wrap(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
RD_HD int64_t sub_wrap(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
RD_HD int64_t neg_wrap(int64_t a) { return (int64_t)(0ull - (uint64_t)a); }
RD_HD int64_t asr64(int64_t v, unsigned s) {  // floor(v / 2^s)
  if (s == 0) return v;
  if (s >= 64) return v < 0 ? -1 : 0;
  return v >> s;  // arithmetic on every CUDA and gcc target
}
RD_HD int64_t max_of(unsigned w) {
  return w >= 64 ? INT64_MAX : (w < 2 ? 0 : (int64_t)((1ull << (w - 1)) - 1ull));
}
RD_HD int64_t min_of(unsigned w) {
  return w >= 64 ? INT64_MIN : (w < 2 ? 0 : neg_wrap((int64_t)(1ull << (w - 1))));
}
RD_HD unsigned sat_flags64(int64_t v, unsigned w) {  // fxp.hpp:163-165
  return (v > max_of(w) ? 2u : 0u) | (v < min_of(w) ? 1u : 0u);
}
RD_HD int64_t sat64(int64_t v, unsigned w) {  // fxp.hpp:175-179
  const int64_t hi = max_of(w), lo = min_of(w);
  return v > hi ? hi : (v < lo ? lo : v);
}
RD_HD int64_t round_even64(int64_t v, unsigned s) {  // fxp.hpp:198-208
  if (s == 0) return v;
  if (s >= 64) return 0;
  const int64_t q = v >> s;
  const uint64_t rem = (uint64_t)v & ((1ull << s) - 1ull);
  const uint64_t half = 1ull << (s - 1);
  if (rem > half) return add_wrap(q, 1);
  if (rem < half) return q;
  return add_wrap(q, (int64_t)((uint64_t)q & 1ull));
}
RD_HD int64_t round_half_up64(int64_t v, unsigned s) {  // fxp.hpp:191-196
  if (s == 0) return v;
  if (s >= 64) return 0;
  return add_wrap(v, (int64_t)(1ull << (s - 1))) >> s;
}

// ---- 32-bit fast paths ---------------------------------------------------
// Q1.15 output of an exact accumulator: round_sat(v, 15, 16) and the flags of
// the rounded value (fxp.hpp:221-231). For |v| < 2^31 the 32-bit form below
// equals the 64-bit one.
RD_HD int32_t rne15_32(int32_t v) {
  const int32_t q = v >> 15;
  const int32_t rem = v & 0x7FFF;
  return q + ((rem > 0x4000) | ((rem == 0x4000) & (q & 1)));
}
RD_HD int32_t sat16(int32_t r) { return r > 32767 ? 32767 : (r < -32768 ? -32768 : r); }
RD_HD unsigned flags16(int32_t r) { return (r > 32767 ? 2u : 0u) | (r < -32768 ? 1u : 0u); }
RD_HD int64_t rne15_64(int64_t v) {
  const int64_t q = v >> 15;
  const int64_t rem = v & 0x7FFF;
  return q + ((rem > 0x4000) | ((rem == 0x4000) & (q & 1)));
}
// round_sat(v, 15, 16) of a 64-bit accumulator; flags into *fl.
// round_sat(v, 15, 16) of an int32 sum whose |v| <= 2^31 - 2^15 (so the
// rounding add cannot wrap), with the same flags as q15_out64
RD_HD int32_t q15_out32(int32_t v, unsigned* fl) {
  const int32_t r = (v + 0x3FFF + ((v >> 15) & 1)) >> 15;
  *fl |= (r > 32767 ? 2u : 0u) | (r < -32768 ? 1u : 0u);
  return r > 32767 ? 32767 : (r < -32768 ? -32768 : r);
}
RD_HD int32_t q15_out64(int64_t v, unsigned* fl) {
  const int64_t r = rne15_64(v);
  *fl |= (r > 32767 ? 2u : 0u) | (r < -32768 ? 1u : 0u);
  return (int32_t)(r > 32767 ? 32767 : (r < -32768 ? -32768 : r));
}
// FFT sub-stage quantiser: round by sh in {0,1} then saturate, flags of the
// rounded value (fft_ref.hpp:315-319). v is a sum of two int16, |v| <= 2^16.
RD_HD int32_t quant1(int32_t v, unsigned sh, unsigned* fl) {
  int32_t r = v;
  if (sh) r = (v >> 1) + ((v & 1) & ((v >> 1) & 1));
  *fl |= flags16(r);
  return sat16(r);
}

// exact complex product components (fxp.hpp:303-311) in 64 bits
RD_HD int64_t cmul_re_raw(cplx a, cplx b) {
  return (int64_t)((int32_t)a.re * b.re) - (int64_t)((int32_t)a.im * b.im);
}
RD_HD int64_t cmul_im_raw(cplx a, cplx b) {
  return (int64_t)((int32_t)a.re * b.im) + (int64_t)((int32_t)a.im * b.re);
}
// cmul_q15 (fxp.hpp:314-325). The real part always fits int32
// (|re| < 2^31); the imaginary part only reaches 2^31 when all four operands
// are -32768, which the 64-bit path handles.
RD_HD cplx cmul_q15(cplx a, cplx b, unsigned* fl) {
  const int32_t re = (int32_t)a.re * b.re - (int32_t)a.im * b.im;
  const int64_t im = cmul_im_raw(a, b);
  const int32_t rr = rne15_32(re);
  const int64_t ri = rne15_64(im);
  *fl |= flags16(rr) | (ri > 32767 ? 2u : 0u) | (ri < -32768 ? 1u : 0u);
  cplx o;
  o.re = (int16_t)sat16(rr);
  o.im = (int16_t)(ri > 32767 ? 32767 : (ri < -32768 ? -32768 : ri));
  return o;
}
// Twiddle multiply: the twiddle table never has both components at -32768,
// so the imaginary sum stays below 2^31 and the 32-bit form is exact.
RD_HD cplx cmul_tw(cplx a, cplx w, unsigned* fl) {
  const int32_t re = (int32_t)a.re * w.re - (int32_t)a.im * w.im;
  const int32_t im = (int32_t)a.re * w.im + (int32_t)a.im * w.re;
  const int32_t rr = rne15_32(re), ri = rne15_32(im);
  *fl |= flags16(rr) | flags16(ri);
  cplx o;
  o.re = (int16_t)sat16(rr);
  o.im = (int16_t)sat16(ri);
  return o;
}
// -j * c with a saturating negate (fft_ref.hpp:322-331). -(-32768) is the
// only input that leaves the 16-bit range; it is selected explicitly so the
// saturation and its sat_pos flag never depend on how the negate is lowered.
RD_HD cplx neg_j(cplx c, unsigned* fl) {
  const bool over = c.re == (int16_t)-32768;
  *fl |= over ? 2u : 0u;
  cplx o;
  o.re = c.im;
  o.im = over ? (int16_t)32767 : (int16_t)(-(int32_t)c.re);
  return o;
}
// covar::power (covar_model.hpp:99-102): re^2 + im^2 in [0, 2^31]
RD_HD uint32_t power_u32(cplx s) {
  return (uint32_t)((int32_t)s.re * s.re) + (uint32_t)((int32_t)s.im * s.im);
}

RD_HD unsigned bitrev(unsigned v, unsigned w) {
#ifdef __CUDA_ARCH__
  return w ? (__brev(v) >> (32 - w)) : 0u;
#else
  unsigned r = 0;
  for (unsigned i = 0; i < w; ++i)
    if ((v >> i) & 1u) r |= 1u << (w - 1 - i);
  return r;
#endif
}
RD_HD unsigned ilog2(unsigned v) {
  unsigned r = 0;
  while ((1u << r) < v) ++r;
  return r;
}
// fft_ref.hpp:123-129
RD_HD unsigned r22_tw_exp(unsigned l2l, unsigned p) {
  const unsigned q = p & ((1u << l2l) - 1u);
  const unsigned k1 = (q >> (l2l - 1)) & 1u;
  const unsigned k2 = (q >> (l2l - 2)) & 1u;
  const unsigned n3 = q & ((1u << (l2l - 2)) - 1u);
  return n3 * (k1 + 2u * k2);
}

}  // namespace rd
