// front_fast.cuh - the PFB + FFT + corner-turn kernel specialised per FFT
// geometry (lane length 2^NL, SPC lanes, taps TT, and whether every
// sub-stage of the scaling schedule halves). Same arithmetic, same outputs,
// as k_front in k_frontend.cu, organised for instruction count. With EXT the
// PFB has run as its own frame-blocked pass (k_pfb_rows.cu) and this kernel
// loads its outputs; otherwise it computes the PFB itself:
//
//  * every thread owns 4 elements of a lane, so each pair of radix-2^2
//    sub-stages (BF2I at s, BF2II at s+1, fft_ref.hpp:334-365) runs in
//    registers and only every second sub-stage exchanges through shared
//    memory (one barrier per exchange, double-buffered);
//  * stage constants fold at compile time; values stay as unpacked int32
//    re/im between sub-stages; with SH1 the schedule's shifts are constants
//    too (the default schedule halves at every sub-stage);
//  * saturation cannot happen in a pass whose PFB outputs are all within the
//    bound `safe_in` the host derives from the scaling schedule and the
//    twiddle table (front_safe_input): such a pass runs the sub-stages with
//    plain rounding, no clamps and no flag tracking. Any other pass runs the
//    same code instantiated with the exact saturation and per-sub-stage flags
//    of fft_ref.hpp:230-234. Values never depend on which path ran.
//
// Thread t of an item owns lane q = t & 1 (spc 2) and quad index t >> 1, so a
// warp's PFB loads read consecutive phases. The geometries are instantiated
// in three translation units (k_front_fast*.cu) so that they compile in
// parallel.
#pragma once
#include <cuda_runtime.h>

#include "fxp.cuh"
#include "rd_internal.h"

namespace rd {

struct C2 {
  int re, im;
};

__device__ __forceinline__ int sext16(uint32_t v) { return (int)(int16_t)(uint16_t)(v & 0xFFFFu); }
__device__ __forceinline__ C2 unpk(uint32_t v) { return C2{sext16(v), (int)v >> 16}; }
__device__ __forceinline__ uint32_t pk(C2 c) {
  return ((uint32_t)(uint16_t)c.im << 16) | (uint32_t)(uint16_t)c.re;
}

// round by sh in {0,1} (round_even, fxp.hpp:198-208), saturate to 16 bits
// (fft_ref.hpp:315-319). FL: the exact path, saturation and direction flags;
// else the bound-checked pass, where no value can leave 16 bits.
template <bool FL>
__device__ __forceinline__ int qsat(int v, unsigned sh, unsigned& ovf, unsigned& fl) {
  const int r = sh ? ((v >> 1) + ((v & (v >> 1)) & 1)) : v;
  if (!FL) return r;
  fl |= (r > 32767 ? 2u : 0u) | (r < -32768 ? 1u : 0u);
  return min(max(r, -32768), 32767);
}

// round_sat(v, 15, 16) of an exact product sum |v| < 2^31 (fxp.hpp:221-231):
// round to nearest even at 2^15 is (v + 0x3FFF + bit15(v)) >> 15.
template <bool FL>
__device__ __forceinline__ int q15(int v, unsigned& ovf, unsigned& fl) {
  const int r = (v + 0x3FFF + ((v >> 15) & 1)) >> 15;
  if (!FL) return r;
  fl |= (r > 32767 ? 2u : 0u) | (r < -32768 ? 1u : 0u);
  return min(max(r, -32768), 32767);
}

// a, t <- (a + t', a - t'), t' = -j t when K1 (saturating negate of t.re)
template <bool FL, bool K1>
__device__ __forceinline__ void bfly(C2& a, C2& t, unsigned sh, unsigned& ovf, unsigned& fl) {
  C2 u = t;
  if (K1) {
    const int n = -t.re;
    if (FL) {
      fl |= n > 32767 ? 2u : 0u;
      u = C2{t.im, min(n, 32767)};
    } else {
      u = C2{t.im, n};  // |t.re| <= 32767 in a bound-checked pass
    }
  }
  const C2 lo{qsat<FL>(a.re + u.re, sh, ovf, fl), qsat<FL>(a.im + u.im, sh, ovf, fl)};
  const C2 hi{qsat<FL>(a.re - u.re, sh, ovf, fl), qsat<FL>(a.im - u.im, sh, ovf, fl)};
  a = lo;
  t = hi;
}

// The halving butterflies of a bound-checked pass on the FMA pipe, exactly.
// An integer v with |v| < 2^22 is held as the float 1.5 x 2^23 + v (bit
// pattern 0x4B400000 + v): around 1.5 x 2^23 the float spacing is 1, so
// fma(s, 0.5, 1.5 x 2^23) of an integer s below 2^17 in magnitude is
// 1.5 x 2^23 + RNE(s / 2) - IEEE round-to-nearest-even on the sum, whose
// integer part has the parity of RNE(s / 2) because 1.5 x 2^23 is even (the
// "magic number" rounding). Every other step (a + (t - 3 x 2^23) = a + t,
// a - t, 3 x 2^23 - t) is exact, and each is written with an explicitly
// rounded intrinsic so that no contraction changes it. Values never depend
// on which pipe computed them.
struct F2 {
  float re, im;
};
constexpr float kMg = 12582912.0f, kMg2 = 25165824.0f;  // 1.5 x 2^23, 3 x 2^23
__device__ __forceinline__ float mg(int v) { return __int_as_float(v + 0x4B400000); }
__device__ __forceinline__ int ung(float f) { return __float_as_int(f) - 0x4B400000; }

// a, t <- (RNE((a + u) / 2), RNE((a - u) / 2)), u = t or -j t, on held values
template <bool K1>
__device__ __forceinline__ void bfly_mg(F2& a, F2& t) {
  const F2 u = K1 ? F2{t.im, __fsub_rn(kMg2, t.re)} : t;
  const F2 lo{__fmaf_rn(__fadd_rn(a.re, __fsub_rn(u.re, kMg2)), 0.5f, kMg),
              __fmaf_rn(__fadd_rn(a.im, __fsub_rn(u.im, kMg2)), 0.5f, kMg)};
  const F2 hi{__fmaf_rn(__fsub_rn(a.re, u.re), 0.5f, kMg),
              __fmaf_rn(__fsub_rn(a.im, u.im), 0.5f, kMg)};
  a = lo;
  t = hi;
}

// a * w rounded once (cmul_q15, fxp.hpp:314-318) for a twiddle w {re, im}
// (kept unpacked in shared memory)
template <bool FL>
__device__ __forceinline__ C2 twm(C2 a, int2 w, unsigned& ovf, unsigned& fl) {
  return C2{q15<FL>(a.re * w.x - a.im * w.y, ovf, fl), q15<FL>(a.re * w.y + a.im * w.x, ovf, fl)};
}

// Two-way dot products of the packed sample {re, im} (signed 16-bit halves)
// with two bytes of b (dp2a: .lo bytes 0-1, .hi bytes 2-3; signed or
// unsigned bytes), accumulated into c
__device__ __forceinline__ int dp2a_lo_ss(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.lo.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ int dp2a_hi_ss(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.hi.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ int dp2a_lo_su(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.lo.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}
__device__ __forceinline__ int dp2a_hi_su(uint32_t a, uint32_t b, int c) {
  int d;
  asm("dp2a.hi.s32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// positions of the quad of quad-index tl for a stage pair whose inner
// distance is 2^P (outer 2^(P+1)): base + {0, d1, d0, d0 + d1}
template <int P>
__device__ __forceinline__ int quad_base(int tl) {
  return (tl & ((1 << P) - 1)) | ((tl >> P) << (P + 2));
}

template <int NL, int SPC>
struct Geo {
  static constexpr int M = 1 << NL;       // lane length
  static constexpr int N = M * SPC;       // FFT size
  static constexpr int TPI = N / 4;       // threads per item
  static constexpr int NTW = (NL - 1) / 2;
};

// smem index of lane element (q, pos): phase order 2*pos + q (spc 2)
template <int SPC>
__device__ __forceinline__ int sidx(int q, int pos) {
  return SPC == 2 ? 2 * pos + q : pos;
}

// Word k of this item's exchange buffer, the item's words starting at word
// ioff of the pass's buffer. The exchanges after the first stage pairs access
// words at strides of 8 to 64 (their lanes differ in address bits 3-6), which
// hit 2 to 4 words in one bank; an XOR of bits 1-4 with (b5, b6, b5, b6) maps
// every such warp access onto distinct banks at spc 2 (a CPU model of every
// instantiation's accesses checked it), keeps bit 0 (the merge reads phase
// pairs as 8-byte words) and is a permutation of each 128-word block.
__device__ __forceinline__ int xw(int ioff, int k) {
  const int a = ioff + k;
  return a ^ (((a >> 4) & 6) * 5);
}
// The swizzle is linear over XOR, and within an exchange a thread's words are
// one base plus offsets in bit positions the base leaves zero (the quad's d0,
// d1 or the merge's lane half; a CPU model checked every access of every
// instantiation), so word base + o sits at xw(base) ^ xk(o): one swizzle a
// stage, then an XOR with a constant for each access.
constexpr int xk(int o) { return o ^ (((o >> 4) & 6) * 5); }

// The lane sub-stages of one item after the PFB. E[j] holds lane element
// quad_base<NL-2>(tl) + {0, d1, d0, d0+d1}[j] of lane q on entry. On return,
// the lane values are in buf[cur] (smem, phase order), cur updated.
template <int NL, int SPC, bool FL, bool SH1, int S>
__device__ __forceinline__ void lane_stages(C2 (&E)[4], int q, int tl, unsigned sched,
                                            const int2* twp, uint32_t* buf0, uint32_t* buf1,
                                            int ioff, int& cur, unsigned& ovf, unsigned& sf) {
  constexpr int M = 1 << NL;
  if constexpr (S + 1 < NL) {
    // stage pair (S, S+1): distances d0 = 2^(P+1), d1 = 2^P
    constexpr int P = NL - 2 - S;
    constexpr int d1 = 1 << P, d0 = 2 << P;
    const int base = quad_base<P>(tl);
    unsigned f0 = 0, f1 = 0;
    const unsigned sh0 = SH1 ? 1u : (sched >> S) & 1u;
    const unsigned sh1 = SH1 ? 1u : (sched >> (S + 1)) & 1u;
    if constexpr (!FL && SH1) {  // both sub-stages halve, nothing saturates
      F2 G[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) G[j] = F2{mg(E[j].re), mg(E[j].im)};
      bfly_mg<false>(G[0], G[2]);  // BF2I, distance d0
      bfly_mg<false>(G[1], G[3]);
      bfly_mg<false>(G[0], G[1]);  // BF2II, distance d1
      bfly_mg<true>(G[2], G[3]);   // odd block: -j on the lower half
#pragma unroll
      for (int j = 0; j < 4; ++j) E[j] = C2{ung(G[j].re), ung(G[j].im)};
    } else {
      bfly<FL, false>(E[0], E[2], sh0, ovf, f0);  // BF2I, distance d0
      bfly<FL, false>(E[1], E[3], sh0, ovf, f0);
      bfly<FL, false>(E[0], E[1], sh1, ovf, f1);  // BF2II, distance d1
      bfly<FL, true>(E[2], E[3], sh1, ovf, f1);   // odd block: -j on the lower half
    }
    if constexpr (S + 2 < NL) {                 // group-closing twiddle
      const int2* tw = twp + (S / 2) * M;
      E[0] = twm<FL>(E[0], __ldg(tw + base), ovf, f1);
      E[1] = twm<FL>(E[1], __ldg(tw + base + d1), ovf, f1);
      E[2] = twm<FL>(E[2], __ldg(tw + base + d0), ovf, f1);
      E[3] = twm<FL>(E[3], __ldg(tw + base + d0 + d1), ovf, f1);
    }
    if (FL) sf |= (f0 << (2 * S)) | (f1 << (2 * (S + 1)));
    // exchange into the next quad layout (or the final layout)
    uint32_t* b = cur ? buf1 : buf0;
    const int A = xw(ioff, sidx<SPC>(q, base));
    b[A] = pk(E[0]);
    b[A ^ xk(SPC * d1)] = pk(E[1]);
    b[A ^ xk(SPC * d0)] = pk(E[2]);
    b[A ^ xk(SPC * (d0 + d1))] = pk(E[3]);
    __syncthreads();
    if constexpr (S + 2 < NL) {
      constexpr int PN = (S + 3 < NL) ? NL - 4 - S : 0;  // next pair, or a single stage
      constexpr int e1 = (S + 3 < NL) ? (1 << PN) : 1;
      constexpr int e0 = (S + 3 < NL) ? (2 << PN) : 2;
      const int nb = (S + 3 < NL) ? quad_base<PN>(tl) : 4 * tl;
      const int An = xw(ioff, sidx<SPC>(q, nb));
      E[0] = unpk(b[An]);
      E[1] = unpk(b[An ^ xk(SPC * e1)]);
      E[2] = unpk(b[An ^ xk(SPC * e0)]);
      E[3] = unpk(b[An ^ xk(SPC * (e0 + e1))]);
      cur ^= 1;
      lane_stages<NL, SPC, FL, SH1, S + 2>(E, q, tl, sched, twp, buf0, buf1, ioff, cur, ovf, sf);
    }
  } else if constexpr (S + 1 == NL) {
    // final single stage (NL odd), distance 1, quad = 4*tl .. 4*tl+3
    unsigned f0 = 0;
    const unsigned sh0 = SH1 ? 1u : (sched >> S) & 1u;
    if constexpr (!FL && SH1) {
      F2 G[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) G[j] = F2{mg(E[j].re), mg(E[j].im)};
      bfly_mg<false>(G[0], G[1]);
      bfly_mg<false>(G[2], G[3]);
#pragma unroll
      for (int j = 0; j < 4; ++j) E[j] = C2{ung(G[j].re), ung(G[j].im)};
    } else {
      bfly<FL, false>(E[0], E[1], sh0, ovf, f0);
      bfly<FL, false>(E[2], E[3], sh0, ovf, f0);
    }
    if (FL) sf |= f0 << (2 * S);
    uint32_t* b = cur ? buf1 : buf0;
    const int A = xw(ioff, sidx<SPC>(q, 4 * tl));
#pragma unroll
    for (int j = 0; j < 4; ++j) b[A ^ xk(SPC * j)] = pk(E[j]);
    __syncthreads();
  }
}

// Calls tap(k, xp) for every tap k, xp pointing at phase ph0 of frame f - k
// of channel c: the chunk, or the delay line for frames before it. Frames
// whose taps all lie in the chunk (all but the first T - 1) take constant
// offsets from one row pointer.
template <int N, int TT, class Tap>
__device__ __forceinline__ void for_taps(const FrontParams& p, int T, unsigned f, unsigned c,
                                         int ph0, Tap&& tap) {
  const uint32_t* xa = p.adc + (size_t)c * p.ld + ph0;
  if (TT && f + 1u >= (unsigned)TT) {
    const uint32_t* x0 = xa + (size_t)f * N;
#pragma unroll
    for (int k = 0; k < TT; ++k) tap(k, x0 - k * N);
    return;
  }
  const uint32_t* xt = p.tail + (size_t)c * (T - 1) * N + ph0;
#pragma unroll
  for (int k = 0; k < (TT ? TT : 16); ++k) {
    if (!TT && k >= T) break;
    const long long fr = (long long)f - k;
    tap(k, fr >= 0 ? xa + (size_t)fr * N : xt + (size_t)(-fr - 1) * N);
  }
}

// The corner-turn tile's row skew: tile row r (frame fb, bin: r = fb N + bin)
// starts at word r (CB + 1) + tile_skew<N>(r). The natural-order stores of a
// warp go to bit-reversed bins, rows a power of two apart; with CB + 1 = 9 or
// 17 words a row, up to 16 (spc 2) or 8 (spc 1) lanes of a store met in one
// bank at N = 1024, 4 or 2 at N = 256. One pad word after every 32 rows
// spreads them over the banks (one word a bank for CB 2^k >= 2). N is a
// multiple of 32 there, so the skew of fb N + bin is the skew of fb N plus the
// skew of bin. The smaller sizes keep the plain layout: it is conflict-free or
// no worse.
template <int N>
__host__ __device__ __forceinline__ constexpr unsigned tile_skew(unsigned r) {
  return N >= 256 ? r >> 5 : 0u;
}

// the tile's words: FB frames of N rows, CB + 1 words a row, plus the skew pads
template <int N>
__host__ __device__ __forceinline__ constexpr size_t tile_words(unsigned FB, unsigned CB) {
  return (size_t)FB * N * (CB + 1u) + tile_skew<N>(FB * N);
}

// One pass over IPP items: PFB into registers (EXT: the PFB pass's outputs,
// k_pfb_rows.cu, loaded), the lane sub-stages, the merge, natural-order
// outputs into the corner-turn tile. Returns whether any value of the pass
// saturated (block-uniform).
template <int NL, int SPC, int TT, bool FL, bool SH1, bool EXT>
__device__ __forceinline__ bool front_pass_body(const FrontParams& p, int T, int q, int tl, bool ok,
                                                unsigned f, unsigned c, const int2* twp,
                                                uint32_t* buf0, uint32_t* buf1, int ioff,
                                                uint32_t* tile_row, unsigned cbp, unsigned& pfl,
                                                unsigned long long& psat, unsigned& sf_out) {
  using G = Geo<NL, SPC>;
  constexpr int M = G::M, N = G::N;
  constexpr int d1 = M / 4, d0 = M / 2;
  C2 E[4];
  unsigned ovf = 0, sf = 0;
  // ---- PFB (pfb_model.hpp:139-177): the thread's 4 phases, taps outer ----
  const int pos0 = tl;  // quad_base<NL-2>(tl) == tl
  const int ph0 = SPC * pos0 + q;
  constexpr int dph1 = SPC * d1, dph2 = SPC * d0;
  // the chunk's last T - 1 frames become the next chunk's delay line
  // (pfb_model.hpp:170-175): this frame's samples go there as they are read
  uint32_t* tail_row = nullptr;
  if (!FL && !EXT && ok && p.tail_out && f + (unsigned)T > p.F)
    tail_row = p.tail_out + ((size_t)c * (T - 1) + (p.F - 1u - f)) * N + ph0;
  auto finish = [&](int j, int yr, int yi, unsigned fr, unsigned fi) {
    if (fr | fi) {
      pfl |= fr | fi;
      ++psat;
    }
    E[j] = C2{yr, yi};
    if (ok && p.tap_pfb)
      p.tap_pfb[((size_t)f * p.C + c) * N + ph0 + (j & 1) * dph1 + (j >> 1) * dph2] = pk(E[j]);
  };
  // round_sat(acc, 15, 16) of an int32 sum (|acc| <= 2^31 - 2^15, pfb32). The
  // exact pass saturates and flags; the bound-checked pass only rounds: a
  // value that would saturate is at least 32768 in magnitude, above any
  // safe_in (<= 32767), so the pass fails its check below and reruns exactly,
  // and the flags and counts come from that rerun
  auto round_out = [&](int j, int vr, int vi) {
    if constexpr (FL) {
      unsigned fr = 0, fi = 0;
      const int yr = q15_out32(vr, &fr), yi = q15_out32(vi, &fi);
      finish(j, yr, yi, fr, fi);
    } else {
      finish(j, (vr + 0x3FFF + ((vr >> 15) & 1)) >> 15, (vi + 0x3FFF + ((vi >> 15) & 1)) >> 15, 0u,
             0u);
    }
  };
  if constexpr (EXT) {
    // already rounded and saturated by the PFB pass, which also counted its
    // flags and wrote the delay line and the taps
#pragma unroll
    for (int j = 0; j < 4; ++j)
      E[j] = ok ? unpk(__ldg(p.pfb_in + ((size_t)f * p.C + c) * N + ph0 + (j & 1) * dph1 +
                            (j >> 1) * dph2))
                : C2{0, 0};
  } else if (p.pfb_dp) {
    // x h = 256 x hh + x hl with byte limbs: re = x.re hr + x.im (-hi),
    // im = x.re hi + x.im hr, two dp2a per limb on the packed sample. The
    // limb sums stay below 2^28; the true sums are below 2^31 (pfb32), so
    // recombining modulo 2^32 gives them exactly
    int hr[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0}, lr[4] = {0, 0, 0, 0}, li[4] = {0, 0, 0, 0};
    if (ok) {
      const uint2* hc = p.coeff_dp + ph0;
      for_taps<N, TT>(p, T, f, c, ph0, [&](int k, const uint32_t* xp) {
        const uint2* hp = hc + (size_t)k * N;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int o = (j & 1) * dph1 + (j >> 1) * dph2;
          const uint32_t xw = __ldg(xp + o);
          if (k == 0 && tail_row) tail_row[o] = xw;
          const uint2 h = __ldg(hp + o);
          hr[j] = dp2a_lo_ss(xw, h.x, hr[j]);
          hi[j] = dp2a_hi_ss(xw, h.x, hi[j]);
          lr[j] = dp2a_lo_su(xw, h.y, lr[j]);
          li[j] = dp2a_hi_su(xw, h.y, li[j]);
        }
      });
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      round_out(j, (int)((uint32_t)hr[j] * 256u + (uint32_t)lr[j]),
                (int)((uint32_t)hi[j] * 256u + (uint32_t)li[j]));
  } else if (p.pfb32) {
    // every partial sum is bounded by 2^15 x the phase's L1 norm < 2^31
    int ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
    if (ok) {
      const int2* hc = p.coeff2 + ph0;
      for_taps<N, TT>(p, T, f, c, ph0, [&](int k, const uint32_t* xp) {
        const int2* hp = hc + (size_t)k * N;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int o = (j & 1) * dph1 + (j >> 1) * dph2;
          const uint32_t xw = __ldg(xp + o);
          if (k == 0 && tail_row) tail_row[o] = xw;
          const C2 x = unpk(xw);
          const int2 h = __ldg(hp + o);
          ar[j] += x.re * h.x - x.im * h.y;
          ai[j] += x.re * h.y + x.im * h.x;
        }
      });
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) round_out(j, ar[j], ai[j]);
  } else {
    long long ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
    if (ok) {
      const uint32_t* hc = p.coeff_t + ph0;
      for_taps<N, TT>(p, T, f, c, ph0, [&](int k, const uint32_t* xp) {
        const uint32_t* hp = hc + (size_t)k * N;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int o = (j & 1) * dph1 + (j >> 1) * dph2;
          const uint32_t xw = __ldg(xp + o);
          if (k == 0 && tail_row) tail_row[o] = xw;
          const C2 x = unpk(xw), hk = unpk(__ldg(hp + o));
          ar[j] += (long long)x.re * hk.re;
          ar[j] -= (long long)x.im * hk.im;
          ai[j] += (long long)x.re * hk.im;
          ai[j] += (long long)x.im * hk.re;
        }
      });
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (FL) {
        unsigned fr = 0, fi = 0;
        const int yr = q15_out64(ar[j], &fr), yi = q15_out64(ai[j], &fi);
        finish(j, yr, yi, fr, fi);
      } else {
        finish(j, (int)rne15_64(ar[j]), (int)rne15_64(ai[j]), 0u, 0u);
      }
    }
  }
  // ---- the pass's bound check: every PFB output within safe_in means no
  // sub-stage can saturate; otherwise the caller runs the exact path ----
  if constexpr (!FL) {
    int m = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) m = max(m, max(abs(E[j].re), abs(E[j].im)));
    if (__syncthreads_or(ok && m > (int)p.safe_in)) return true;
  }
  // ---- lane sub-stages (fft_ref.hpp:269-276) ----
  int cur = 0;
  lane_stages<NL, SPC, FL, SH1, 0>(E, q, tl, p.sched, twp, buf0, buf1, ioff, cur, ovf, sf);
  uint32_t* b = cur ? buf1 : buf0;
  // ---- merge (fft_ref.hpp:380-406) and natural bins (:291-296) ----
  if constexpr (SPC == 2) {
    // thread (q, tl) of M/2 threads takes positions j = tid and j + M/2
    const int t = 2 * tl + q;
    const unsigned shm = SH1 ? 1u : (p.sched >> NL) & 1u;
    unsigned fm = 0;
    const int2* tw = twp + G::NTW * M;
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2) {
      const int j = t + h2 * (M / 2);
      // phases 2j, 2j + 1 (j = t + h2 M / 2)
      const uint2 eo = *reinterpret_cast<const uint2*>(b + (xw(ioff, 2 * t) ^ xk(h2 * M)));
      C2 e = unpk(eo.x);
      C2 o = twm<FL>(unpk(eo.y), __ldg(tw + j), ovf, fm);
      if constexpr (!FL && SH1) {
        F2 ge{mg(e.re), mg(e.im)}, go{mg(o.re), mg(o.im)};
        bfly_mg<false>(ge, go);
        e = C2{ung(ge.re), ung(ge.im)};
        o = C2{ung(go.re), ung(go.im)};
      } else {
        bfly<FL, false>(e, o, shm, ovf, fm);
      }
      const unsigned bin = bitrev((unsigned)j, NL);
      // rows bin and bin + M; M is a multiple of 32 wherever the skew is on
      const unsigned row = bin * cbp + tile_skew<N>(bin);
      if (ok) {
        tile_row[row] = pk(e);
        tile_row[row + M * cbp + tile_skew<N>(M)] = pk(o);
      }
    }
    if (FL) sf |= fm << (2 * NL);
  } else {
    const int base = 4 * tl;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int bin = (int)bitrev((unsigned)(base + j), NL);
      if (ok) tile_row[bin * cbp + tile_skew<N>(bin)] = b[xw(ioff, base) ^ xk(j)];
    }
  }
  if (FL && ok) sf_out |= sf;
  __syncthreads();  // the tile and the exchange buffers are reused next pass
  return false;
}

// The exact-flags recomputation, kept out of line so it does not weigh on the
// register allocation of the common path.
template <int NL, int SPC, int TT, bool SH1, bool EXT>
__device__ __noinline__ void front_pass_flags(const FrontParams& p, int T, int q, int tl, bool ok,
                                              unsigned f, unsigned c, const int2* twp,
                                              uint32_t* buf0, uint32_t* buf1, int ioff,
                                              uint32_t* tile_row,
                                              unsigned cbp, unsigned* sf_out) {
  unsigned pfl = 0, sf = 0;
  unsigned long long psat = 0;
  front_pass_body<NL, SPC, TT, true, SH1, EXT>(p, T, q, tl, ok, f, c, twp, buf0, buf1, ioff, tile_row, cbp,
                                          pfl, psat, sf);
  *sf_out |= sf;
  // the PFB flags and saturation count of the pass (the whole block runs
  // this rerun, so every lane of the warp is here)
  const unsigned a = __reduce_or_sync(0xffffffffu, pfl);
  for (int o = 16; o > 0; o >>= 1) psat += __shfl_xor_sync(0xffffffffu, psat, o);
  if ((threadIdx.x & 31u) == 0u) {
    if (a) atomicOr(&p.stats->pfb_flags, a);
    if (psat) atomicAdd(&p.stats->pfb_sat, psat);
  }
}

// EXT (the PFB computed by its own pass) holds no PFB accumulators: four
// CTAs an SM; the fused form keeps three (80 registers)
template <int NL, int SPC, int TT, bool SH1, bool EXT>
__global__ void __launch_bounds__(256, EXT ? 4 : 3) k_front_fast(FrontParams p, unsigned FB, unsigned CB) {
  using G = Geo<NL, SPC>;
  constexpr int N = G::N, M = G::M, TPI = G::TPI;
  constexpr int IPP = 256 / TPI;  // items per pass
  extern __shared__ __align__(16) uint32_t sm[];
  // the twiddles {re, im} are read from global memory through L1 (20 KB at
  // N = 1024: in shared memory they cost a CTA per SM)
  const int2* s_tw = p.tw2;
  uint32_t* s_buf = sm;                   // [2][IPP][N]
  uint32_t* s_tile = s_buf + 2 * IPP * N; // [FB][N][CB+1], rows skewed (tile_skew)
  const unsigned cbp = CB + 1u;
  const int tid = threadIdx.x;
  const int item = tid / TPI, t = tid % TPI;
  const int q = SPC == 2 ? (t & 1) : 0;
  const int tl = SPC == 2 ? (t >> 1) : t;
  const int T = TT ? TT : (int)p.T;
  // the two exchange buffers of the pass; this item's words start at ioff
  uint32_t* buf0 = s_buf;
  uint32_t* buf1 = s_buf + IPP * N;
  const int ioff = item * N;
  const unsigned f0 = blockIdx.x * FB, c0 = blockIdx.y * CB;
  const unsigned n_items = FB * CB;
  unsigned pfl = 0, sf = 0;
  unsigned long long psat = 0;
  if (p.tail_out && p.F + 1u < (unsigned)T) {
    // a chunk shorter than the delay line keeps the old line's first frames
    // (spread over the whole grid: at full scale that is 11 x 1024 words a
    // channel)
    const unsigned D = (unsigned)T - 1u, keep = D - p.F;
    const unsigned nthr = gridDim.x * gridDim.y * 256u;
    const unsigned g = (blockIdx.y * gridDim.x + blockIdx.x) * 256u + tid;
    for (unsigned i = g; i < p.C * keep * N; i += nthr) {
      const unsigned c = i / (keep * N), r = i % (keep * N);
      const unsigned k = p.F + r / N, ph = r % N;
      p.tail_out[((size_t)c * D + k) * N + ph] = p.tail[((size_t)c * D + (k - p.F)) * N + ph];
    }
  }
  __syncthreads();
  for (unsigned base = 0; base < n_items; base += IPP) {
    const unsigned it = base + item;
    const unsigned fb = it / CB, cc = it % CB;
    const unsigned f = f0 + fb, c = c0 + cc;
    const bool ok = it < n_items && f < p.F && c < p.C;
    uint32_t* tile_row = s_tile + (size_t)fb * N * cbp + tile_skew<N>(fb * N) + cc;
    const bool big = front_pass_body<NL, SPC, TT, false, SH1, EXT>(p, T, q, tl, ok, f, c, s_tw, buf0,
                                                              buf1, ioff, tile_row, cbp, pfl, psat, sf);
    if (big)  // the exact path: saturation and per-sub-stage flags
      front_pass_flags<NL, SPC, TT, SH1, EXT>(p, T, q, tl, ok, f, c, s_tw, buf0, buf1, ioff, tile_row, cbp,
                                         &sf);
  }
  __syncthreads();
  // the tile [FB][N][CB] into the ring [slot][bin][C], CB channels of a bin
  // contiguous
  if ((CB & (CB - 1u)) == 0u) {
    // CB a power of two (it divides 256): every thread keeps one channel and
    // steps over (frame, bin) rows
    const unsigned lcb = (unsigned)__ffs(CB) - 1u;
    const unsigned cc = tid & (CB - 1u), c = c0 + cc;
    const unsigned rows = FB * N;
    if (c < p.C)
      for (unsigned r = (unsigned)tid >> lcb; r < rows; r += 256u >> lcb) {
        const unsigned fb = r / N, bin = r % N;
        const unsigned f = f0 + fb;
        if (f < p.F) {
          unsigned slot = p.ring_base + f;
          if (slot >= p.ring_frames) slot -= p.ring_frames;
          p.ring[((size_t)slot * N + bin) * p.C + c] = s_tile[r * cbp + tile_skew<N>(r) + cc];
        }
      }
  } else {
    const unsigned tile_n = FB * N * CB;
    for (unsigned k = tid; k < tile_n; k += 256u) {
      const unsigned fb = k / (N * CB), rem = k % (N * CB);
      const unsigned bin = rem / CB, cc = rem % CB;
      const unsigned f = f0 + fb, c = c0 + cc;
      if (f < p.F && c < p.C) {
        unsigned slot = p.ring_base + f;
        if (slot >= p.ring_frames) slot -= p.ring_frames;
        const unsigned r = fb * N + bin;
        p.ring[((size_t)slot * N + bin) * p.C + c] = s_tile[(size_t)r * cbp + tile_skew<N>(r) + cc];
      }
    }
  }
  const unsigned a = __reduce_or_sync(0xffffffffu, pfl);
  const unsigned b = __reduce_or_sync(0xffffffffu, sf);
  unsigned long long cnt = psat;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((tid & 31) == 0) {
    if (a) atomicOr(&p.stats->pfb_flags, a);
    if (b) atomicOr(&p.stats->fft_flags, b);
    if (cnt) atomicAdd(&p.stats->pfb_sat, cnt);
  }
}

template <int NL, int SPC, int TT, bool SH1, bool EXT = false>
void launch_fast(const FrontParams& p, cudaStream_t s) {
  using G = Geo<NL, SPC>;
  constexpr int N = G::N, TPI = G::TPI, IPP = 256 / TPI;
  unsigned CB = p.C < 16u ? p.C : 16u;
  unsigned FB = 1;
  while (FB * CB < (unsigned)IPP) FB *= 2;   // at least one full pass of items
  while (FB * CB * N > 8192u && FB > 1u) FB /= 2;
  while (FB * CB * N > 8192u && CB > 1u) CB /= 2;
  const size_t smem = (2u * IPP * N + tile_words<N>(FB, CB)) * sizeof(uint32_t);
  static PerDevice attr;
  attr.once([] {
    cudaFuncSetAttribute(k_front_fast<NL, SPC, TT, SH1, EXT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, 120 * 1024);
  });
  const dim3 grid((p.F + FB - 1) / FB, (p.C + CB - 1) / CB);
  k_front_fast<NL, SPC, TT, SH1, EXT><<<grid, 256, smem, s>>>(p, FB, CB);
}

// The taps specialised at compile time (and, for them, the schedule that
// halves at every sub-stage); other tap counts up to 16 run the generic-tap
// instantiation. False when T > 16.
template <int NL, int SPC>
bool dispatch_t(const FrontParams& p, cudaStream_t s) {
  const uint32_t all = (2u << NL) - 1u;  // sub-stages 0 .. NL (the merge at NL)
  const bool sh1 = (p.sched & all) == all;
  if (p.pfb_in) {  // the PFB pass ran (k_pfb_rows.cu: taps 4, 8, 16)
    switch (p.T) {
      case 4: sh1 ? launch_fast<NL, SPC, 4, true, true>(p, s) : launch_fast<NL, SPC, 4, false, true>(p, s); return true;
      case 8: sh1 ? launch_fast<NL, SPC, 8, true, true>(p, s) : launch_fast<NL, SPC, 8, false, true>(p, s); return true;
      case 16: sh1 ? launch_fast<NL, SPC, 16, true, true>(p, s) : launch_fast<NL, SPC, 16, false, true>(p, s); return true;
      default: return false;
    }
  }
  switch (p.T) {
    case 4: sh1 ? launch_fast<NL, SPC, 4, true>(p, s) : launch_fast<NL, SPC, 4, false>(p, s); return true;
    case 8: sh1 ? launch_fast<NL, SPC, 8, true>(p, s) : launch_fast<NL, SPC, 8, false>(p, s); return true;
    case 16: sh1 ? launch_fast<NL, SPC, 16, true>(p, s) : launch_fast<NL, SPC, 16, false>(p, s); return true;
    default:
      if (p.T <= 16) {
        launch_fast<NL, SPC, 0, false>(p, s);
        return true;
      }
      return false;
  }
}

// Per translation unit: the geometries it instantiates.
bool launch_front_fast_small(const FrontParams& p, cudaStream_t s);  // N 16, 64
bool launch_front_fast_256(const FrontParams& p, cudaStream_t s);    // N 256
bool launch_front_fast_1024(const FrontParams& p, cudaStream_t s);   // N 1024

}  // namespace rd
