/*
 * orc_port.c - plain-C restatement of the reference model's chain.
 *
 * TEST INFRASTRUCTURE ONLY. This is the CPU oracle that checks the CUDA
 * product and the CPU baseline it is timed against. It restates, in this
 * project's own code, the algorithms of the reference's bit-exact model
 * (fpga-professional-association/agilex-7-radar-detect, model/cpp), each
 * function citing the reference lines it follows, and composes them in the
 * order rtl/top/benchmark_sim_top.sv wires the blocks. It is pinned against
 * the reference's own golden vectors (model/vectors) and against the
 * reference headers themselves (oracle/ref_chain.cpp) by tests/.
 *
 * Nothing in the product links or loads this file.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"

/* ------------------------------------------------------------------------ */
/* fxp primitives (model/cpp/fxp/fxp.hpp)                                   */
/* ------------------------------------------------------------------------ */

typedef int64_t wide;
typedef struct { int16_t re, im; } cpx;

static cpx unpack(uint32_t p) {
  cpx c;
  c.re = (int16_t)(uint16_t)(p & 0xFFFFu);
  c.im = (int16_t)(uint16_t)(p >> 16);
  return c;
}
static uint32_t pack(cpx c) {
  return ((uint32_t)(uint16_t)c.im << 16) | (uint32_t)(uint16_t)c.re;
}

/* wrap-safe arithmetic, fxp.hpp:87-110 */
static wide add_wrap(wide a, wide b) { return (wide)((uint64_t)a + (uint64_t)b); }
static wide sub_wrap(wide a, wide b) { return (wide)((uint64_t)a - (uint64_t)b); }
static wide neg_wrap(wide a) { return (wide)(0ULL - (uint64_t)a); }
static wide asr(wide v, unsigned s) {
  if (s == 0) return v;
  if (s >= 64) return v < 0 ? -1 : 0;
  uint64_t logical = (uint64_t)v >> s;
  uint64_t fill = v < 0 ? (~0ULL << (64 - s)) : 0ULL;
  return (wide)(logical | fill);
}
/* fxp.hpp:116-126 */
static wide max_of(unsigned w) {
  if (w >= 64) return INT64_MAX;
  if (w < 2) return 0;
  return (wide)((1ULL << (w - 1)) - 1ULL);
}
static wide min_of(unsigned w) {
  if (w >= 64) return INT64_MIN;
  if (w < 2) return 0;
  return neg_wrap((wide)(1ULL << (w - 1)));
}
/* packed {sat_pos<<1 | sat_neg}, fxp.hpp:148-165 */
static unsigned sat_flags(wide v, unsigned w) {
  return (v > max_of(w) ? 2u : 0u) | (v < min_of(w) ? 1u : 0u);
}
static wide sat(wide v, unsigned w) {
  if (v > max_of(w)) return max_of(w);
  if (v < min_of(w)) return min_of(w);
  return v;
}
/* fxp.hpp:191-215 */
static wide round_half_up(wide v, unsigned s) {
  if (s == 0) return v;
  if (s >= 64) return 0;
  return asr(add_wrap(v, (wide)(1ULL << (s - 1))), s);
}
static wide round_even(wide v, unsigned s) {
  if (s == 0) return v;
  if (s >= 64) return 0;
  wide q = asr(v, s);
  uint64_t rem = (uint64_t)v & ((1ULL << s) - 1ULL);
  uint64_t half = 1ULL << (s - 1);
  if (rem > half) return add_wrap(q, 1);
  if (rem < half) return q;
  return add_wrap(q, (wide)((uint64_t)q & 1ULL));
}
static wide rnd(wide v, unsigned s) { return round_even(v, s); }
static wide round_sat(wide v, unsigned s, unsigned w) { return sat(rnd(v, s), w); }
static unsigned round_sat_flags(wide v, unsigned s, unsigned w) {
  return sat_flags(rnd(v, s), w);
}
/* fxp.hpp:261-311 */
static int32_t mul_q15(int16_t a, int16_t b) { return (int32_t)((wide)a * (wide)b); }
static wide cmul_re_raw(cpx a, cpx b) {
  return sub_wrap((wide)mul_q15(a.re, b.re), (wide)mul_q15(a.im, b.im));
}
static wide cmul_im_raw(cpx a, cpx b) {
  return add_wrap((wide)mul_q15(a.re, b.im), (wide)mul_q15(a.im, b.re));
}
/* fxp.hpp:314-318, rounded once after the exact two-term sum */
static cpx cmul_q15(cpx a, cpx b, unsigned* fl) {
  wide r = cmul_re_raw(a, b), i = cmul_im_raw(a, b);
  cpx o;
  if (fl) *fl |= round_sat_flags(r, 15, 16) | round_sat_flags(i, 15, 16);
  o.re = (int16_t)round_sat(r, 15, 16);
  o.im = (int16_t)round_sat(i, 15, 16);
  return o;
}
/* fxp.hpp:334-352 */
static unsigned growth_bits(unsigned n) {
  if (n <= 1) return 0;
  unsigned b = 0, v = n - 1u;
  while (v) { v >>= 1; ++b; }
  return b;
}

int orc_fxp_apply(const uint32_t* op, const int64_t* a, const int64_t* b,
                  const uint32_t* sh, const uint32_t* w, uint64_t n, int64_t* y,
                  uint8_t* flags) {
  /* the op dispatch of fxp_ops.hpp:109-177 */
  for (uint64_t i = 0; i < n; ++i) {
    wide r = 0;
    unsigned f = 0;
    const wide A = a[i], B = b[i];
    const unsigned S = sh[i], W = w[i];
    switch (op[i]) {
      case RD_OP_SAT: r = sat(A, W); f = sat_flags(A, W); break;
      case RD_OP_TRUNC: r = asr(A, S); break;
      case RD_OP_ROUND_EVEN: r = round_even(A, S); break;
      case RD_OP_ROUND_HALF_UP: r = round_half_up(A, S); break;
      case RD_OP_ROUND: r = rnd(A, S); break;
      case RD_OP_ROUND_SAT: r = round_sat(A, S, W); f = round_sat_flags(A, S, W); break;
      case RD_OP_ADD_SAT: r = sat(add_wrap(A, B), W); f = sat_flags(add_wrap(A, B), W); break;
      case RD_OP_SUB_SAT: r = sat(sub_wrap(A, B), W); f = sat_flags(sub_wrap(A, B), W); break;
      case RD_OP_NEG_SAT: r = sat(neg_wrap(A), W); f = sat_flags(neg_wrap(A), W); break;
      case RD_OP_MUL_Q15:
        r = mul_q15((int16_t)(uint16_t)((uint64_t)A & 0xFFFF), (int16_t)(uint16_t)((uint64_t)B & 0xFFFF));
        break;
      case RD_OP_MUL_Q15_RS: {
        wide p = mul_q15((int16_t)(uint16_t)((uint64_t)A & 0xFFFF), (int16_t)(uint16_t)((uint64_t)B & 0xFFFF));
        r = round_sat(p, 15, 16);
        f = round_sat_flags(p, 15, 16);
        break;
      }
      case RD_OP_CMUL_RE:
      case RD_OP_CMUL_IM: {
        cpx ca = unpack((uint32_t)((uint64_t)A & 0xFFFFFFFFu));
        cpx cb = unpack((uint32_t)((uint64_t)B & 0xFFFFFFFFu));
        wide raw = op[i] == RD_OP_CMUL_RE ? cmul_re_raw(ca, cb) : cmul_im_raw(ca, cb);
        r = round_sat(raw, 15, 16);
        f = round_sat_flags(raw, 15, 16);
        break;
      }
      case RD_OP_ACC_W: r = (wide)(W + growth_bits((uint32_t)((uint64_t)A & 0xFFFFFFFFu))); break;
      case RD_OP_GROWTH_BITS: r = (wide)growth_bits((uint32_t)((uint64_t)A & 0xFFFFFFFFu)); break;
      default: return RD_EINVAL;
    }
    y[i] = r;
    flags[i] = (uint8_t)f;
  }
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* Twiddle table: W_1024^e = exp(-j 2 pi e / 1024) in Q1.15, RNE then       */
/* saturate, with exact quadrant symmetry (the algorithm of                 */
/* model/python/gen_fft_twiddles.py:97-162; table fft_twiddle_table.hpp:43) */
/* ------------------------------------------------------------------------ */

static uint32_t g_tw[1024];
static pthread_once_t g_tw_once = PTHREAD_ONCE_INIT;

static int32_t q15_of(double x) {
  double v = nearbyint(x * 32768.0); /* default rounding mode: ties to even */
  if (v > 32767.0) return 32767;
  if (v < -32768.0) return -32768;
  return (int32_t)v;
}

static void build_twiddles(void) {
  for (unsigned e = 0; e < 1024; ++e) {
    unsigned quadrant = e / 256, rem = e % 256;
    double c0 = 1.0, s0 = 0.0;
    if (rem != 0) {
      double th = 2.0 * 3.14159265358979323846 * (double)rem / 1024.0;
      c0 = cos(th);
      s0 = sin(th);
    }
    double c, s;
    switch (quadrant) {
      case 0: c = c0; s = s0; break;
      case 1: c = -s0; s = c0; break;
      case 2: c = -c0; s = -s0; break;
      default: c = s0; s = -c0; break;
    }
    cpx w;
    w.re = (int16_t)q15_of(c);
    w.im = (int16_t)q15_of(-s);
    g_tw[e] = pack(w);
  }
}

void orc_twiddles(uint32_t* out) {
  pthread_once(&g_tw_once, build_twiddles);
  memcpy(out, g_tw, sizeof(g_tw));
}

/* ------------------------------------------------------------------------ */
/* FFT (model/cpp/fft/fft_ref.hpp)                                          */
/* ------------------------------------------------------------------------ */

static unsigned log2u(unsigned v) {
  unsigned r = 0;
  while ((1u << r) < v) ++r;
  return r;
}
static unsigned bitrev(unsigned v, unsigned w) { /* fft_ref.hpp:93-99 */
  unsigned r = 0;
  for (unsigned i = 0; i < w; ++i)
    if ((v >> i) & 1u) r |= 1u << (w - 1 - i);
  return r;
}
static cpx tw(unsigned l2l, unsigned e) { /* fft_ref.hpp:131-133 */
  return unpack(g_tw[e << (10 - l2l)]);
}
static unsigned r22_tw_exp(unsigned l2l, unsigned p) { /* fft_ref.hpp:123-129 */
  unsigned q = p & ((1u << l2l) - 1u);
  unsigned k1 = (q >> (l2l - 1)) & 1u;
  unsigned k2 = (q >> (l2l - 2)) & 1u;
  unsigned n3 = q & ((1u << (l2l - 2)) - 1u);
  return n3 * (k1 + 2u * k2);
}
/* round once then saturate, flags of the rounded value (fft_ref.hpp:315-319) */
static int16_t quant(wide v, unsigned sh, unsigned* acc) {
  wide r = rnd(v, sh);
  *acc |= sat_flags(r, 16);
  return (int16_t)sat(r, 16);
}
/* -j * c with a saturating negate (fft_ref.hpp:322-331) */
static cpx neg_j(cpx c, unsigned* acc) {
  *acc |= sat_flags(neg_wrap(c.re), 16);
  cpx o;
  o.re = c.im;
  o.im = (int16_t)sat(neg_wrap(c.re), 16);
  return o;
}
/* one BF2I/BF2II sub-stage in place (fft_ref.hpp:334-365) */
static void butterfly_stage(cpx* v, unsigned m, unsigned nl, unsigned s,
                            unsigned sched, unsigned* acc) {
  const unsigned l = 1u << (nl - s), half = l / 2, sh = (sched >> s) & 1u;
  const int bf2ii = (s % 2) == 1;
  for (unsigned b = 0; b < m; b += l) {
    const int k1 = bf2ii && (((b / l) & 1u) != 0u);
    for (unsigned i = 0; i < half; ++i) {
      cpx a = v[b + i], t = v[b + half + i];
      if (k1) t = neg_j(t, acc);
      cpx lo, hi;
      lo.re = quant((wide)a.re + t.re, sh, acc);
      lo.im = quant((wide)a.im + t.im, sh, acc);
      hi.re = quant((wide)a.re - t.re, sh, acc);
      hi.im = quant((wide)a.im - t.im, sh, acc);
      v[b + i] = lo;
      v[b + half + i] = hi;
    }
  }
}
/* the group-closing twiddle multiplier (fft_ref.hpp:368-377) */
static void twiddle_stage(cpx* v, unsigned m, unsigned nl, unsigned s, unsigned* acc) {
  const unsigned l2l = nl - s + 1;
  for (unsigned i = 0; i < m; ++i) v[i] = cmul_q15(v[i], tw(l2l, r22_tw_exp(l2l, i)), acc);
}

/* fft::Engine::run (fft_ref.hpp:250-308). out/bins may be NULL. */
static void fft_frame(unsigned n, unsigned p, unsigned sched, int reorder,
                      const uint32_t* in, uint32_t* out, uint32_t* bins,
                      unsigned* stage_flags /* [log2 n] */) {
  const unsigned m = n / p, nl = log2u(m);
  cpx lane[2][1024];
  cpx beats[1024];
  for (unsigned t = 0; t < m; ++t)
    for (unsigned q = 0; q < p; ++q) lane[q][t] = unpack(in[t * p + q]);
  for (unsigned q = 0; q < p; ++q)
    for (unsigned s = 0; s < nl; ++s) {
      butterfly_stage(lane[q], m, nl, s, sched, &stage_flags[s]);
      if ((s % 2) == 1 && s + 1 < nl) twiddle_stage(lane[q], m, nl, s, &stage_flags[s]);
    }
  if (p == 1) {
    for (unsigned j = 0; j < m; ++j) beats[j] = lane[0][j];
  } else { /* radix-2 DIT merge (fft_ref.hpp:380-406) */
    const unsigned sh = (sched >> nl) & 1u;
    for (unsigned j = 0; j < m; ++j) {
      const cpx w = tw(nl + 1, bitrev(j & ((1u << nl) - 1u), nl));
      const cpx t = cmul_q15(lane[1][j], w, &stage_flags[nl]);
      const cpx e = lane[0][j];
      cpx lo, hi;
      lo.re = quant((wide)e.re + t.re, sh, &stage_flags[nl]);
      lo.im = quant((wide)e.im + t.im, sh, &stage_flags[nl]);
      hi.re = quant((wide)e.re - t.re, sh, &stage_flags[nl]);
      hi.im = quant((wide)e.im - t.im, sh, &stage_flags[nl]);
      beats[2 * j] = lo;
      beats[2 * j + 1] = hi;
    }
  }
  for (unsigned j = 0; j < m; ++j) {
    const unsigned mj = bitrev(j, nl);
    for (unsigned q = 0; q < p; ++q) {
      if (bins) bins[mj + q * (n / p)] = pack(beats[j * p + q]);
      if (out)
        out[j * p + q] = pack(reorder ? beats[bitrev(j, nl) * p + q] : beats[j * p + q]);
    }
  }
}

static int fft_cfg_ok(unsigned n, unsigned spc) { /* fft_ref.hpp:216-219 */
  return n >= 8 && n <= 1024 && (n & (n - 1)) == 0 && (spc == 1 || spc == 2) &&
         n / spc >= 4;
}

int orc_fft_run(uint32_t n_fft, uint32_t spc, uint32_t scale_sched, int reorder,
                const rd_cplx16* in, uint32_t frames, rd_cplx16* out,
                rd_cplx16* bins, uint8_t* stage_flags) {
  if (!fft_cfg_ok(n_fft, spc)) return RD_EINVAL;
  pthread_once(&g_tw_once, build_twiddles);
  const unsigned st = log2u(n_fft);
  for (uint32_t f = 0; f < frames; ++f) {
    unsigned sf[11] = {0};
    fft_frame(n_fft, spc, scale_sched, reorder, in + (size_t)f * n_fft,
              out ? out + (size_t)f * n_fft : NULL, bins ? bins + (size_t)f * n_fft : NULL, sf);
    if (stage_flags)
      for (unsigned s = 0; s < st; ++s) stage_flags[(size_t)f * st + s] = (uint8_t)sf[s];
  }
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* PFB (model/cpp/pfb/pfb_model.hpp:139-177, 242-251)                       */
/* ------------------------------------------------------------------------ */

/* One output of lane p: acc = sum_k h_p[k] * x[n-k], exact int64, quantised
 * once with round_sat(acc, 15, 16). `hist(k)` supplies x[n-k]. */
static cpx pfb_out(const cpx* h, unsigned taps, const cpx* xs /* xs[k] = x[n-k] */,
                   unsigned* f_re, unsigned* f_im) {
  wide re = 0, im = 0;
  for (unsigned k = 0; k < taps; ++k) {
    re = add_wrap(re, cmul_re_raw(xs[k], h[k]));
    im = add_wrap(im, cmul_im_raw(xs[k], h[k]));
  }
  cpx y;
  y.re = (int16_t)round_sat(re, 15, 16);
  y.im = (int16_t)round_sat(im, 15, 16);
  *f_re = round_sat_flags(re, 15, 16);
  *f_im = round_sat_flags(im, 15, 16);
  return y;
}

int orc_pfb_run(uint32_t phases, uint32_t taps, const rd_cplx16* coeff,
                rd_cplx16* state, const rd_cplx16* in, uint32_t beats,
                rd_cplx16* out, uint8_t* flags_out) {
  if (taps == 0 || taps > 64) return RD_EINVAL;
  cpx h[64], xs[64];
  /* sequence view: index j < taps-1 are the delay line, oldest first */
  const unsigned d = taps - 1;
  for (unsigned p = 0; p < phases; ++p) {
    for (unsigned k = 0; k < taps; ++k) h[k] = unpack(coeff[(size_t)p * taps + k]);
    for (uint32_t t = 0; t < beats; ++t) {
      for (unsigned k = 0; k < taps; ++k) {
        /* x[n-k]: beat t-k of the input, or delay-line entry k-t-1 */
        xs[k] = (k <= t) ? unpack(in[(size_t)(t - k) * phases + p])
                         : unpack(state[(size_t)(k - t - 1) * phases + p]);
      }
      unsigned fr, fi;
      const cpx y = pfb_out(h, taps, xs, &fr, &fi);
      out[(size_t)t * phases + p] = pack(y);
      if (flags_out) flags_out[(size_t)t * phases + p] = (uint8_t)((fr << 2) | fi);
    }
    /* advance the delay line (pfb_model.hpp:170-175) */
    if (d > 0) {
      rd_cplx16 ns[64];
      for (unsigned k = 0; k < d; ++k)
        ns[k] = (k < beats) ? in[(size_t)(beats - 1 - k) * phases + p]
                            : state[(size_t)(k - beats) * phases + p];
      for (unsigned k = 0; k < d; ++k) state[(size_t)k * phases + p] = ns[k];
    }
  }
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* Beamformer dot product (beamformer_model.hpp:162-179)                    */
/* ------------------------------------------------------------------------ */

static cpx bf_dot(const cpx* x, const cpx* w, unsigned n, wide* are, wide* aim,
                  unsigned* f_re, unsigned* f_im) {
  wide r = 0, i = 0;
  for (unsigned a = 0; a < n; ++a) {
    r = add_wrap(r, cmul_re_raw(x[a], w[a]));
    i = add_wrap(i, cmul_im_raw(x[a], w[a]));
  }
  cpx y;
  y.re = (int16_t)round_sat(r, 15, 16);
  y.im = (int16_t)round_sat(i, 15, 16);
  *f_re = sat_flags(rnd(r, 15), 16);
  *f_im = sat_flags(rnd(i, 15), 16);
  if (are) *are = r;
  if (aim) *aim = i;
  return y;
}

int orc_bf_run(uint32_t n_ant, uint32_t n_beams, const rd_cplx16* w,
               const rd_cplx16* x, uint64_t n_vec, rd_cplx16* y, int64_t* acc,
               uint8_t* flags) {
  cpx* wc = malloc(sizeof(cpx) * (size_t)n_ant * n_beams);
  cpx* xc = malloc(sizeof(cpx) * n_ant);
  for (size_t i = 0; i < (size_t)n_ant * n_beams; ++i) wc[i] = unpack(w[i]);
  for (uint64_t v = 0; v < n_vec; ++v) {
    for (unsigned a = 0; a < n_ant; ++a) xc[a] = unpack(x[v * n_ant + a]);
    for (unsigned b = 0; b < n_beams; ++b) {
      wide r, i;
      unsigned fr, fi;
      cpx o = bf_dot(xc, wc + (size_t)b * n_ant, n_ant, &r, &i, &fr, &fi);
      y[v * n_beams + b] = pack(o);
      if (acc) {
        acc[(v * n_beams + b) * 2] = r;
        acc[(v * n_beams + b) * 2 + 1] = i;
      }
      if (flags) flags[v * n_beams + b] = (uint8_t)((fr << 2) | fi);
    }
  }
  free(wc);
  free(xc);
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* Power and cross power (covar_model.hpp:99-151)                           */
/* ------------------------------------------------------------------------ */

static wide power(cpx s) { return (wide)mul_q15(s.re, s.re) + (wide)mul_q15(s.im, s.im); }
/* X * conj(Y) through the operand-swap wiring (covar_model.hpp:137-145) */
static void cross_power(cpx x, cpx y, wide* re, wide* im) {
  cpx b;
  b.re = y.im;
  b.im = y.re;
  *re = cmul_im_raw(x, b);
  *im = neg_wrap(cmul_re_raw(x, b));
}

int orc_power_run(const rd_cplx16* x, uint64_t n, int64_t* p) {
  for (uint64_t i = 0; i < n; ++i) p[i] = power(unpack(x[i]));
  return RD_OK;
}
int orc_cross_power_run(const rd_cplx16* x, const rd_cplx16* y, uint64_t n, int64_t* c) {
  for (uint64_t i = 0; i < n; ++i) cross_power(unpack(x[i]), unpack(y[i]), &c[2 * i], &c[2 * i + 1]);
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* Integrator (covar_model.hpp:186-288)                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
  wide acc;
  uint32_t count, window_id;
  uint32_t sticky, sat_count;
} integ;

typedef struct {
  wide acc;
  uint32_t window_id, sample_count;
  int flushed, truncated;
} integ_result;

/* One step in block or exponential mode with a fixed configuration. Returns 1
 * when a window result is registered (covar_model.hpp:204-262). */
static int integ_step(integ* s, unsigned acc_w, unsigned wl_cfg, int exp_mode,
                      unsigned exp_k, int valid, wide data, int flush, integ_result* out) {
  const unsigned wl = wl_cfg == 0 ? 1u : wl_cfg;
  const int accept = valid;
  wide raw = s->acc;
  if (accept) raw = exp_mode ? add_wrap(s->acc, asr(sub_wrap(data, s->acc), exp_k))
                             : add_wrap(s->acc, data);
  const unsigned step_flags = accept ? sat_flags(raw, acc_w) : 0u;
  const wide acc_next = sat(raw, acc_w);
  const unsigned count_next = accept ? s->count + 1u : s->count;
  const int close = accept && count_next >= wl;
  const int flush_emit = flush && !close && count_next != 0u;
  const int emit = close || flush_emit;
  if (emit && out) {
    out->acc = acc_next;
    out->window_id = s->window_id;
    out->sample_count = count_next;
    out->flushed = flush;
    out->truncated = count_next != wl;
  }
  if (flush) { /* sticky flags cleared by flush (fxp.hpp:361-370) */
    s->sticky = 0;
    s->sat_count = 0;
  } else if (accept) {
    s->sticky |= step_flags;
    if (step_flags && s->sat_count != 0xFFFFFFFFu) s->sat_count++;
  }
  if (flush) {
    s->acc = 0;
    s->count = 0;
    s->window_id = 0;
  } else if (close) {
    s->acc = exp_mode ? acc_next : 0;
    s->count = 0;
    s->window_id = (s->window_id + 1u) & 0xFFFFu;
  } else {
    s->acc = acc_next;
    s->count = count_next;
  }
  return emit;
}

/* ------------------------------------------------------------------------ */
/* CFAR (model/cpp/cfar/cfar_model.hpp:134-340)                             */
/* ------------------------------------------------------------------------ */

typedef struct {
  int enable, go, dense;
  unsigned gl, gg, rl, rg; /* guard lead/lag, ref lead/lag after the clamp */
  unsigned alpha;
} cfar_cfg;

static cfar_cfg cfar_clamp(const rd_config* c) { /* cfar_model.hpp:134-141 */
  cfar_cfg k;
  k.enable = c->cfar_enable != 0;
  k.go = c->cfar_mode == RD_CFAR_GO;
  k.dense = c->cfar_out_mode == RD_CFAR_DENSE;
  k.gl = c->guard_lead > c->max_guard ? c->max_guard : c->guard_lead;
  k.gg = c->guard_lag > c->max_guard ? c->max_guard : c->guard_lag;
  k.rl = c->ref_lead > c->max_ref ? c->max_ref : c->ref_lead;
  k.rg = c->ref_lag > c->max_ref ? c->max_ref : c->ref_lag;
  k.alpha = c->alpha;
  return k;
}

static void set_bits(uint64_t* w, unsigned lsb, unsigned n, uint64_t v) {
  for (unsigned i = 0; i < n; ++i) {
    unsigned b = lsb + i;
    if ((v >> i) & 1ULL) w[b / 64] |= 1ULL << (b % 64);
  }
}

/* 176-bit event layout, cfar_model.hpp:75-84 */
static rd_event make_event(unsigned kind, unsigned bin, unsigned frame_id,
                           unsigned ref_cnt, unsigned alpha, unsigned det,
                           unsigned sup, uint64_t cut, uint64_t sum, int sof,
                           int eof, uint32_t frame, uint16_t beam) {
  rd_event e;
  memset(&e, 0, sizeof(e));
  set_bits(e.w, 0, 2, kind);
  set_bits(e.w, 2, 16, bin);
  set_bits(e.w, 18, 16, frame_id);
  set_bits(e.w, 34, 7, ref_cnt);
  set_bits(e.w, 41, 16, alpha);
  set_bits(e.w, 57, 16, det);
  set_bits(e.w, 73, 16, sup);
  set_bits(e.w, 89, 40, cut);
  set_bits(e.w, 129, 47, sum);
  e.frame = frame;
  e.beam = beam;
  e.kind = (uint8_t)kind;
  e.framing = (uint8_t)((sof ? 1 : 0) | (eof ? 2 : 0));
  return e;
}

/* run_frame over n clamped cells (cfar_model.hpp:243-340). Writes up to
 * cap events into ev and returns the number produced. `pre` is scratch of
 * n+1 entries for the prefix sums that stand in for the reference's
 * per-cell reference-window loops (same integer sums). */
static uint64_t cfar_frame(const uint64_t* cells, unsigned n, const cfar_cfg* k,
                           unsigned frame_id, uint32_t frame, uint16_t beam,
                           uint64_t* pre, rd_event* ev, uint64_t cap,
                           unsigned* det_out, unsigned* sup_out) {
  pre[0] = 0;
  for (unsigned i = 0; i < n; ++i) pre[i + 1] = pre[i] + cells[i];
  const int usable = k->go ? (k->rl != 0 && k->rg != 0) : (k->rl + k->rg) != 0;
  unsigned det = 0, sup = 0;
  uint64_t m = 0;
  for (unsigned i = 0; i < n; ++i) {
    const int64_t hi = (int64_t)i + k->gl + k->rl; /* last lead cell */
    const int64_t lo = (int64_t)i - (int64_t)k->gg - (int64_t)k->rg; /* first lag cell */
    const int ok = hi < (int64_t)n && lo >= 0;
    uint64_t sl = 0, sg = 0;
    if (ok) {
      sl = pre[i + k->gl + k->rl + 1] - pre[i + k->gl + 1];
      sg = pre[i - k->gg] - pre[i - k->gg - k->rg];
    }
    uint64_t ssum;
    unsigned sn;
    if (k->go) {
      const int take_lead = (sl * k->rg) >= (sg * k->rl);
      ssum = take_lead ? sl : sg;
      sn = take_lead ? k->rl : k->rg;
    } else {
      ssum = sl + sg;
      sn = k->rl + k->rg;
    }
    const int evaluable = ok && k->enable && usable;
    const int detected = evaluable && ((cells[i] * sn) << 8) > ((uint64_t)k->alpha * ssum);
    if (detected) ++det;
    if (!evaluable) ++sup;
    if (!(detected || k->dense)) continue;
    const unsigned kind = detected ? RD_EV_DETECT : (!evaluable ? RD_EV_SUPPRESSED : RD_EV_BIN);
    if (m < cap)
      ev[m] = make_event(kind, i, frame_id, evaluable ? sn : 0u, k->alpha, 0, 0,
                         cells[i], evaluable ? ssum : 0u, m == 0, 0, frame, beam);
    ++m;
  }
  if (m < cap)
    ev[m] = make_event(RD_EV_SUMMARY, n, frame_id, 0, k->alpha, det, sup, 0, 0,
                       m == 0, 1, frame, beam);
  ++m;
  *det_out = det;
  *sup_out = sup;
  return m;
}

int orc_cfar_run(const int64_t* cells, uint32_t n, uint32_t frames,
                 const rd_config* c, const uint32_t* frame_ids, rd_event* events,
                 uint64_t cap, uint64_t* n_events) {
  cfar_cfg k = cfar_clamp(c);
  uint64_t* pre = malloc(sizeof(uint64_t) * (n + 1));
  uint64_t* cl = malloc(sizeof(uint64_t) * (n ? n : 1));
  rd_event* tmp = malloc(sizeof(rd_event) * (n + 1));
  uint64_t tot = 0;
  for (uint32_t f = 0; f < frames; ++f) {
    for (uint32_t i = 0; i < n; ++i) {
      const int64_t v = cells[(size_t)f * n + i];
      cl[i] = v < 0 ? 0u : (uint64_t)v; /* clamp_cell, cfar_model.hpp:238-240 */
    }
    unsigned d, s;
    uint64_t m = cfar_frame(cl, n, &k, frame_ids[f], frame_ids[f], (uint16_t)f, pre, tmp, n + 1, &d, &s);
    for (uint64_t j = 0; j < m; ++j) {
      if (tot + j < cap) events[tot + j] = tmp[j];
    }
    tot += m;
  }
  free(pre);
  free(cl);
  free(tmp);
  *n_events = tot;
  return tot > cap ? RD_ETRUNC : RD_OK;
}

/* ------------------------------------------------------------------------ */
/* Packets (packet_model.hpp:74-260; DMA tap benchmark_sim_top.sv:1818-1936)*/
/* ------------------------------------------------------------------------ */

uint32_t rd_flit_words(uint32_t packet_w) { return (packet_w + 5u + 31u) / 32u; }
uint32_t rd_detection_flits(uint32_t packet_w) {
  return packet_w ? 1u + (176u + packet_w - 1u) / packet_w : 0u;
}

static void flit_set(uint32_t* w, unsigned bit, unsigned v) {
  if (v) w[bit / 32] |= 1u << (bit % 32);
}

/* make_flit: data at bit 5, eof bit 4, sof bit 3, vc bits 2:1, odd parity in
 * bit 0 (packet_model.hpp:86-91, 241-260). `data` supplies bit i of the
 * payload word. */
static void make_flit(uint32_t* w, unsigned words, unsigned pw, unsigned vc,
                      int sof, int eof, const uint64_t* data_bits, unsigned data_lsb,
                      unsigned data_n) {
  memset(w, 0, words * 4);
  flit_set(w, 1, vc & 1u);
  flit_set(w, 2, (vc >> 1) & 1u);
  flit_set(w, 3, (unsigned)sof);
  flit_set(w, 4, (unsigned)eof);
  for (unsigned i = 0; i < pw; ++i) {
    unsigned src = data_lsb + i;
    unsigned v = (i < data_n && src < 192) ? (unsigned)((data_bits[src / 64] >> (src % 64)) & 1ULL) : 0u;
    flit_set(w, 5 + i, v);
  }
  unsigned pop = 0;
  for (unsigned k = 0; k < words; ++k) pop += (unsigned)__builtin_popcount(w[k]);
  flit_set(w, 0, (pop & 1u) == 0u);
}

static void packet_flits(const rd_event* e, unsigned pw, unsigned src, unsigned dest,
                         unsigned vc, unsigned seq, uint32_t* out) {
  const unsigned words = rd_flit_words(pw), nfl = rd_detection_flits(pw);
  /* header {seq16,len6,type3,vc2,src5,dest4}, packet_model.hpp:150-159 */
  uint64_t hdr[3] = {0, 0, 0};
  hdr[0] = ((uint64_t)(dest & 0xFu)) | ((uint64_t)(src & 0x1Fu) << 4) |
           ((uint64_t)(vc & 0x3u) << 9) | ((uint64_t)0u << 11) |
           ((uint64_t)(nfl & 0x3Fu) << 14) | ((uint64_t)(seq & 0xFFFFu) << 20);
  make_flit(out, words, pw, vc, 1, nfl == 1, hdr, 0, 64);
  for (unsigned f = 1; f < nfl; ++f)
    make_flit(out + f * words, words, pw, vc, 0, f + 1 == nfl, e->w, (f - 1) * pw, pw);
}

int orc_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w, uint32_t src_id,
                  uint32_t dest, uint32_t vc, uint32_t seq0, uint32_t* flits) {
  const unsigned words = rd_flit_words(packet_w), nfl = rd_detection_flits(packet_w);
  for (uint64_t i = 0; i < n; ++i)
    packet_flits(&ev[i], packet_w, src_id, dest, vc, (unsigned)((seq0 + i) & 0xFFFFu),
                 flits + i * nfl * words);
  return RD_OK;
}

/* ------------------------------------------------------------------------ */
/* History (model/cpp/history/history_model.hpp:191-467), bookkeeping and   */
/* storage. Storage is [slot][natural bin][antenna] (stored_bin with        */
/* bit_reversed = false maps (beat, lane) to bin = lane*M + beat, :147-150). */
/* ------------------------------------------------------------------------ */

typedef struct {
  unsigned n_ant, n, lanes, frames_max;
  uint32_t* store;        /* [frames_max][n][n_ant] */
  uint32_t* resident;     /* [frames_max] */
  unsigned* beat;         /* per antenna */
  unsigned* slot;
  uint32_t* frame;
  int* in_frame;
  uint32_t frames_done;
  unsigned done_slot, depth, epoch;
  int skew_prev, framing;
  uint32_t c_overwrite, c_skew, c_wbeat, c_read, c_collision, c_error;
} histm;

static void sat_bump(uint32_t* c, uint32_t by) {
  uint64_t v = (uint64_t)*c + by;
  *c = v > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)v;
}
static unsigned clog2(unsigned v) {
  unsigned w = 0;
  while ((1u << w) < v) ++w;
  return w;
}
static unsigned w_of(unsigned c) { unsigned w = clog2(c); return w == 0 ? 1u : w; }

static void hist_init(histm* h, unsigned n_ant, unsigned n, unsigned lanes, unsigned fm) {
  memset(h, 0, sizeof(*h));
  h->n_ant = n_ant;
  h->n = n;
  h->lanes = lanes;
  h->frames_max = fm;
  h->store = calloc((size_t)fm * n * n_ant, sizeof(uint32_t));
  h->resident = malloc(sizeof(uint32_t) * fm);
  for (unsigned i = 0; i < fm; ++i) h->resident[i] = 0xFFFFFFFFu;
  h->beat = calloc(n_ant, sizeof(unsigned));
  h->slot = calloc(n_ant, sizeof(unsigned));
  h->frame = calloc(n_ant, sizeof(uint32_t));
  h->in_frame = calloc(n_ant, sizeof(int));
  h->depth = fm;
}
static void hist_free(histm* h) {
  free(h->store); free(h->resident); free(h->beat); free(h->slot);
  free(h->frame); free(h->in_frame);
}
/* settle_ without depth changes (history_model.hpp:410-433) */
static void hist_settle(histm* h) {
  for (;;) {
    int all_past = 1;
    for (unsigned a = 0; a < h->n_ant; ++a)
      if (h->frame[a] == h->frames_done) all_past = 0;
    if (!all_past) break;
    if (h->frames_done >= h->depth) sat_bump(&h->c_overwrite, 1);
    h->frames_done += 1;
    if (h->frames_done != 1) h->done_slot = (h->done_slot + 1 == h->depth) ? 0u : h->done_slot + 1u;
  }
  int skew_now = 0;
  for (unsigned a = 0; a < h->n_ant; ++a)
    if (h->frame[a] - h->frames_done >= h->depth) skew_now = 1;
  if (skew_now && !h->skew_prev) sat_bump(&h->c_skew, 1);
  h->skew_prev = skew_now;
}
/* write_beat (history_model.hpp:228-255): `samples` are the beat's lanes */
static void hist_write_beat(histm* h, unsigned ant, const uint32_t* samples, int sof, int eof) {
  const unsigned m = h->n / h->lanes;
  const int err = (eof && h->beat[ant] != m - 1) || (!eof && h->beat[ant] == m - 1) ||
                  (sof && h->beat[ant] != 0) || (!sof && h->beat[ant] == 0);
  if (err) h->framing = 1;
  for (unsigned l = 0; l < h->lanes; ++l) {
    const unsigned bin = l * m + h->beat[ant];
    h->store[((size_t)h->slot[ant] * h->n + bin) * h->n_ant + ant] = samples[l];
  }
  sat_bump(&h->c_wbeat, 1);
  h->in_frame[ant] = !eof;
  if (eof) {
    h->resident[h->slot[ant]] = h->frame[ant];
    h->beat[ant] = 0;
    h->frame[ant] += 1;
    h->slot[ant] = (h->slot[ant] + 1 == h->depth) ? 0 : h->slot[ant] + 1;
  } else {
    h->beat[ant] += 1;
  }
  hist_settle(h);
}
static unsigned hist_readable(const histm* h) { /* :373-376 */
  const unsigned dm2 = h->depth <= 2 ? 0u : h->depth - 2u;
  return h->frames_done >= dm2 ? dm2 : (unsigned)h->frames_done;
}
/* read (history_model.hpp:283-337); vec may be NULL */
static void hist_read(histm* h, unsigned bin, unsigned frame_off, uint32_t* vec,
                      uint32_t* frame_id, unsigned* flags) {
  const unsigned depth_mask = (1u << clog2(h->frames_max + 1)) - 1u;
  const unsigned slot_w = w_of(h->frames_max);
  const unsigned slot_mask = (1u << slot_w) - 1u;
  const unsigned ext_mask = (1u << (slot_w + 1)) - 1u;
  const unsigned bin_p = bin & 0xFFFFu, off_p = frame_off & 0xFFFFu;
  const unsigned rd = hist_readable(h);
  const int oor = (bin_p >= h->n) || (rd == 0) || (off_p >= rd);
  const unsigned off_clamped = rd == 0 ? 0u : rd - 1u;
  const unsigned off_safe = oor ? off_clamped : (off_p & depth_mask);
  const unsigned off_ext = off_safe & ext_mask, done_ext = h->done_slot & ext_mask;
  const unsigned slot = (done_ext >= off_ext) ? ((done_ext - off_ext) & slot_mask)
                                              : (((done_ext - off_ext + h->depth) & ext_mask) & slot_mask);
  const unsigned write_slot = (h->done_slot + 1 == h->depth) ? 0u : (h->done_slot + 1) & slot_mask;
  const int collision = (h->frames_done != 0) && (slot == write_slot);
  const uint32_t fid = (uint32_t)(h->frames_done - 1u - off_safe);
  const int stale = (uint32_t)(h->frames_done - fid) > h->depth;
  const unsigned b = bin_p % h->n;
  if (vec)
    for (unsigned a = 0; a < h->n_ant; ++a) vec[a] = h->store[((size_t)slot * h->n + b) * h->n_ant + a];
  *frame_id = fid;
  *flags = (oor ? 1u : 0u) | (collision ? 2u : 0u) | (stale ? 4u : 0u);
  sat_bump(&h->c_read, 1);
  if (collision) sat_bump(&h->c_collision, 1);
  if (oor) sat_bump(&h->c_error, 1);
}

/* ------------------------------------------------------------------------ */
/* Threading helper: static partition of [0, n) over t workers.             */
/* ------------------------------------------------------------------------ */

typedef void (*range_fn)(void* ctx, uint64_t lo, uint64_t hi, int tid);
typedef struct { range_fn fn; void* ctx; uint64_t lo, hi; int tid; } pjob;
static void* pjob_run(void* p) {
  pjob* j = (pjob*)p;
  j->fn(j->ctx, j->lo, j->hi, j->tid);
  return NULL;
}
static void parallel_for(uint64_t n, int threads, range_fn fn, void* ctx) {
  if (threads <= 1 || n < 2) { fn(ctx, 0, n, 0); return; }
  if ((uint64_t)threads > n) threads = (int)n;
  pthread_t th[256];
  pjob jobs[256];
  if (threads > 256) threads = 256;
  for (int t = 0; t < threads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].lo = n * (uint64_t)t / (uint64_t)threads;
    jobs[t].hi = n * (uint64_t)(t + 1) / (uint64_t)threads;
    jobs[t].tid = t;
  }
  for (int t = 1; t < threads; ++t) pthread_create(&th[t], NULL, pjob_run, &jobs[t]);
  pjob_run(&jobs[0]);
  for (int t = 1; t < threads; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* The chain                                                                */
/* ------------------------------------------------------------------------ */

struct orc_chain {
  rd_config cfg;
  cpx* coeff;         /* [N][T] */
  cpx* weights;       /* [B][C] */
  cpx* delay;         /* [C][T-1][N] delay line, delay[k] = x[n-1-k] */
  uint32_t* px;
  uint32_t* py;
  uint32_t n_pairs;
  integ* cov_re;      /* [N][P] */
  integ* cov_im;
  histm hist;
  uint32_t align_seq;
  uint64_t frame;
  rd_stats st;
  /* the beat-stream covariance engine: pairs (2p, 2p+1) mod B */
  unsigned eng_pairs;
  integ eng_re[128], eng_im[128];
};

/* The RTL's telemetry-only beat-stream covariance engine (covar::Engine,
 * covar_model.hpp:318-416, as benchmark_sim_top.sv:1124-1200 wires it): one
 * source vector per beamformer beat - the beams of the beat's bin_par 0, the
 * even bin 2g of beat g - pairs (2p, 2p+1) mod B, 40-bit block integrators
 * over n_fft beats, no flush. The multiplier pipeline only delays when a
 * product lands; between calls the clock runs on, so every beat has landed. */
static unsigned engine_pair_count(const rd_config* c) {
  const unsigned most = c->n_beams >= 2 ? c->n_beams / 2u : 1u;
  return c->engine_pairs < most ? c->engine_pairs : most;
}

int orc_chain_create(const rd_config* c, const rd_cplx16* coeff,
                     const rd_cplx16* weights, const uint32_t* pair_x,
                     const uint32_t* pair_y, uint32_t n_pairs, orc_chain** out) {
  const unsigned N = c->n_fft, T = c->taps, C = c->n_chan, B = c->n_beams;
  if (!fft_cfg_ok(N, c->spc) || T == 0 || T > 64 || C == 0 || B == 0) return RD_EINVAL;
  if (c->hist_frames < 4 || (c->hist_frames & (c->hist_frames - 1)) != 0) return RD_EINVAL;
  pthread_once(&g_tw_once, build_twiddles);
  orc_chain* ch = calloc(1, sizeof(*ch));
  ch->cfg = *c;
  ch->coeff = malloc(sizeof(cpx) * N * T);
  for (unsigned i = 0; i < N * T; ++i) ch->coeff[i] = unpack(coeff[i]);
  ch->weights = malloc(sizeof(cpx) * B * C);
  for (unsigned i = 0; i < B * C; ++i) ch->weights[i] = unpack(weights[i]);
  ch->delay = calloc((size_t)C * (T > 1 ? T - 1 : 1) * N, sizeof(cpx));
  if (c->cov_source != RD_COV_OFF) {
    ch->n_pairs = n_pairs;
    ch->px = malloc(sizeof(uint32_t) * (n_pairs ? n_pairs : 1));
    ch->py = malloc(sizeof(uint32_t) * (n_pairs ? n_pairs : 1));
    memcpy(ch->px, pair_x, sizeof(uint32_t) * n_pairs);
    memcpy(ch->py, pair_y, sizeof(uint32_t) * n_pairs);
    ch->cov_re = calloc((size_t)N * (n_pairs ? n_pairs : 1), sizeof(integ));
    ch->cov_im = calloc((size_t)N * (n_pairs ? n_pairs : 1), sizeof(integ));
  }
  hist_init(&ch->hist, C, N, c->spc, c->hist_frames);
  ch->st.hist_depth = ch->hist.depth;
  ch->eng_pairs = engine_pair_count(c);
  *out = ch;
  return RD_OK;
}

/* request_depth + the settle_ that lands it (history_model.hpp:260-266,
 * 435-451): between calls no antenna is mid-frame, so it lands at once and
 * discards the history */
int orc_chain_set_history_depth(orc_chain* ch, uint32_t frames) {
  histm* h = &ch->hist;
  unsigned d = frames == 0 ? 1u : frames;
  if (d > h->frames_max) d = h->frames_max;
  h->depth = d;
  h->epoch += 1;
  h->frames_done = 0;
  h->done_slot = 0;
  h->skew_prev = 0;
  for (unsigned a = 0; a < h->n_ant; ++a) {
    h->beat[a] = 0;
    h->slot[a] = 0;
    h->frame[a] = 0;
  }
  for (unsigned i = 0; i < h->frames_max; ++i) h->resident[i] = 0xFFFFFFFFu;
  ch->st.hist_frames_done = 0;
  ch->st.hist_depth = h->depth;
  ch->st.hist_epoch = h->epoch;
  return RD_OK;
}

void orc_chain_destroy(orc_chain* ch) {
  if (!ch) return;
  free(ch->coeff); free(ch->weights); free(ch->delay); free(ch->px); free(ch->py);
  free(ch->cov_re); free(ch->cov_im);
  hist_free(&ch->hist);
  free(ch);
}

int orc_chain_set_coeff(orc_chain* ch, const rd_cplx16* coeff) {
  const unsigned n = ch->cfg.n_fft * ch->cfg.taps;
  for (unsigned i = 0; i < n; ++i) ch->coeff[i] = unpack(coeff[i]);
  return RD_OK;
}
int orc_chain_set_weights(orc_chain* ch, const rd_cplx16* w) {
  const unsigned n = ch->cfg.n_beams * ch->cfg.n_chan;
  for (unsigned i = 0; i < n; ++i) ch->weights[i] = unpack(w[i]);
  return RD_OK;
}

typedef struct {
  orc_chain* ch;
  const rd_cplx16* adc;
  uint64_t ld, frames;
  uint32_t* pfb;       /* [F][C][N] */
  uint32_t* spec;      /* [F][N][C] */
  uint32_t* beams;     /* [F][B][N] */
  uint64_t* cells;     /* [F][B][N] */
  unsigned* flags_t;   /* per thread: [0] pfb, [1] bf, [2..12] fft stages */
  uint64_t* cnt_t;     /* per thread: [0] pfb sat, [1] bf sat */
  rd_event** ev;       /* per (frame, beam) */
  uint64_t* nev;
  unsigned* det;
  unsigned* sup;
  /* covariance results: per window (of this call) accumulators */
  int64_t* cov_acc;    /* [max_w][N][P][2] */
  uint32_t max_w;
  uint32_t* cov_wclose;/* frame (call-relative) where window w closed */
  integ_result* cov_hdr;
  unsigned* cov_wflags;/* [max_w] per thread-merged sticky flags */
  uint32_t n_windows;
  int threads;
} chain_ctx;

/* Phase A: PFB, sequential over frames per (channel, phase). */
static void ph_pfb(void* p, uint64_t lo, uint64_t hi, int tid) {
  chain_ctx* x = p;
  orc_chain* ch = x->ch;
  const unsigned N = ch->cfg.n_fft, T = ch->cfg.taps, C = ch->cfg.n_chan;
  cpx xs[64];
  unsigned fl = 0;
  uint64_t ns = 0;
  for (uint64_t u = lo; u < hi; ++u) {
    const unsigned a = (unsigned)(u / N), ph = (unsigned)(u % N);
    const cpx* h = ch->coeff + (size_t)ph * T;
    cpx* dl = ch->delay + (size_t)a * (T > 1 ? T - 1 : 1) * N;
    for (uint64_t f = 0; f < x->frames; ++f) {
      xs[0] = unpack(x->adc[a * x->ld + f * N + ph]);
      for (unsigned k = 1; k < T; ++k) xs[k] = dl[(size_t)(k - 1) * N + ph];
      unsigned fr, fi;
      const cpx y = pfb_out(h, T, xs, &fr, &fi);
      if (fr | fi) { fl |= fr | fi; ++ns; }
      x->pfb[(f * C + a) * N + ph] = pack(y);
      /* advance after the evaluation (pfb_model.hpp:170-175) */
      for (unsigned k = T > 1 ? T - 2 : 0; k > 0; --k) dl[(size_t)k * N + ph] = dl[(size_t)(k - 1) * N + ph];
      if (T > 1) dl[ph] = xs[0];
    }
  }
  x->flags_t[tid * 16 + 0] |= fl;
  x->cnt_t[tid * 4 + 0] += ns;
}

/* Phase B: FFT per (frame, channel), natural bins into [F][N][C]. */
static void ph_fft(void* p, uint64_t lo, uint64_t hi, int tid) {
  chain_ctx* x = p;
  orc_chain* ch = x->ch;
  const unsigned N = ch->cfg.n_fft, C = ch->cfg.n_chan;
  uint32_t bins[1024];
  unsigned sf[11] = {0};
  for (uint64_t u = lo; u < hi; ++u) {
    const uint64_t f = u / C;
    const unsigned a = (unsigned)(u % C);
    fft_frame(N, ch->cfg.spc, ch->cfg.scale_sched, 1, x->pfb + (f * C + a) * N, NULL, bins, sf);
    for (unsigned k = 0; k < N; ++k) x->spec[(f * N + k) * C + a] = bins[k];
  }
  for (unsigned s = 0; s < 11; ++s) x->flags_t[tid * 16 + 2 + s] |= sf[s];
}

/* Phase D: beamform + power per (frame, bin). */
static void ph_bf(void* p, uint64_t lo, uint64_t hi, int tid) {
  chain_ctx* x = p;
  orc_chain* ch = x->ch;
  const unsigned N = ch->cfg.n_fft, C = ch->cfg.n_chan, B = ch->cfg.n_beams;
  cpx xv[128];
  unsigned fl = 0;
  uint64_t ns = 0;
  for (uint64_t u = lo; u < hi; ++u) {
    const uint64_t f = u / N;
    const unsigned bin = (unsigned)(u % N);
    for (unsigned a = 0; a < C; ++a) xv[a] = unpack(x->spec[(f * N + bin) * C + a]);
    for (unsigned b = 0; b < B; ++b) {
      unsigned fr, fi;
      const cpx y = bf_dot(xv, ch->weights + (size_t)b * C, C, NULL, NULL, &fr, &fi);
      if (fr | fi) { fl |= fr | fi; ++ns; }
      x->beams[(f * B + b) * N + bin] = pack(y);
      x->cells[(f * B + b) * N + bin] = (uint64_t)power(y); /* >= 0: clamp_cell is identity */
    }
  }
  x->flags_t[tid * 16 + 1] |= fl;
  x->cnt_t[tid * 4 + 1] += ns;
}

/* Phase E: covariance integrators per bin, sequential over frames. */
static void ph_cov(void* p, uint64_t lo, uint64_t hi, int tid) {
  chain_ctx* x = p;
  orc_chain* ch = x->ch;
  const rd_config* c = &ch->cfg;
  const unsigned N = c->n_fft, C = c->n_chan, B = c->n_beams, P = ch->n_pairs;
  cpx src[128];
  (void)tid;
  for (uint64_t bin = lo; bin < hi; ++bin) {
    uint32_t w = 0;
    for (uint64_t f = 0; f < x->frames; ++f) {
      if (c->cov_source == RD_COV_CHANNEL) {
        for (unsigned a = 0; a < C; ++a) src[a] = unpack(x->spec[(f * N + bin) * C + a]);
      } else {
        for (unsigned b = 0; b < B; ++b) src[b] = unpack(x->beams[(f * B + b) * N + bin]);
      }
      int emitted = 0;
      for (unsigned q = 0; q < P; ++q) {
        wide re, im;
        cross_power(src[ch->px[q]], src[ch->py[q]], &re, &im);
        integ* sr = &ch->cov_re[bin * P + q];
        integ* si = &ch->cov_im[bin * P + q];
        integ_result rr = {0, 0, 0, 0, 0}, ri = {0, 0, 0, 0, 0};
        const int er = integ_step(sr, c->cov_acc_w, c->cov_window, c->cov_mode == RD_COV_EXP,
                                  c->cov_exp_k, 1, re, 0, &rr);
        const int ei = integ_step(si, c->cov_acc_w, c->cov_window, c->cov_mode == RD_COV_EXP,
                                  c->cov_exp_k, 1, im, 0, &ri);
        (void)ei;
        if (er) {
          emitted = 1;
          if (w < x->max_w) {
            int64_t* acc = x->cov_acc + (((size_t)w * N + bin) * P + q) * 2;
            acc[0] = rr.acc;
            acc[1] = ri.acc;
            __atomic_fetch_or(&x->cov_wflags[w], sr->sticky | si->sticky, __ATOMIC_RELAXED);
            if (bin == 0 && q == 0) {
              x->cov_hdr[w] = rr;
              x->cov_wclose[w] = (uint32_t)f;
            }
          }
        }
      }
      if (emitted) ++w;
    }
    if (bin == 0) x->n_windows = w;
  }
}

/* Phase F: CFAR per (frame, beam). */
static void ph_cfar(void* p, uint64_t lo, uint64_t hi, int tid) {
  chain_ctx* x = p;
  orc_chain* ch = x->ch;
  const unsigned N = ch->cfg.n_fft, B = ch->cfg.n_beams;
  cfar_cfg k = cfar_clamp(&ch->cfg);
  uint64_t* pre = malloc(sizeof(uint64_t) * (N + 1));
  rd_event* tmp = malloc(sizeof(rd_event) * (N + 1));
  (void)tid;
  for (uint64_t u = lo; u < hi; ++u) {
    const uint64_t f = u / B;
    const unsigned b = (unsigned)(u % B);
    const uint64_t gf = ch->frame + f;
    unsigned d, s;
    const uint64_t m = cfar_frame(x->cells + (f * B + b) * N, N, &k, (unsigned)(gf & 0xFFFFu),
                                  (uint32_t)gf, (uint16_t)b, pre, tmp, N + 1, &d, &s);
    x->ev[u] = malloc(sizeof(rd_event) * m);
    memcpy(x->ev[u], tmp, sizeof(rd_event) * m);
    x->nev[u] = m;
    x->det[u] = d;
    x->sup[u] = s;
  }
  free(pre);
  free(tmp);
}

int orc_chain_process(orc_chain* ch, const rd_cplx16* adc, uint64_t n, uint64_t ld,
                      rd_output* out, int threads) {
  const rd_config* c = &ch->cfg;
  const unsigned N = c->n_fft, C = c->n_chan, B = c->n_beams, M = N / c->spc;
  if (n % N != 0) return RD_EINVAL;
  if (threads < 1) threads = 1;
  const uint64_t F = n / N;
  chain_ctx x;
  memset(&x, 0, sizeof(x));
  x.ch = ch;
  x.adc = adc;
  x.ld = ld;
  x.frames = F;
  x.threads = threads;
  x.pfb = malloc(sizeof(uint32_t) * F * C * N + 4);
  x.spec = malloc(sizeof(uint32_t) * F * C * N + 4);
  x.beams = malloc(sizeof(uint32_t) * F * B * N + 4);
  x.cells = malloc(sizeof(uint64_t) * F * B * N + 8);
  x.flags_t = calloc((size_t)threads * 16, sizeof(unsigned));
  x.cnt_t = calloc((size_t)threads * 4, sizeof(uint64_t));
  x.ev = calloc(F * B + 1, sizeof(rd_event*));
  x.nev = calloc(F * B + 1, sizeof(uint64_t));
  x.det = calloc(F * B + 1, sizeof(unsigned));
  x.sup = calloc(F * B + 1, sizeof(unsigned));

  parallel_for((uint64_t)C * N, threads, ph_pfb, &x);
  parallel_for(F * C, threads, ph_fft, &x);

  /* Phase C: history writes and the align reads (bookkeeping + storage).
   * The chain's reads are frame_off 0 after each frame: they return the
   * frame just written, so the beamformer reads the spectra directly. */
  for (uint64_t f = 0; f < F; ++f) {
    for (unsigned a = 0; a < C; ++a)
      for (unsigned j = 0; j < M; ++j) {
        uint32_t lanes[2];
        for (unsigned q = 0; q < c->spc; ++q) lanes[q] = x.spec[(f * N + q * M + j) * C + a];
        hist_write_beat(&ch->hist, a, lanes, j == 0, j == M - 1);
      }
    unsigned hflags_any = 0;
    for (unsigned bin = 0; bin < N; ++bin) {
      uint32_t fid;
      unsigned fl;
      hist_read(&ch->hist, bin, 0, NULL, &fid, &fl);
      hflags_any |= fl;
      /* the frame just written: the model's ids count from the depth epoch */
      if (fid != ch->hist.frames_done - 1u) { hflags_any |= 0x100; }
    }
    /* align: N/2 beats of bin pairs, all lanes present (align_model.hpp:321-359) */
    sat_bump(&ch->st.align_beats, N / 2);
    ch->align_seq = (ch->align_seq + N / 2) & 0xFFFFu;
    if (hflags_any & 0xFF) ch->st.align_fault |= 8u; /* kUserHist */
    if (hflags_any & 0x100) { /* the read did not return the frame just written */
      free(x.pfb); free(x.spec); free(x.beams); free(x.cells);
      return RD_EDEVICE;
    }
  }

  parallel_for(F * N, threads, ph_bf, &x);

  uint32_t max_w = 0;
  if (c->cov_source != RD_COV_OFF && ch->n_pairs) {
    const unsigned wl = c->cov_window ? c->cov_window : 1u;
    max_w = (uint32_t)(F / wl + 2);
    x.max_w = max_w;
    x.cov_acc = calloc((size_t)max_w * N * ch->n_pairs * 2, sizeof(int64_t));
    x.cov_wclose = calloc(max_w, sizeof(uint32_t));
    x.cov_hdr = calloc(max_w, sizeof(integ_result));
    x.cov_wflags = calloc(max_w, sizeof(unsigned));
    parallel_for(N, threads, ph_cov, &x);
  }

  if (ch->eng_pairs) { /* the beat-stream engine, beat by beat in the beamformer's order */
    const unsigned Pe = ch->eng_pairs;
    for (uint64_t f = 0; f < F; ++f)
      for (unsigned g = 0; g < N / 2u; ++g) {
        const unsigned bin = 2u * g;
        for (unsigned p = 0; p < Pe; ++p) {
          const cpx a = unpack(x.beams[(f * B + (2u * p) % B) * N + bin]);
          const cpx b = unpack(x.beams[(f * B + (2u * p + 1u) % B) * N + bin]);
          wide re, im;
          cross_power(a, b, &re, &im);
          integ_result rr = {0, 0, 0, 0, 0}, ri = {0, 0, 0, 0, 0};
          const int er = integ_step(&ch->eng_re[p], 40, N, 0, 0, 1, re, 0, &rr);
          integ_step(&ch->eng_im[p], 40, N, 0, 0, 1, im, 0, &ri);
          if (p == 0 && er) {
            ch->st.engine_window = rr.window_id;
            ch->st.engine_samples = rr.sample_count;
          }
        }
      }
    unsigned sat = 0;
    for (unsigned p = 0; p < Pe; ++p) sat |= ch->eng_re[p].sticky | ch->eng_im[p].sticky;
    ch->st.engine_sat = sat != 0;
  }

  parallel_for(F * B, threads, ph_cfar, &x);

  /* outputs */
  int trunc = 0;
  const unsigned words = rd_flit_words(c->packet_w), nfl = rd_detection_flits(c->packet_w);
  out->n_events = 0;
  out->n_flits = 0;
  out->flit_words = words;
  out->n_frames = F;
  for (uint64_t u = 0; u < F * B; ++u) {
    for (uint64_t j = 0; j < x.nev[u]; ++j) {
      const rd_event* e = &x.ev[u][j];
      if (out->events) {
        if (out->n_events < out->cap_events) out->events[out->n_events] = *e;
        else trunc = 1;
      }
      if (out->flits) {
        if (out->n_flits + nfl <= out->cap_flits)
          packet_flits(e, c->packet_w, c->src_id, c->dest, c->vc, ch->st.next_seq,
                       out->flits + out->n_flits * words);
        else
          trunc = 1;
      }
      out->n_events++;
      out->n_flits += nfl;
      ch->st.packets++;
      ch->st.flits += nfl;
      ch->st.next_seq = (ch->st.next_seq + 1u) & 0xFFFFu;
    }
    ch->st.cfar_det += x.det[u];
    ch->st.cfar_sup += x.sup[u];
    ch->st.cfar_frames++;
    free(x.ev[u]);
  }
  out->n_cov_windows = 0;
  if (max_w) {
    const size_t per = (size_t)N * ch->n_pairs * 2;
    for (uint32_t w = 0; w < x.n_windows; ++w) {
      if (w < out->cap_cov_windows) {
        if (out->cov_windows) {
          rd_cov_window* h = &out->cov_windows[w];
          memset(h, 0, sizeof(*h));
          h->window_id = x.cov_hdr[w].window_id;
          h->sample_count = x.cov_hdr[w].sample_count;
          h->end_frame = (uint32_t)(ch->frame + x.cov_wclose[w]);
          h->flushed = (uint8_t)x.cov_hdr[w].flushed;
          h->truncated = (uint8_t)x.cov_hdr[w].truncated;
          h->sat_flags = (uint8_t)x.cov_wflags[w];
        }
        if (out->cov_acc) memcpy(out->cov_acc + w * per, x.cov_acc + w * per, per * sizeof(int64_t));
      } else {
        trunc = 1;
      }
    }
    out->n_cov_windows = x.n_windows;
    unsigned cf = 0;
    uint64_t cs = 0;
    for (size_t k = 0; k < (size_t)N * ch->n_pairs; ++k) {
      cf |= ch->cov_re[k].sticky | ch->cov_im[k].sticky;
      cs += ch->cov_re[k].sat_count + ch->cov_im[k].sat_count;
    }
    ch->st.cov_flags = cf;
    ch->st.cov_sat_steps = cs;
  }
  /* taps */
  if (out->tap_pfb) memcpy(out->tap_pfb, x.pfb, sizeof(uint32_t) * F * C * N);
  if (out->tap_spectrum) memcpy(out->tap_spectrum, x.spec, sizeof(uint32_t) * F * C * N);
  if (out->tap_beams) memcpy(out->tap_beams, x.beams, sizeof(uint32_t) * F * B * N);
  if (out->tap_power)
    for (uint64_t i = 0; i < F * B * N; ++i) out->tap_power[i] = (uint32_t)x.cells[i];
  for (int t = 0; t < threads; ++t) {
    ch->st.pfb_flags |= x.flags_t[t * 16 + 0];
    ch->st.bf_flags |= x.flags_t[t * 16 + 1];
    for (unsigned s = 0; s < 11; ++s) ch->st.fft_stage_flags[s] |= x.flags_t[t * 16 + 2 + s];
    ch->st.pfb_sat_samples += x.cnt_t[t * 4 + 0];
    ch->st.bf_sat_samples += x.cnt_t[t * 4 + 1];
  }
  ch->frame += F;
  ch->st.frames += F;
  ch->st.hist_frames_done = ch->hist.frames_done;
  ch->st.hist_write_beats = ch->hist.c_wbeat;
  ch->st.hist_reads = ch->hist.c_read;
  ch->st.hist_collisions = ch->hist.c_collision;
  ch->st.hist_errors = ch->hist.c_error;
  ch->st.hist_overwrites = ch->hist.c_overwrite;
  ch->st.hist_skew = ch->hist.c_skew;
  free(x.pfb); free(x.spec); free(x.beams); free(x.cells);
  free(x.flags_t); free(x.cnt_t); free(x.ev); free(x.nev); free(x.det); free(x.sup);
  free(x.cov_acc); free(x.cov_wclose); free(x.cov_hdr); free(x.cov_wflags);
  return trunc ? RD_ETRUNC : RD_OK;
}

int orc_chain_flush_cov(orc_chain* ch, rd_output* out) {
  const unsigned N = ch->cfg.n_fft, P = ch->n_pairs;
  out->n_cov_windows = 0;
  if (!ch->cov_re) return RD_OK;
  int opened = 0;
  for (unsigned bin = 0; bin < N; ++bin)
    for (unsigned q = 0; q < P; ++q) {
      integ_result rr = {0, 0, 0, 0, 0}, ri = {0, 0, 0, 0, 0};
      const rd_config* c = &ch->cfg;
      const int er = integ_step(&ch->cov_re[bin * P + q], c->cov_acc_w, c->cov_window,
                                c->cov_mode == RD_COV_EXP, c->cov_exp_k, 0, 0, 1, &rr);
      integ_step(&ch->cov_im[bin * P + q], c->cov_acc_w, c->cov_window,
                 c->cov_mode == RD_COV_EXP, c->cov_exp_k, 0, 0, 1, &ri);
      if (!er) continue;
      if (!opened) {
        if (out->cap_cov_windows < 1) return RD_ETRUNC;
        rd_cov_window* h = &out->cov_windows[0];
        memset(h, 0, sizeof(*h));
        h->window_id = rr.window_id;
        h->sample_count = rr.sample_count;
        h->end_frame = (uint32_t)ch->frame;
        h->flushed = (uint8_t)rr.flushed;
        h->truncated = (uint8_t)rr.truncated;
        out->n_cov_windows = 1;
        opened = 1;
      }
      if (out->cov_acc) {
        out->cov_acc[((size_t)bin * P + q) * 2] = rr.acc;
        out->cov_acc[((size_t)bin * P + q) * 2 + 1] = ri.acc;
      }
    }
  return RD_OK;
}

int orc_chain_stats(const orc_chain* ch, rd_stats* st) {
  *st = ch->st;
  return RD_OK;
}

int orc_chain_read_history(orc_chain* ch, uint32_t bin, uint32_t frame_off, rd_cplx16* vec,
                           uint32_t* frame_id, uint32_t* flags) {
  unsigned fl;
  hist_read(&ch->hist, bin, frame_off, vec, frame_id, &fl);
  *flags = fl;
  ch->st.hist_reads = ch->hist.c_read;
  ch->st.hist_errors = ch->hist.c_error;
  ch->st.hist_collisions = ch->hist.c_collision;
  return RD_OK;
}

const char* orc_name(void) { return "orc_port (plain-C restatement)"; }
