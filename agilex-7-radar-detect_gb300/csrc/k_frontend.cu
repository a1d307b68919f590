// k_frontend.cu - polyphase FIR bank + streaming radix-2^2 FFT + corner turn.
//
// One CTA owns a block of (frame, channel) items. For each item, thread e
// holds one FFT element: it first computes the PFB output of phase
// p(e) (pfb_model.hpp:139-177: exact int64 accumulation of T products, one
// round_sat), which is exactly the lane-q, index-i input of the
// decimation-in-time FFT (fft_ref.hpp:261-266, lane q = p mod spc). It then
// runs every BF2I/BF2II sub-stage of its lane (fft_ref.hpp:334-365) and the
// group twiddles (:368-377), exchanging partners through warp shuffles when
// the butterfly span is below 32 and through shared memory above, then the
// radix-2 DIT merge (:380-406). The natural-order spectrum of the item lands
// in a shared-memory tile [frame][bin][channel] that is written to the
// history ring coalesced - the corner turn of history_model.hpp:147-159
// (bin-major, antenna-minor) without a second pass over HBM.
#include <cuda_runtime.h>

#include "fxp.cuh"
#include "rd_internal.h"

namespace rd {

__device__ const uint32_t g_tw[1024] = {
#include "twiddle_q15.inc"
};
static const uint32_t h_tw[1024] = {
#include "twiddle_q15.inc"
};

const uint32_t* twiddles_device() {
  const uint32_t* p = nullptr;
  cudaGetSymbolAddress((void**)&p, g_tw);
  return p;
}

static unsigned host_bitrev(unsigned v, unsigned w) {
  unsigned r = 0;
  for (unsigned i = 0; i < w; ++i)
    if ((v >> i) & 1u) r |= 1u << (w - 1 - i);
  return r;
}

uint32_t front_safe_input(uint32_t n, uint32_t spc, uint32_t sched) {
  // |wr| + |wi| over the table bounds what a twiddle product can grow
  uint64_t sw = 0;
  for (int i = 0; i < 1024; ++i) {
    const int wr = (int16_t)(uint16_t)(h_tw[i] & 0xFFFFu), wi = (int16_t)(uint16_t)(h_tw[i] >> 16);
    const uint64_t s = (uint64_t)(wr < 0 ? -wr : wr) + (uint64_t)(wi < 0 ? -wi : wi);
    if (s > sw) sw = s;
  }
  unsigned nl = 0;
  while ((1u << nl) < n / spc) ++nl;
  // the per-component bound after every sub-stage of the kernel's sequence:
  // a butterfly output is RNE((a +- t) / 2^sh), at most M when it scales and
  // 2M when it does not; a twiddle product rounded at 2^15 grows M by at most
  // sw / 2^15 (plus one for the rounding)
  auto fits = [&](uint64_t m) {
    auto bf = [&](unsigned stage) {
      m = ((sched >> stage) & 1u) ? m : 2 * m;
      return m <= 32767u;
    };
    auto tw = [&]() {
      m = (m * sw + 16384u) / 32768u + 1u;
      return m <= 32767u;
    };
    for (unsigned st = 0; st < nl; st += 2) {
      if (st + 1 < nl) {
        if (!bf(st) || !bf(st + 1)) return false;
        if (st + 2 < nl && !tw()) return false;
      } else if (!bf(st)) {
        return false;
      }
    }
    if (spc == 2) {  // merge: twiddle on the odd lane, then a butterfly
      const uint64_t e = m;
      if (!tw()) return false;
      m = m > e ? m : e;
      if (!bf(nl)) return false;
    }
    return true;
  };
  uint32_t lo = 0, hi = 32767;  // largest fitting input bound
  if (!fits(0)) return 0;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1u) / 2u;
    if (fits(mid)) lo = mid;
    else hi = mid - 1u;
  }
  return lo;
}

void twiddle_positions(uint32_t n, uint32_t spc, uint32_t* out, uint32_t* words) {
  const unsigned m = n / spc, nl = ilog2(m);
  const unsigned n_tw = (nl - 1u) / 2u;
  for (unsigned k = 0; k < n_tw; ++k) {
    const unsigned s = 2u * k + 1u, l2l = nl - s + 1u;
    for (unsigned i = 0; i < m; ++i) out[k * m + i] = h_tw[r22_tw_exp(l2l, i) << (10u - l2l)];
  }
  unsigned total = n_tw * m;
  if (spc == 2) {
    for (unsigned i = 0; i < m; ++i) out[total + i] = h_tw[host_bitrev(i, nl) << (10u - nl - 1u)];
    total += m;
  }
  *words = total;
}

// Exchange with element e ^ h of the same item (h uniform over the block).
__device__ __forceinline__ uint32_t xchg(uint32_t val, unsigned h, uint32_t* xs) {
  if (h < 32) return __shfl_xor_sync(0xffffffffu, val, h);
  xs[threadIdx.x] = val;
  __syncthreads();
  const uint32_t r = xs[threadIdx.x ^ h];
  __syncthreads();
  return r;
}

// One FFT element. e = q*m + i is the thread's (lane, position) in the item;
// returns its value after the last sub-stage. twp holds the per-position
// twiddles (twiddle_positions). Stage flags of sub-stage g accumulate into
// *sf bits [2g+1:2g].
__device__ __forceinline__ uint32_t fft_elem(uint32_t v, unsigned e, unsigned nl,
                                             unsigned spc, unsigned sched,
                                             const uint32_t* twp, uint32_t* xs,
                                             unsigned* sf) {
  const unsigned m = 1u << nl;
  const unsigned q = e >> nl, i = e & (m - 1u);
  for (unsigned s = 0; s < nl; ++s) {
    const unsigned half = 1u << (nl - 1u - s);
    const unsigned sh = (sched >> s) & 1u;
    const bool hi = (i & half) != 0u;
    const bool k1 = (s & 1u) && ((i >> (nl - s)) & 1u);
    unsigned fl = 0;
    const cplx cur = unpack(v);
    const cplx mine = (hi && k1) ? neg_j(cur, &fl) : cur;
    const cplx o = unpack(xchg(pack(mine), half, xs));
    cplx r;
    if (!hi) {
      r.re = (int16_t)quant1((int32_t)mine.re + o.re, sh, &fl);
      r.im = (int16_t)quant1((int32_t)mine.im + o.im, sh, &fl);
    } else {
      r.re = (int16_t)quant1((int32_t)o.re - mine.re, sh, &fl);
      r.im = (int16_t)quant1((int32_t)o.im - mine.im, sh, &fl);
    }
    if ((s & 1u) && s + 1u < nl) r = cmul_tw(r, unpack(twp[(s >> 1) * m + i]), &fl);
    *sf |= fl << (2u * s);
    v = pack(r);
  }
  if (spc == 2) {
    const unsigned sh = (sched >> nl) & 1u;
    unsigned fl = 0;
    const cplx cur = unpack(v);
    cplx mine = cur;
    if (q == 1u) mine = cmul_tw(cur, unpack(twp[((nl - 1u) / 2u) * m + i]), &fl);
    const cplx o = unpack(xchg(pack(mine), m, xs));
    cplx r;
    if (q == 0u) {
      r.re = (int16_t)quant1((int32_t)mine.re + o.re, sh, &fl);
      r.im = (int16_t)quant1((int32_t)mine.im + o.im, sh, &fl);
    } else {
      r.re = (int16_t)quant1((int32_t)o.re - mine.re, sh, &fl);
      r.im = (int16_t)quant1((int32_t)o.im - mine.im, sh, &fl);
    }
    *sf |= fl << (2u * nl);
    v = pack(r);
  }
  return v;
}

// natural bin of the element e after fft_elem (fft_ref.hpp:291-296)
__device__ __forceinline__ unsigned fft_bin(unsigned e, unsigned nl) {
  const unsigned m = 1u << nl;
  return bitrev(e & (m - 1u), nl) + (e >> nl) * m;
}

__device__ __forceinline__ void reduce_stats(DevStats* st, unsigned pfl, unsigned long long psat,
                                             unsigned sf) {
  const unsigned a = __reduce_or_sync(0xffffffffu, pfl);
  const unsigned b = __reduce_or_sync(0xffffffffu, sf);
  unsigned long long c = psat;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31u) == 0u) {
    if (a) atomicOr(&st->pfb_flags, a);
    if (b) atomicOr(&st->fft_flags, b);
    if (c) atomicAdd(&st->pfb_sat, c);
  }
}

// PFB input x[f-k] of phase `ph` of channel c (delay line for f-k < 0)
__device__ __forceinline__ uint32_t pfb_in(const FrontParams& p, unsigned T, unsigned c,
                                           long long fr, unsigned ph) {
  return fr >= 0 ? __ldg(p.adc + (size_t)c * p.ld + (size_t)fr * p.N + ph)
                 : __ldg(p.tail + ((size_t)c * (T - 1u) + (size_t)(-fr - 1)) * p.N + ph);
}

template <int TT, int MAXT>
__global__ void __launch_bounds__(MAXT) k_front(FrontParams p, unsigned FB, unsigned CB,
                                               unsigned twn) {
  extern __shared__ uint32_t sm[];
  const unsigned tid = threadIdx.x, nth = blockDim.x;
  uint32_t* s_tw = sm;
  uint32_t* s_x = sm + twn;
  uint32_t* s_tile = s_x + nth;
  const unsigned cbp = CB + 1u;  // padded row: bit-reversed bins hit distinct banks
  for (unsigned k = tid; k < twn; k += nth) s_tw[k] = p.tw_pos[k];

  const unsigned N = p.N, spc = p.spc;
  const unsigned T = TT ? (unsigned)TT : p.T;
  const unsigned m = N / spc, nl = ilog2(m);
  const unsigned ipp = nth / N;
  const unsigned item = tid / N, e = tid % N;
  const unsigned ph = spc == 2u ? 2u * (e & (m - 1u)) + (e >> nl) : e;
  constexpr int TR = TT ? TT : 1;
  uint32_t h[TR];
  uint32_t xn[TR];  // inputs of the next item (prefetched)
  if (TT) {
#pragma unroll
    for (int k = 0; k < TR; ++k) h[k] = p.coeff_t[(size_t)k * N + ph];
  }
  const unsigned f0 = blockIdx.x * FB;
  const unsigned c0 = blockIdx.y * CB;
  const unsigned n_items = FB * CB;
  unsigned pfl = 0, sf = 0;
  unsigned long long psat = 0;

  auto item_ok = [&](unsigned it, unsigned& f, unsigned& c) {
    f = f0 + it / CB;
    c = c0 + it % CB;
    return it < n_items && f < p.F && c < p.C;
  };
  if (TT) {
    unsigned f, c;
    if (item_ok(item, f, c)) {
#pragma unroll
      for (int k = 0; k < TR; ++k) xn[k] = pfb_in(p, T, c, (long long)f - k, ph);
    }
  }
  __syncthreads();

  for (unsigned base = 0; base < n_items; base += ipp) {
    const unsigned it = base + item;
    unsigned f, c;
    const bool ok = item_ok(it, f, c);
    uint32_t v = 0;
    if (ok) {
      long long are = 0, aim = 0;
      if (TT) {
        uint32_t xc[TR];
#pragma unroll
        for (int k = 0; k < TR; ++k) xc[k] = xn[k];
        unsigned f2, c2;  // issue the next item's loads before the math
        if (item_ok(it + ipp, f2, c2)) {
#pragma unroll
          for (int k = 0; k < TR; ++k) xn[k] = pfb_in(p, T, c2, (long long)f2 - k, ph);
        }
#pragma unroll
        for (int k = 0; k < TR; ++k) {
          const cplx x = unpack(xc[k]), hk = unpack(h[k]);
          are += (long long)((int32_t)x.re * hk.re - (int32_t)x.im * hk.im);
          aim += (long long)((int32_t)x.re * hk.im) + (long long)((int32_t)x.im * hk.re);
        }
      } else {
        for (unsigned k = 0; k < T; ++k) {
          const cplx x = unpack(pfb_in(p, T, c, (long long)f - k, ph));
          const cplx hk = unpack(__ldg(p.coeff_t + (size_t)k * N + ph));
          are += (long long)((int32_t)x.re * hk.re - (int32_t)x.im * hk.im);
          aim += (long long)((int32_t)x.re * hk.im) + (long long)((int32_t)x.im * hk.re);
        }
      }
      unsigned fr = 0, fi = 0;
      const int32_t yr = q15_out64(are, &fr);
      const int32_t yi = q15_out64(aim, &fi);
      if (fr | fi) {
        pfl |= fr | fi;
        ++psat;
      }
      v = pack2(yr, yi);
      if (p.tap_pfb) p.tap_pfb[((size_t)f * p.C + c) * N + ph] = v;
    }
    unsigned sfi = 0;
    const uint32_t r = fft_elem(v, e, nl, spc, p.sched, s_tw, s_x, &sfi);
    if (ok) {
      sf |= sfi;
      s_tile[((f - f0) * N + fft_bin(e, nl)) * cbp + (c - c0)] = r;
    }
  }
  __syncthreads();
  const unsigned tile_n = FB * N * CB;
  for (unsigned t = tid; t < tile_n; t += nth) {
    const unsigned fb = t / (N * CB), rem = t % (N * CB);
    const unsigned bin = rem / CB, cc = rem % CB;
    const unsigned f = f0 + fb, c = c0 + cc;
    if (f < p.F && c < p.C) {
      unsigned slot = p.ring_base + f;
      if (slot >= p.ring_frames) slot -= p.ring_frames;
      p.ring[((size_t)slot * N + bin) * p.C + c] = s_tile[(fb * N + bin) * cbp + cc];
    }
  }
  reduce_stats(p.stats, pfl, psat, sf);
}

static PerDevice g_front_attr;

unsigned launch_front(const FrontParams& p, cudaStream_t s) {
  // the PFB as its own pass, then the FFT kernel on its outputs
  if ((p.pfb_buf || p.tap_pfb) && pfb_rows_ok(p) && front_fast_ok(p.N, p.spc)) {
    uint32_t* out = p.tap_pfb ? p.tap_pfb : p.pfb_buf;
    launch_pfb_rows(p, out, s);  // it writes tail_out too
    FrontParams q = p;
    q.pfb_in = out;
    if (launch_front_fast(q, s)) return 2;
  }
  if (launch_front_fast(p, s)) return 1;  // it writes tail_out too
  const unsigned nth = p.N > 256u ? p.N : 256u;
  const unsigned ipp = nth / p.N;
  unsigned CB = 8192u / p.N;
  if (CB < 1u) CB = 1u;
  if (CB > p.C) CB = p.C;
  unsigned FB = ipp / CB;
  if (FB < 1u) FB = 1u;
  while (FB * CB * p.N > 8192u && FB > 1u) FB >>= 1;
  const unsigned m = p.N / p.spc, nl = ilog2(m);
  const unsigned twn = ((nl - 1u) / 2u) * m + (p.spc == 2u ? m : 0u);
  const dim3 grid((p.F + FB - 1) / FB, (p.C + CB - 1) / CB);
  const size_t smem = (twn + nth + (size_t)FB * p.N * (CB + 1u)) * sizeof(uint32_t);
  g_front_attr.once([] {
    const int lim = 96 * 1024;
    cudaFuncSetAttribute(k_front<0, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<4, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<8, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<16, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<0, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<4, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<8, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    cudaFuncSetAttribute(k_front<16, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
  });
  if (nth <= 256u) {
    switch (p.T) {
      case 4: k_front<4, 256><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      case 8: k_front<8, 256><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      case 16: k_front<16, 256><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      default: k_front<0, 256><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
    }
  } else {
    switch (p.T) {
      case 4: k_front<4, 1024><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      case 8: k_front<8, 1024><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      case 16: k_front<16, 1024><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
      default: k_front<0, 1024><<<grid, nth, smem, s>>>(p, FB, CB, twn); break;
    }
  }
  if (!p.tail_out || p.T <= 1) return 1;
  launch_tail_update(p.adc, p.ld, p.tail, p.tail_out, p.F, p.C, p.N, p.T, s);
  return 2;
}

// New delay line after a chunk of F frames: tail'[c][k] = frame F-1-k of the
// chunk when it exists, else tail[c][k-F] (pfb_model.hpp:170-175).
__global__ void k_tail(const uint32_t* adc, uint64_t ld, const uint32_t* old_tail,
                       uint32_t* new_tail, uint32_t F, uint32_t C, uint32_t N, uint32_t D) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t n = (uint64_t)C * D * N;
  if (i >= n) return;
  const uint32_t p = (uint32_t)(i % N);
  const uint32_t k = (uint32_t)((i / N) % D);
  const uint32_t c = (uint32_t)(i / ((uint64_t)N * D));
  new_tail[i] = (k < F) ? adc[(size_t)c * ld + (size_t)(F - 1 - k) * N + p]
                        : old_tail[((size_t)c * D + (k - F)) * N + p];
}

void launch_tail_update(const uint32_t* adc, uint64_t ld, const uint32_t* old_tail,
                        uint32_t* new_tail, uint32_t F, uint32_t C, uint32_t N, uint32_t T,
                        cudaStream_t s) {
  if (T <= 1) return;
  const uint32_t D = T - 1;
  const uint64_t n = (uint64_t)C * D * N;
  k_tail<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(adc, ld, old_tail, new_tail, F, C, N, D);
}

// ---- per-block entry points ---------------------------------------------

// pfb::PfbModel::step over `beats` beats, one thread per (beat, phase).
__global__ void k_pfb_block(uint32_t P, uint32_t T, const uint32_t* coeff, const uint32_t* state,
                            const uint32_t* in, uint32_t beats, uint32_t* out, uint8_t* flags) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)beats * P) return;
  const uint32_t t = (uint32_t)(i / P), ph = (uint32_t)(i % P);
  long long are = 0, aim = 0;
  for (uint32_t k = 0; k < T; ++k) {
    const uint32_t xw = k <= t ? in[(size_t)(t - k) * P + ph] : state[(size_t)(k - t - 1) * P + ph];
    const cplx x = unpack(xw), h = unpack(coeff[(size_t)ph * T + k]);
    are += (long long)((int32_t)x.re * h.re - (int32_t)x.im * h.im);
    aim += (long long)((int32_t)x.re * h.im) + (long long)((int32_t)x.im * h.re);
  }
  unsigned fr = 0, fi = 0;
  const int32_t yr = q15_out64(are, &fr), yi = q15_out64(aim, &fi);
  out[i] = pack2(yr, yi);
  if (flags) flags[i] = (uint8_t)((fr << 2) | fi);
}

void launch_pfb_block(uint32_t phases, uint32_t taps, const uint32_t* coeff,
                      const uint32_t* state, const uint32_t* in, uint32_t beats, uint32_t* out,
                      uint8_t* flags, cudaStream_t s) {
  const uint64_t n = (uint64_t)beats * phases;
  if (n) k_pfb_block<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(phases, taps, coeff, state, in,
                                                                  beats, out, flags);
}

// fft::transform on independent frames; one item of N threads per frame.
__global__ void k_fft_block(uint32_t N, uint32_t spc, uint32_t sched, int reorder,
                            const uint32_t* tw_pos, unsigned twn, const uint32_t* in,
                            uint32_t frames, uint32_t* out, uint32_t* bins,
                            uint8_t* stage_flags) {
  extern __shared__ uint32_t sm[];
  uint32_t* s_tw = sm;
  uint32_t* s_x = sm + twn;
  uint32_t* s_fl = s_x + blockDim.x;
  const unsigned tid = threadIdx.x, nth = blockDim.x;
  for (unsigned k = tid; k < twn; k += nth) s_tw[k] = tw_pos[k];
  const unsigned ipp = nth / N, item = tid / N, e = tid % N;
  if (tid < ipp) s_fl[tid] = 0;
  const unsigned m = N / spc, nl = ilog2(m);
  const unsigned q = e >> nl, i = e & (m - 1u);
  const unsigned ph = spc == 2u ? 2u * i + q : e;
  const unsigned stages = ilog2(N);
  __syncthreads();
  for (uint64_t f0 = (uint64_t)blockIdx.x * ipp; f0 < frames; f0 += (uint64_t)gridDim.x * ipp) {
    const uint64_t f = f0 + item;
    const bool ok = f < frames;
    const uint32_t v = ok ? in[f * N + ph] : 0u;
    unsigned sf = 0;
    const uint32_t r = fft_elem(v, e, nl, spc, sched, s_tw, s_x, &sf);
    if (ok) {
      const unsigned j = bitrev(i, nl);
      if (bins) bins[f * N + (spc == 2u ? j + q * m : j)] = r;
      if (out) {
        const unsigned o = reorder ? (spc == 2u ? 2u * j + q : j) : (spc == 2u ? 2u * i + q : i);
        out[f * N + o] = r;
      }
      if (sf) atomicOr(&s_fl[item], sf);
    }
    __syncthreads();
    if (ok && e < stages && stage_flags) stage_flags[f * stages + e] = (uint8_t)((s_fl[item] >> (2u * e)) & 3u);
    __syncthreads();
    if (e == 0u) s_fl[item] = 0;
    __syncthreads();
  }
}

void launch_fft_block(uint32_t n, uint32_t spc, uint32_t sched, int reorder,
                      const uint32_t* tw_pos, const uint32_t* in, uint32_t frames, uint32_t* out,
                      uint32_t* bins, uint8_t* stage_flags, cudaStream_t s) {
  const unsigned nth = n > 256u ? n : 256u;
  const unsigned ipp = nth / n;
  unsigned grid = (frames + ipp - 1) / ipp;
  if (grid > 4096u) grid = 4096u;
  if (grid == 0u) return;
  const unsigned m = n / spc, nl = ilog2(m);
  const unsigned twn = ((nl - 1u) / 2u) * m + (spc == 2u ? m : 0u);
  const size_t smem = (twn + nth + ipp) * sizeof(uint32_t);
  k_fft_block<<<grid, nth, smem, s>>>(n, spc, sched, reorder, tw_pos, twn, in, frames, out, bins,
                                      stage_flags);
}

// Slow-time vectors for the Doppler transform: out[(c * N + bin) * H + k] is
// channel c, bin `bin` of stream frame g_first + k, read from the ring.
__global__ void k_doppler_gather(const uint32_t* ring, uint32_t R, uint64_t g_first, uint32_t N,
                                 uint32_t C, uint32_t H, uint32_t* out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t total = (uint64_t)C * N * H;
  if (i >= total) return;
  const uint64_t v = i / H;
  const uint32_t k = (uint32_t)(i - v * H);
  const uint32_t c = (uint32_t)(v / N), bin = (uint32_t)(v - (uint64_t)c * N);
  const uint64_t slot = (g_first + k) % R;
  out[i] = ring[(slot * N + bin) * C + c];
}

void launch_doppler_gather(const uint32_t* ring, uint32_t R, uint64_t g_first, uint32_t N,
                           uint32_t C, uint32_t H, uint32_t* out, cudaStream_t s) {
  const uint64_t total = (uint64_t)C * N * H;
  if (total) k_doppler_gather<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(ring, R, g_first, N, C, H, out);
}

}  // namespace rd
