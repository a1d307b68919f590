// k_pfb_rows.cu - the polyphase filter bank as its own pass, frame-blocked.
//
// y[f][p] = round_sat(sum_k h[k][p] x[f - k][p], 15, 16) per channel
// (pfb_model.hpp:139-177): the same products and the same rounding as the
// fused front kernel, but organised for the load path. There a thread
// computed one (frame, channel) item's 4 phases and loaded, per tap, the
// sample and the coefficient: every sample was read by T items and every
// coefficient by every item, and those loads took most of the kernel's
// L1 bandwidth. Here a thread owns one phase of one channel over RF
// consecutive output frames (threads run over channel x phase, phase fastest): its T coefficients stay in registers, and each
// input sample is loaded once and used by every output frame it reaches.
//
// The sums are int32 multiply-adds (the bank's L1 norms keep every partial
// sum inside int32: pfb32), with the imaginary parts left out when the bank is
// real (every hi = 0, the reference's default prototype). Outputs are
// rounded and saturated exactly, with the model's flags and saturation
// count, and written as [F][C][N] for the FFT pass. The chunk's last T - 1
// frames are copied into the next delay line on the way.
#include <cuda_runtime.h>

#include "fxp.cuh"
#include "rd_internal.h"

namespace rd {

namespace {

constexpr unsigned kPfbThreads = 128u;
constexpr int kRF = 16;  // output frames per thread

template <int TT, bool REAL>
__global__ void __launch_bounds__(kPfbThreads, 4) k_pfb_rows(FrontParams p, uint32_t* out) {
  constexpr int NI = kRF + TT - 1;  // input frames of the block
  // threads over (channel, phase), the phase fastest: a 16- or 64-point
  // bank fills the CTA with several channels
  const unsigned N = p.N;
  const unsigned t = blockIdx.x * kPfbThreads + threadIdx.x;
  const unsigned c = t / N, ph = t - c * N;
  const int f0 = (int)(blockIdx.z * kRF);
  const int F = (int)p.F;
  const bool live = c < p.C;
  int hr[TT], hi[TT];
#pragma unroll
  for (int k = 0; k < TT; ++k) {
    const int2 h = live ? __ldg(p.coeff2 + (size_t)k * N + ph) : make_int2(0, 0);
    hr[k] = h.x;
    hi[k] = h.y;
  }
  // the block's input frames f0 - (TT - 1) .. f0 + kRF - 1, unpacked; the
  // chunk's last TT - 1 frames are copied into the next call's delay line
  // (pfb_model.hpp:170-175) by the block whose outputs they are
  int xr[NI], xi[NI];
  const uint32_t* xa = p.adc + (size_t)c * p.ld + ph;
  uint32_t* to = p.tail_out ? p.tail_out + (size_t)c * (TT - 1) * N + ph : nullptr;
  if (f0 >= TT - 1 && f0 + kRF <= F) {  // every input in the chunk (all blocks but the ends)
    const uint32_t* x0 = xa + (size_t)(f0 - (TT - 1)) * N;
#pragma unroll
    for (int d = 0; d < NI; ++d) {
      const uint32_t xw = live ? __ldg(x0 + (size_t)d * N) : 0u;
      xr[d] = (int)(int16_t)(uint16_t)(xw & 0xFFFFu);
      xi[d] = (int)xw >> 16;
    }
  } else {
    const uint32_t* xt = p.tail + (size_t)c * (TT - 1) * N + ph;
#pragma unroll
    for (int d = 0; d < NI; ++d) {
      const int fi = f0 - (TT - 1) + d;
      uint32_t xw = 0u;
      if (live && fi < F)
        xw = fi >= 0 ? __ldg(xa + (size_t)fi * N) : __ldg(xt + (size_t)(-fi - 1) * N);
      xr[d] = (int)(int16_t)(uint16_t)(xw & 0xFFFFu);
      xi[d] = (int)xw >> 16;
    }
  }
  if (to && live && f0 + kRF + TT - 1 > F) {  // the block holds some of the last TT - 1 frames
#pragma unroll
    for (int r = 0; r < kRF; ++r) {
      const int fi = f0 + r;
      if (fi < F && fi + TT > F) {
        const int d = r + TT - 1;
        to[(size_t)(F - 1 - fi) * N] = ((uint32_t)(uint16_t)xi[d] << 16) | (uint16_t)xr[d];
      }
    }
  }
  // output r takes input r - k + TT - 1 at tap k
  int ar[kRF], ai[kRF];
#pragma unroll
  for (int r = 0; r < kRF; ++r) ar[r] = ai[r] = 0;
#pragma unroll
  for (int k = 0; k < TT; ++k) {
#pragma unroll
    for (int r = 0; r < kRF; ++r) {
      const int d = r - k + TT - 1;
      if (REAL) {
        ar[r] += xr[d] * hr[k];
        ai[r] += xi[d] * hr[k];
      } else {
        ar[r] += xr[d] * hr[k] - xi[d] * hi[k];
        ai[r] += xr[d] * hi[k] + xi[d] * hr[k];
      }
    }
  }
  // round_sat(v, 15, 16) (q15_out32): rounded in 32 bits, saturated and
  // packed {im, re} by one cvt.pack.sat; the flags only when some output of
  // the warp saturated. A sum v saturates exactly when v + 0x40004000 leaves
  // [0, 2^31) (the rounded value passes 32767 from v = 0x3FFFC000 on and
  // -32768 below v = -0x40004000), so one add and the sign bit tell it.
  unsigned sacc = 0;
  const size_t ostep = (size_t)p.C * N;
  uint32_t* o = out + ((size_t)f0 * p.C + c) * N + ph;
  const int nout = live ? min(kRF, F - f0) : 0;  // outputs of the thread in the chunk
#pragma unroll
  for (int r = 0; r < kRF; ++r, o += ostep) {
    const int yr = (ar[r] + 0x3FFF + ((ar[r] >> 15) & 1)) >> 15;
    const int yi = (ai[r] + 0x3FFF + ((ai[r] >> 15) & 1)) >> 15;
    uint32_t w;
    asm("cvt.pack.sat.s16.s32 %0, %1, %2;" : "=r"(w) : "r"(yi), "r"(yr));
    if (r < nout) {
      *o = w;
      sacc |= ((unsigned)ar[r] + 0x40004000u) | ((unsigned)ai[r] + 0x40004000u);
    }
  }
  if (__any_sync(0xffffffffu, (sacc >> 31) != 0u)) {
    unsigned fl = 0, nsat = 0;
#pragma unroll
    for (int r = 0; r < kRF; ++r) {
      if (!live || f0 + r >= F) continue;
      unsigned fr = 0, fi = 0;
      q15_out32(ar[r], &fr);
      q15_out32(ai[r], &fi);
      if (fr | fi) {
        fl |= fr | fi;
        ++nsat;
      }
    }
    const unsigned a = __reduce_or_sync(0xffffffffu, fl);
    const unsigned ns = __reduce_add_sync(0xffffffffu, nsat);
    if ((threadIdx.x & 31u) == 0u && p.stats) {
      if (a) atomicOr(&p.stats->pfb_flags, a);
      if (ns) atomicAdd(&p.stats->pfb_sat, (unsigned long long)ns);
    }
  }
}

template <int TT>
void launch_t(const FrontParams& p, uint32_t* out, cudaStream_t s) {
  const dim3 grid((unsigned)(((uint64_t)p.C * p.N + kPfbThreads - 1u) / kPfbThreads), 1u,
                  (p.F + kRF - 1u) / kRF);
  if (p.coeff_real)
    k_pfb_rows<TT, true><<<grid, kPfbThreads, 0, s>>>(p, out);
  else
    k_pfb_rows<TT, false><<<grid, kPfbThreads, 0, s>>>(p, out);
}

}  // namespace

bool pfb_rows_ok(const FrontParams& p) {
  return p.pfb32 && (p.T == 4u || p.T == 8u || p.T == 16u) && p.F > 0u;
}

void launch_pfb_rows(const FrontParams& p, uint32_t* out, cudaStream_t s) {
  switch (p.T) {
    case 4: launch_t<4>(p, out, s); break;
    case 8: launch_t<8>(p, out, s); break;
    default: launch_t<16>(p, out, s); break;
  }
}

}  // namespace rd
