// k_engine.cu - the RTL's telemetry-only beat-stream covariance engine.
//
// covar::Engine (covar_model.hpp:318-416) as benchmark_sim_top.sv:1124-1200
// wires it: one source vector per beamformer beat - the beams of the beat's
// bin_par 0, i.e. the even bin 2g of beat g, beats in bin order frame after
// frame - pairs (2p, 2p+1) mod B, and per pair two 40-bit block integrators
// (covar_model.hpp:204-262) closing every n_fft beats, never flushed. The
// multiplier pipeline only delays when a product lands; between calls the
// clock runs on, so at a call's end every beat has landed.
//
// Windows are independent in block mode (the accumulator restarts at each
// close), so a launch splits its beats into window segments: the first one
// continues the window the previous launch left open (its accumulator comes
// in), the last may stay open (its accumulator goes out). A warp takes one
// (segment, pair): its lanes form the cross powers (re = xr yr + xi yi,
// im = xi yr - xr yi, exact in int64) and sum them with their magnitudes. When
// the carried accumulator plus the magnitudes stays inside the 40-bit range
// no partial sum can leave it, so the window's value is the plain sum and no
// saturation happens; otherwise lane 0 reruns the segment step by step with
// the integrator's saturation and sticky flag. Only the sticky flag (any
// pair) is telemetry on the device; the closed windows' ids and counts
// follow from the beat count on the host.
#include <cuda_runtime.h>

#include "rd_internal.h"

namespace rd {

namespace {

constexpr long long kAccMax = (1ll << 39) - 1;  // 40-bit signed range
constexpr long long kAccMin = -(1ll << 39);

__device__ __forceinline__ void cross(uint32_t xw, uint32_t yw, long long& re, long long& im) {
  const long long xr = (int16_t)(xw & 0xFFFFu), xi = (int16_t)(xw >> 16);
  const long long yr = (int16_t)(yw & 0xFFFFu), yi = (int16_t)(yw >> 16);
  re = xr * yr + xi * yi;
  im = xi * yr - xr * yi;
}

// one accepted integrator step in block mode (add, saturate to 40 bits,
// flag); returns whether the step saturated
__device__ __forceinline__ bool sat_step(long long& acc, long long d) {
  const long long raw = acc + d;  // |acc| <= 2^39, |d| <= 2^31: no 64-bit wrap
  acc = raw > kAccMax ? kAccMax : (raw < kAccMin ? kAccMin : raw);
  return raw != acc;
}

__global__ void __launch_bounds__(256) k_engine(EngineParams p) {
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
  if (warp >= p.n_seg * p.pairs) return;  // warp-uniform
  const unsigned seg = warp / p.pairs, pr = warp % p.pairs;
  const unsigned N = p.N, B = p.B, half = N / 2u;
  // the segment's beats [t0, t1) of this launch
  const uint64_t start = (uint64_t)seg * N;  // in window-aligned beats from the open window's start
  const uint64_t t0 = start > p.count0 ? start - p.count0 : 0u;
  const uint64_t end = start + N - p.count0;
  const uint64_t t1 = end < p.beats ? end : p.beats;
  const unsigned xb = (2u * pr) % B, yb = (2u * pr + 1u) % B;
  const long long acc0 = seg == 0u ? p.acc_in[2u * pr] : 0ll;
  const long long aci0 = seg == 0u ? p.acc_in[2u * pr + 1u] : 0ll;
  long long sr = 0, si = 0, mr = 0, mi = 0;
  for (uint64_t t = t0 + lane; t < t1; t += 32u) {
    const uint64_t f = t / half;
    const unsigned bin = 2u * (unsigned)(t - f * half);
    const uint32_t* row = p.beams + ((size_t)f * N + bin) * B;
    long long re, im;
    cross(row[xb], row[yb], re, im);
    sr += re;
    si += im;
    mr += re < 0 ? -re : re;
    mi += im < 0 ? -im : im;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
    mr += __shfl_xor_sync(0xffffffffu, mr, o);
    mi += __shfl_xor_sync(0xffffffffu, mi, o);
  }
  if (lane != 0u) return;
  long long ar = acc0 + sr, ai = aci0 + si;
  bool sat = false;
  const long long br = (acc0 < 0 ? -acc0 : acc0) + mr, bi = (aci0 < 0 ? -aci0 : aci0) + mi;
  if (br > kAccMax || bi > kAccMax) {  // some partial sum may leave the range: step by step
    ar = acc0;
    ai = aci0;
    for (uint64_t t = t0; t < t1; ++t) {
      const uint64_t f = t / half;
      const unsigned bin = 2u * (unsigned)(t - f * half);
      const uint32_t* row = p.beams + ((size_t)f * N + bin) * B;
      long long re, im;
      cross(row[xb], row[yb], re, im);
      sat |= sat_step(ar, re);
      sat |= sat_step(ai, im);
    }
  }
  if (sat) atomicOr(&p.stats->eng_sat, 1u);
  if (t1 == p.beats) {  // the launch's last segment: the window it leaves open
    const bool closed = (p.count0 + p.beats) % N == 0u;
    p.acc_out[2u * pr] = closed ? 0ll : ar;
    p.acc_out[2u * pr + 1u] = closed ? 0ll : ai;
  }
}

}  // namespace

void launch_engine(const EngineParams& p, cudaStream_t s) {
  if (!p.pairs || !p.beats) return;
  const uint64_t warps = (uint64_t)p.n_seg * p.pairs;
  k_engine<<<(unsigned)((warps * 32u + 255u) / 256u), 256, 0, s>>>(p);
}

}  // namespace rd
