// k_backend.cu - beamforming, power, covariance integration, CA/GO-CFAR,
// event packing and packet flits.
#include <cuda_runtime.h>

#include <atomic>

#include "fxp.cuh"
#include "rd_internal.h"

namespace rd {

// ---------------------------------------------------------------------------
// Beamforming + power (CUDA-core integer form).
//
// Y[f][b][bin] = round_sat(sum_a X[f][bin][a] * W[b][a], 15, 16), the exact
// int64 dot product of bf::dot (beamformer_model.hpp:162-179), then
// power = re^2 + im^2 (covar_model.hpp:99-102), the CFAR cell. A CTA owns 64
// bins of one frame; the 256 threads split as 64 bins x 4 beam groups and each
// keeps BPT beams' accumulators in registers. The spectrum tile is staged in
// shared memory with a padded row so the 64 bin-threads of a warp pair read
// distinct banks; every weight read is a warp-wide broadcast.
// ---------------------------------------------------------------------------
// The weights arrive split into limbs, w = wh * 256 + wl with wh in
// [-128, 127] and wl in [0, 255] (set at rd_chain_set_weights), so every
// product term is exact in int32: |x * wh| <= 2^22, |x * wl| < 2^23, and a
// 64-channel block of complex terms stays below 2^31. Blocks are combined in
// int64 as acc = 256 * acc_h + acc_l - the same integer bf::dot sums.
// CC > 0 fixes the channel count at compile time (every shared-memory offset
// of the channel loop a constant); CC = 0 takes it from the parameters.
template <int BPT, int CC>
__global__ void __launch_bounds__(256) k_beam(BeamParams p) {
  extern __shared__ uint32_t sm[];
  const unsigned C = CC ? (unsigned)CC : p.C, B = p.B, N = p.N;
  const unsigned xs = C + 1;  // padded row
  int4* s_w = reinterpret_cast<int4*>(sm);          // [B][C] limbs
  int4* s_w3 = reinterpret_cast<int4*>(sm + 4u * B * C);  // [B][C] {re, im, re + im, 0}
  uint32_t* s_x = sm + 8u * B * C;
  const unsigned tid = threadIdx.x;
  const unsigned bin0 = blockIdx.x * 64u;
  const uint64_t f = blockIdx.y;
  unsigned slot = p.ring_base + (unsigned)f;
  if (slot >= p.ring_frames) slot -= p.ring_frames;
  for (unsigned k = tid; k < B * C; k += 256u) {
    const uint32_t w = p.weights[k];
    const int wr = (int)(int16_t)(uint16_t)(w & 0xFFFFu), wi = (int)w >> 16;
    s_w3[k] = make_int4(wr, wi, wr + wi, 0);
  }
  const uint32_t* xsrc = p.ring + ((size_t)slot * N + bin0) * C;
  const unsigned nb = (N - bin0) < 64u ? (N - bin0) : 64u;
  int xmax = 0;
  auto absmax = [&](uint32_t v) {
    xmax = max(xmax, max(abs((int)(int16_t)(uint16_t)(v & 0xFFFFu)), abs((int)v >> 16)));
  };
  if (p.cshift >= 0 && (C & 3u) == 0u) {
    // the tile's nb x C words are contiguous (16-byte aligned): quad loads,
    // row and column by shift
    const uint4* src4 = reinterpret_cast<const uint4*>(xsrc);
    const unsigned nq = nb * C / 4u, cm = C - 1u;
    for (unsigned q = tid; q < nq; q += 256u) {
      const uint4 v = src4[q];
      const unsigned k = 4u * q;
      uint32_t* d = s_x + (k >> p.cshift) * xs + (k & cm);
      d[0] = v.x;
      d[1] = v.y;
      d[2] = v.z;
      d[3] = v.w;
      absmax(v.x);
      absmax(v.y);
      absmax(v.z);
      absmax(v.w);
    }
  } else {
    for (unsigned k = tid; k < nb * C; k += 256u) {
      const uint32_t v = xsrc[k];
      s_x[(k / C) * xs + (k % C)] = v;
      absmax(v);
    }
  }
  // every sum is at most max|x| x the largest beam L1 norm of the weights:
  // within x_safe the plain int32 sum is exact
  const bool wide = __syncthreads_or(xmax > (int)p.x_safe) != 0;
  if (wide) {  // the limb weights of the exact int64 path (block-uniform)
    for (unsigned k = tid; k < B * C; k += 256u) s_w[k] = p.w_limbs[k];
    __syncthreads();
  }
  const unsigned bl = tid & 63u, bg = tid >> 6;
  const unsigned bin = bin0 + bl;
  unsigned fl_any = 0;
  unsigned long long nsat = 0;
  // beam b's rounded output y (round_sat(., 15, 16)) to the power cells
  auto out = [&](unsigned b, int32_t yr, int32_t yi, unsigned fr, unsigned fi) {
    if (fr | fi) {
      fl_any |= fr | fi;
      ++nsat;
    }
    cplx y;
    y.re = (int16_t)yr;
    y.im = (int16_t)yi;
    p.power[(f * B + b) * N + bin] = power_u32(y);
    if (p.beams_bn) p.beams_bn[(f * N + bin) * B + b] = pack(y);
  };
  if (bl < nb && !wide) {
    // three products a complex term (Gauss): re = sum xr wr - sum xi wi,
    // im = sum (xr + xi)(wr + wi) - sum xr wr - sum xi wi. The sums run
    // modulo 2^32; the true re and im are below 2^31 - 2^15 in magnitude
    // (x_safe), so the wrapped results are the exact integers.
    const uint32_t* xr = s_x + bl * xs;
    const int4* w3 = s_w3 + bg * C;  // beam bg + 4 j at w3 + 4 j C
    uint32_t sac[BPT], sbd[BPT], sk[BPT];
#pragma unroll
    for (int j = 0; j < BPT; ++j) sac[j] = sbd[j] = sk[j] = 0u;
#pragma unroll(CC ? 16 : 4)
    for (unsigned a = 0; a < C; ++a) {
      const uint32_t xv = xr[a];
      const int x_re = (int)(int16_t)(uint16_t)(xv & 0xFFFFu), x_im = (int)xv >> 16;
      const uint32_t x_s = (uint32_t)(x_re + x_im);
#pragma unroll
      for (int j = 0; j < BPT; ++j) {
        const unsigned b = bg + 4u * j;
        if (BPT == 1 || b < B) {
          const int4 w = w3[4u * j * C + a];
          sac[j] += (uint32_t)(x_re * w.x);
          sbd[j] += (uint32_t)(x_im * w.y);
          sk[j] += x_s * (uint32_t)w.z;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
      const unsigned b = bg + 4u * j;
      if (b < B) {
        unsigned fr = 0, fi = 0;
        const int32_t yr = q15_out32((int32_t)(sac[j] - sbd[j]), &fr);
        const int32_t yi = q15_out32((int32_t)(sk[j] - sac[j] - sbd[j]), &fi);
        out(b, yr, yi, fr, fi);
      }
    }
  } else if (bl < nb) {
    long long ar[BPT], ai[BPT];
#pragma unroll
    for (int j = 0; j < BPT; ++j) ar[j] = ai[j] = 0;
    const uint32_t* xr = s_x + bl * xs;
    for (unsigned a0 = 0; a0 < C; a0 += 64u) {
      const unsigned a1 = (a0 + 64u) < C ? (a0 + 64u) : C;
      int hr[BPT], hi[BPT], lr[BPT], li[BPT];
#pragma unroll
      for (int j = 0; j < BPT; ++j) hr[j] = hi[j] = lr[j] = li[j] = 0;
      for (unsigned a = a0; a < a1; ++a) {
        const uint32_t xv = xr[a];
        const int x_re = (int)(int16_t)(uint16_t)(xv & 0xFFFFu), x_im = (int)xv >> 16;
#pragma unroll
        for (int j = 0; j < BPT; ++j) {
          const unsigned b = bg + 4u * j;
          if (BPT == 1 || b < B) {
            const int4 w = s_w[b * C + a];  // {wh.re, wh.im, wl.re, wl.im}
            hr[j] += x_re * w.x - x_im * w.y;
            hi[j] += x_re * w.y + x_im * w.x;
            lr[j] += x_re * w.z - x_im * w.w;
            li[j] += x_re * w.w + x_im * w.z;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < BPT; ++j) {
        ar[j] += (long long)hr[j] * 256 + lr[j];
        ai[j] += (long long)hi[j] * 256 + li[j];
      }
    }
#pragma unroll
    for (int j = 0; j < BPT; ++j) {
      const unsigned b = bg + 4u * j;
      if (b < B) {
        unsigned fr = 0, fi = 0;
        const int32_t yr = q15_out64(ar[j], &fr), yi = q15_out64(ai[j], &fi);
        out(b, yr, yi, fr, fi);
      }
    }
  }
  const unsigned a = __reduce_or_sync(0xffffffffu, fl_any);
  for (int o = 16; o > 0; o >>= 1) nsat += __shfl_xor_sync(0xffffffffu, nsat, o);
  if ((tid & 31u) == 0u) {
    if (a) atomicOr(&p.stats->bf_flags, a);
    if (nsat) atomicAdd(&p.stats->bf_sat, nsat);
  }
}

template <int BPT, int CC>
static void launch_beam_k(const BeamParams& p, dim3 grid, size_t smem, cudaStream_t s) {
  static PerDevice attr;
  attr.once([] {
    cudaFuncSetAttribute(k_beam<BPT, CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  });
  k_beam<BPT, CC><<<grid, 256, smem, s>>>(p);
}

// The channel counts of the workloads (16, 32, 64) at compile time (up to 64
// beams)
template <int BPT>
static void launch_beam_b(const BeamParams& p, dim3 grid, size_t smem, cudaStream_t s) {
  if constexpr (BPT > 16) {
    launch_beam_k<BPT, 0>(p, grid, smem, s);
  } else {
    switch (p.C) {
      case 16: launch_beam_k<BPT, 16>(p, grid, smem, s); break;
      case 32: launch_beam_k<BPT, 32>(p, grid, smem, s); break;
      case 64: launch_beam_k<BPT, 64>(p, grid, smem, s); break;
      default: launch_beam_k<BPT, 0>(p, grid, smem, s); break;
    }
  }
}

void launch_beam(const BeamParams& p, cudaStream_t s) {
  const unsigned bpt = (p.B + 3u) / 4u;
  const dim3 grid((p.N + 63u) / 64u, p.F);
  const size_t smem = ((size_t)8u * p.B * p.C + 64u * (p.C + 1u)) * sizeof(uint32_t);
  if (bpt <= 1) launch_beam_b<1>(p, grid, smem, s);
  else if (bpt <= 2) launch_beam_b<2>(p, grid, smem, s);
  else if (bpt <= 4) launch_beam_b<4>(p, grid, smem, s);
  else if (bpt <= 8) launch_beam_b<8>(p, grid, smem, s);
  else if (bpt <= 16) launch_beam_b<16>(p, grid, smem, s);
  else launch_beam_b<32>(p, grid, smem, s);
}

// ---------------------------------------------------------------------------
// Covariance: one covar::Integrator pair (re, im) per (bin, pair), stepped
// once per frame with X[x] * conj(X[y]) (covar_model.hpp:119-151, 204-262).
// A CTA owns BT bins x QB pairs. The source vectors of FB frames are staged in
// shared memory per barrier: the next batch is loaded into registers while
// the current one is integrated, so the loop carries no exposed load latency.
// Integrator state lives in registers for the whole chunk. Window count and
// id are the same for every integrator of the stream (they all step on every
// frame), so the host tracks them and passes where windows close.
//
// EXACT: no step can saturate - exponential mode (the accumulator stays
// between its old value and the input, |.| <= 2^31, inside any acc_w >= 33)
// or block mode with window * 2^31 <= 2^(acc_w-1) - 1 (covar_pkg's
// window_max_exact) - so the sum is a plain int64 sum and the flags stay 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void integ_step(long long& acc, long long x, unsigned exp_mode,
                                           unsigned k, unsigned acc_w, unsigned& sticky,
                                           unsigned& satcnt) {
  const long long raw =
      exp_mode ? add_wrap(acc, asr64(sub_wrap(x, acc), k)) : add_wrap(acc, x);
  const unsigned fl = sat_flags64(raw, acc_w);
  acc = sat64(raw, acc_w);
  sticky |= fl;
  if (fl && satcnt != 0xFFFFFFFFu) ++satcnt;
}

constexpr unsigned kCovPre = 4;  // prefetch registers per thread

// MODE: 0 = exact block mode, 1 = exact exponential mode, 2 = saturating
// (either mode, sequential). In exact block mode the chunk's frames are split
// at window boundaries across blockIdx.z (windows are independent there): the
// first segment carries the open window's accumulator in, the last one
// carries its accumulator out, every other one starts from zero.
template <int MODE>
__global__ void __launch_bounds__(256) k_cov(CovParams p, unsigned BT, unsigned QB, unsigned FB) {
  extern __shared__ uint32_t s_src[];  // [FB][BT][S]
  const unsigned tid = threadIdx.x, nth = blockDim.x;
  const unsigned S = p.S, row = BT * S, per_batch = FB * row;
  const unsigned bin0 = blockIdx.x * BT;
  const unsigned bl = tid / QB, q = blockIdx.y * QB + tid % QB;
  const unsigned bin = bin0 + bl;
  const bool live = bl < BT && bin < p.N && q < p.P;
  const size_t k = (size_t)bin * p.P + q;
  // this CTA's frame segment
  const unsigned z = blockIdx.z, nz = gridDim.z;
  const unsigned first = p.wl - p.count0;  // frames until the open window closes
  const unsigned lo = z == 0 ? 0u : first + (z - 1u) * p.wl;
  const unsigned hi_ = z == 0 ? first : first + z * p.wl;
  const unsigned hi = (nz == 1u || hi_ > p.F) ? p.F : hi_;
  const bool carry_in = z == 0, carry_out = z + 1u == nz;
  long long are = 0, aim = 0;
  unsigned st_re = 0, st_im = 0, sc_re = 0, sc_im = 0, xi = 0, yi = 0;
  if (live) {
    if (carry_in) {
      are = p.acc_re[k];
      aim = p.acc_im[k];
    }
    if (MODE == 2) {
      st_re = p.sticky[k] >> 2;
      st_im = p.sticky[k] & 3u;
      sc_re = p.satcnt[2 * k];
      sc_im = p.satcnt[2 * k + 1];
    }
    xi = bl * S + p.px[q];
    yi = bl * S + p.py[q];
  }
  uint32_t pre[kCovPre];
  auto load = [&](unsigned fbase) {
#pragma unroll
    for (unsigned j = 0; j < kCovPre; ++j) {
      const unsigned w = tid + j * nth;
      uint32_t v = 0;
      if (w < per_batch) {
        const unsigned fl = w / row, r = w % row;
        const unsigned f = fbase + fl, b = bin0 + r / S, a = r % S;
        if (f < hi && b < p.N) {
          if (p.src_beam) {
            v = __ldg(p.beams_bn + ((size_t)f * p.N + b) * S + a);
          } else {
            unsigned slot = p.ring_base + f;
            if (slot >= p.ring_frames) slot -= p.ring_frames;
            v = __ldg(p.ring + ((size_t)slot * p.N + b) * S + a);
          }
        }
      }
      pre[j] = v;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (unsigned j = 0; j < kCovPre; ++j) {
      const unsigned w = tid + j * nth;
      if (w < per_batch) s_src[w] = pre[j];
    }
  };
  unsigned count = carry_in ? p.count0 : 0u;
  unsigned w = carry_in ? 0u : z;  // window index of this segment's close
  load(lo);
  store();
  __syncthreads();
  for (unsigned fbase = lo; fbase < hi; fbase += FB) {
    if (fbase + FB < hi) load(fbase + FB);
    const unsigned nf = (hi - fbase) < FB ? (hi - fbase) : FB;
    for (unsigned fl = 0; fl < nf; ++fl) {
      if (live) {
        const uint32_t xv = s_src[fl * row + xi], yv = s_src[fl * row + yi];
        const int xr = (int)(int16_t)(uint16_t)(xv & 0xFFFFu), xm = (int)xv >> 16;
        const int yr = (int)(int16_t)(uint16_t)(yv & 0xFFFFu), ym = (int)yv >> 16;
        // X * conj(Y) through the operand-swap wiring: b = {Y.im, Y.re},
        // re = im(X*b), im = -re(X*b) (covar_model.hpp:137-145)
        if (MODE == 0) {
          are += (long long)xr * yr;
          are += (long long)xm * ym;
          aim += (long long)xm * yr;
          aim -= (long long)xr * ym;
        } else {
          const long long cre = (long long)xr * yr + (long long)xm * ym;
          const long long cim = (long long)xm * yr - (long long)xr * ym;
          if (MODE == 1) {
            are += (cre - are) >> p.exp_k;
            aim += (cim - aim) >> p.exp_k;
          } else {
            integ_step(are, cre, p.exp_mode, p.exp_k, p.acc_w, st_re, sc_re);
            integ_step(aim, cim, p.exp_mode, p.exp_k, p.acc_w, st_im, sc_im);
          }
        }
      }
      if (++count >= p.wl) {  // uniform over the block
        if (live && w < p.n_windows) {
          long long* o = p.out + (((size_t)w * p.N + bin) * p.P + q) * 2;
          o[0] = are;
          o[1] = aim;
          if (MODE == 2 && (st_re | st_im)) atomicOr(&p.win_flags[w], st_re | st_im);
        }
        if (MODE != 1 && !(MODE == 2 && p.exp_mode)) are = aim = 0;
        count = 0;
        ++w;
      }
    }
    __syncthreads();
    store();
    __syncthreads();
  }
  if (live && carry_out) {
    p.acc_re_out[k] = are;
    p.acc_im_out[k] = aim;
    if (MODE == 2) {
      p.sticky[k] = (st_re << 2) | st_im;
      const unsigned old_re = p.satcnt[2 * k], old_im = p.satcnt[2 * k + 1];
      p.satcnt[2 * k] = sc_re;
      p.satcnt[2 * k + 1] = sc_im;
      const unsigned long long d = (unsigned long long)(sc_re - old_re) + (sc_im - old_im);
      if (d) atomicAdd(&p.stats->cov_sat_steps, d);
      if (st_re | st_im) atomicOr(&p.stats->cov_flags, st_re | st_im);
    }
  }
}

// Exact block mode (MODE 0 of k_cov) with the source vectors staged once per
// batch as unpacked {re, im} int32 pairs, so a (bin, pair) thread spends a
// frame on two 64-bit shared loads and four multiply-adds. A CTA's frames are
// one window segment (split as in k_cov), so the window closes at most once,
// after the loop, and no frame needs a count check. SS > 0 fixes the source
// width at compile time for launches of one bin a CTA (BT = 1), so a frame's
// staged row is a constant stride.
template <int SS>
__global__ void __launch_bounds__(256) k_cov_block(CovParams p, unsigned BT, unsigned QB,
                                                   unsigned FB) {
  extern __shared__ int2 s_xy[];  // [FB][BT][S]
  const unsigned tid = threadIdx.x, nth = blockDim.x;
  const unsigned S = SS ? (unsigned)SS : p.S, row = SS ? (unsigned)SS : BT * S;
  const unsigned per_batch = FB * row;
  const unsigned bin0 = blockIdx.x * BT;
  const unsigned bl = SS ? 0u : tid / QB, q = blockIdx.y * QB + (SS ? tid : tid % QB);
  const unsigned bin = bin0 + bl;
  const bool live = (SS ? tid < QB : bl < BT) && bin < p.N && q < p.P;
  const size_t k = (size_t)bin * p.P + q;
  const unsigned z = blockIdx.z, nz = gridDim.z;
  const unsigned first = p.wl - p.count0;  // frames until the open window closes
  const unsigned lo = z == 0 ? 0u : first + (z - 1u) * p.wl;
  const unsigned hi_ = z == 0 ? first : first + z * p.wl;
  const unsigned hi = (nz == 1u || hi_ > p.F) ? p.F : hi_;
  const unsigned xi = live ? bl * S + p.px[q] : 0u, yi = live ? bl * S + p.py[q] : 0u;
  long long are = 0, aim = 0;
  uint32_t pre[kCovPre];
  // row and S powers of two (the usual geometries): the staged word's frame,
  // bin and channel by shifts
  const int rsh = (row & (row - 1u)) == 0u ? __ffs(row) - 1 : -1;
  const int ssh = (S & (S - 1u)) == 0u ? __ffs(S) - 1 : -1;
  const bool pow2 = rsh >= 0 && ssh >= 0;
  auto load = [&](unsigned fbase) {
#pragma unroll
    for (unsigned j = 0; j < kCovPre; ++j) {
      const unsigned w = tid + j * nth;
      uint32_t v = 0;
      if (w < per_batch) {
        unsigned fl, r, bq, a;
        if (pow2) {
          fl = w >> rsh;
          r = w & (row - 1u);
          bq = r >> ssh;
          a = r & (S - 1u);
        } else {
          fl = w / row;
          r = w % row;
          bq = r / S;
          a = r % S;
        }
        const unsigned f = fbase + fl, b = bin0 + bq;
        if (f < hi && b < p.N) {
          if (p.src_beam) {
            v = __ldg(p.beams_bn + ((size_t)f * p.N + b) * S + a);
          } else {
            unsigned slot = p.ring_base + f;
            if (slot >= p.ring_frames) slot -= p.ring_frames;
            v = __ldg(p.ring + ((size_t)slot * p.N + b) * S + a);
          }
        }
      }
      pre[j] = v;
    }
  };
  int smax = 0;
  auto store = [&]() {
    smax = 0;
#pragma unroll
    for (unsigned j = 0; j < kCovPre; ++j) {
      const unsigned w = tid + j * nth;
      if (w < per_batch) {
        const int re = (int)(int16_t)(uint16_t)(pre[j] & 0xFFFFu), im = (int)pre[j] >> 16;
        s_xy[w] = make_int2(re, im);
        smax = max(smax, max(abs(re), abs(im)));
      }
    }
  };
  if (lo < hi) load(lo);
  for (unsigned fbase = lo; fbase < hi; fbase += FB) {
    __syncthreads();
    store();
    // with every value of the batch <= 5792 in magnitude, 32 frames sum at
    // most 32 x 2 x 5792^2 < 2^31 per pair: exact in int32, folded into the
    // int64 sums every 32 frames
    const bool wide = __syncthreads_or(smax > 5792) != 0;
    if (fbase + FB < hi) load(fbase + FB);
    const unsigned nf = (hi - fbase) < FB ? (hi - fbase) : FB;
    if (live && !wide) {
      const int2* xs = s_xy + xi;
      const int2* ys = s_xy + yi;
      for (unsigned s0 = 0; s0 < nf; s0 += 32u) {
        const unsigned s1 = (nf - s0) < 32u ? nf : s0 + 32u;
        int sr = 0, si = 0;
#pragma unroll(SS ? 8 : 4)
        for (unsigned fl = s0; fl < s1; ++fl) {
          const int2 x = xs[fl * row], y = ys[fl * row];
          sr += x.x * y.x + x.y * y.y;
          si += x.y * y.x - x.x * y.y;
        }
        are += sr;
        aim += si;
      }
    } else if (live) {
      const int2* xs = s_xy + xi;
      const int2* ys = s_xy + yi;
      // X * conj(Y) through the operand-swap wiring (covar_model.hpp:137-145)
#pragma unroll 4
      for (unsigned fl = 0; fl < nf; ++fl) {
        const int2 x = xs[fl * row], y = ys[fl * row];
        are += (long long)x.x * y.x;
        are += (long long)x.y * y.y;
        aim += (long long)x.y * y.x;
        aim -= (long long)x.x * y.y;
      }
    }
  }
  if (!live) return;
  if (z == 0u) {  // the open window carried in
    are += p.acc_re[k];
    aim += p.acc_im[k];
  }
  if (z < p.n_windows) {  // this segment closes window z of the launch
    long long* o = p.out + (((size_t)z * p.N + bin) * p.P + q) * 2;
    o[0] = are;
    o[1] = aim;
    are = aim = 0;
  }
  if (z + 1u == nz) {  // the window left open carried out
    p.acc_re_out[k] = are;
    p.acc_im_out[k] = aim;
  }
}

void launch_cov(const CovParams& p, cudaStream_t s) {
  if (p.P == 0 || p.F == 0) return;
  unsigned QB, BT;
  if (p.P >= 256u) {
    QB = 256u;
    BT = 1u;
  } else {
    QB = p.P;
    BT = 256u / p.P;
  }
  const unsigned nth = ((BT * QB + 31u) / 32u) * 32u;
  const int mode = !p.exact ? 2 : (p.exp_mode ? 1 : 0);
  // frames staged per barrier: as many as the prefetch registers hold (the
  // block kernel folds its int32 sums every 32 frames; the sequential
  // integrators stage at most 32)
  unsigned FB = (kCovPre * nth) / (BT * p.S);
  if (FB > (mode == 0 ? 128u : 32u)) FB = mode == 0 ? 128u : 32u;
  if (FB < 1u) FB = 1u;
  // segments: the open window, every whole window, the trailing partial one
  unsigned nz = 1;
  if (mode == 0) {
    const unsigned first = p.wl - p.count0;
    nz = first >= p.F ? 1u : 1u + (p.F - first + p.wl - 1u) / p.wl;
  }
  const dim3 grid((p.N + BT - 1u) / BT, (p.P + QB - 1u) / QB, nz);
  const size_t smem = (size_t)FB * BT * p.S * sizeof(uint32_t);
  if (mode == 0) {
    if (BT == 1u && (p.S == 16u || p.S == 32u || p.S == 64u)) {
      if (p.S == 16u) k_cov_block<16><<<grid, nth, 2 * smem, s>>>(p, BT, QB, FB);
      else if (p.S == 32u) k_cov_block<32><<<grid, nth, 2 * smem, s>>>(p, BT, QB, FB);
      else k_cov_block<64><<<grid, nth, 2 * smem, s>>>(p, BT, QB, FB);
    } else {
      k_cov_block<0><<<grid, nth, 2 * smem, s>>>(p, BT, QB, FB);
    }
  }
  else if (mode == 1) k_cov<1><<<grid, nth, smem, s>>>(p, BT, QB, FB);
  else k_cov<2><<<grid, nth, smem, s>>>(p, BT, QB, FB);
}

// ---------------------------------------------------------------------------
// CFAR (cfar_model.hpp:243-340) in two launches.
// Decide: a warp per CFAR frame (frame x beam), or for frames of at most 64
// cells several frames a warp. The warp loads its cells with 16-byte loads
// (4 cells a lane), builds the prefix sums in shared memory, decides every
// cell (the lead/lag reference sums as prefix differences - the same integers
// the model's loops add) and keeps a ballot mask of the cells that emit, the
// frame's event count, its detected / suppressed counts and its first
// detections. The grid is one persistent wave; the event counts are summed
// per 8-frame group and per 64 groups.
// Emit: a CTA takes 64 frames (256 when frames are at most 64 cells). Its
// first event's offset sums the block totals and group totals before it; a
// scan of its frames' counts places every event, and each thread writes one
// event and builds its packet in shared memory, the round's packets leaving
// as one coalesced run.
// ---------------------------------------------------------------------------
constexpr unsigned kCfarWarps = 8;        // decide: warps per CTA, frames per group
constexpr unsigned kEmitFrames = 64;      // emit: frames per CTA (frames of 65+ cells)
constexpr unsigned kCfarBlock = 64;       // groups per block total

// 8-frame groups of a launch; the totals array holds their counts, then one
// total per 64 groups (cfar_tiles words)
__host__ __device__ __forceinline__ uint64_t cfar_groups(uint64_t frames) {
  return (frames + kCfarWarps - 1u) / kCfarWarps;
}

__device__ __forceinline__ uint64_t cell_at(const CfarParams& p, uint64_t u, unsigned i) {
  if (p.power_u32) return p.power_u32[u * p.n + i];
  const long long v = p.cells_i64[u * p.n + i];
  return v < 0 ? 0ull : (uint64_t)v;  // clamp_cell (cfar_model.hpp:238-240)
}

// Cells 4 at a time: lane l of row r holds cells 128 r + 4 l .. + 3.
__device__ __forceinline__ void cells4(const CfarParams& p, uint64_t u, unsigned i0, bool vec,
                                       uint64_t* c) {
  if (vec && i0 < p.n) {  // n % 4 == 0: the whole quad is in the frame
    if (p.power_u32) {
      const uint4 v = __ldcs(reinterpret_cast<const uint4*>(p.power_u32 + u * p.n + i0));
      c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
    } else {
      const longlong2* q = reinterpret_cast<const longlong2*>(p.cells_i64 + u * p.n + i0);
      const longlong2 a = __ldcs(q), b = __ldcs(q + 1);
      c[0] = a.x < 0 ? 0ull : (uint64_t)a.x;
      c[1] = a.y < 0 ? 0ull : (uint64_t)a.y;
      c[2] = b.x < 0 ? 0ull : (uint64_t)b.x;
      c[3] = b.y < 0 ? 0ull : (uint64_t)b.y;
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) c[k] = i0 + k < p.n ? cell_at(p, u, i0 + k) : 0ull;
}

// The chain's 32-bit power cells kept in 32 bits: half the registers of the
// 64-bit form, so a 1024-cell frame's 32 cells a lane leave room for two CTAs
// an SM.
__device__ __forceinline__ void cells4(const CfarParams& p, uint64_t u, unsigned i0, bool vec,
                                       uint32_t* c) {
  const uint32_t* row = p.power_u32 + u * p.n;
  if (vec && i0 < p.n) {
    const uint4 v = __ldcs(reinterpret_cast<const uint4*>(row + i0));
    c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
    return;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) c[k] = i0 + k < p.n ? row[i0 + k] : 0u;
}

// The frame's cells, 4 a lane per row: lane l of row r holds cells
// 128 r + 4 l .. + 3 (zero past the frame). R >= ceil(n / 128) bounds the
// rows at compile time; every row is loaded before the first scan step.
// Tc = uint32_t reads the 32-bit power cells only.
template <int R, class Tc>
__device__ __forceinline__ void load_cells(const CfarParams& p, uint64_t u, bool vec,
                                           Tc (&c)[R][4]) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (int r = 0; r < R; ++r) cells4(p, u, (unsigned)r * 128u + lane * 4u, vec, c[r]);
}

__device__ __forceinline__ void store4(uint64_t* d, uint64_t a, uint64_t b, uint64_t c,
                                       uint64_t e) {
  reinterpret_cast<ulonglong2*>(d)[0] = make_ulonglong2(a, b);
  reinterpret_cast<ulonglong2*>(d)[1] = make_ulonglong2(c, e);
}
__device__ __forceinline__ void store4(uint32_t* d, uint32_t a, uint32_t b, uint32_t c,
                                       uint32_t e) {
  reinterpret_cast<uint4*>(d)[0] = make_uint4(a, b, c, e);
}

// Inclusive prefix sums pre[1..n] of the loaded cells (pre[0] = 0),
// warp-cooperative, in Tp: uint64_t, or uint32_t modulo 2^32 when every
// window sum the decisions take is below 2^32 (a difference of two wrapped
// prefixes is then the exact sum). pre + 1 sits on a 16-byte boundary, so
// lane l's pre[4l + 1 .. 4l + 4] are aligned 16-byte stores.
template <int R, class Tp, class Tc>
__device__ __forceinline__ void warp_prefix(const CfarParams& p, const Tc (&c)[R][4], Tp* pre,
                                            bool vec) {
  const unsigned lane = threadIdx.x & 31u;
  if (lane == 0) pre[0] = 0;
  Tp carry = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const Tp t0 = (Tp)c[r][0], t1 = t0 + (Tp)c[r][1], t2 = t1 + (Tp)c[r][2],
             t3 = t2 + (Tp)c[r][3];
    Tp x = t3;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const Tp t = __shfl_up_sync(0xffffffffu, x, o);
      if ((int)lane >= o) x += t;
    }
    const Tp b = carry + x - t3;
    const unsigned i0 = (unsigned)r * 128u + lane * 4u;
    if (vec && i0 < p.n) {
      store4(pre + i0 + 1, b + t0, b + t1, b + t2, b + t3);
    } else {
      if (i0 < p.n) pre[i0 + 1] = b + t0;
      if (i0 + 1 < p.n) pre[i0 + 2] = b + t1;
      if (i0 + 2 < p.n) pre[i0 + 3] = b + t2;
      if (i0 + 3 < p.n) pre[i0 + 4] = b + t3;
    }
    carry += __shfl_sync(0xffffffffu, x, 31);
  }
  __syncwarp();
}

__device__ __forceinline__ void set_field(uint64_t* w, unsigned lsb, unsigned n, uint64_t v) {
  v &= (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
  const unsigned wi = lsb >> 6, sh = lsb & 63u;
  w[wi] |= v << sh;
  if (sh + n > 64u) w[wi + 1] |= v >> (64u - sh);
}

// 176-bit event of cfar_model.hpp:75-84 (fields masked to their widths)
__device__ __forceinline__ void make_event(rd_event* e, unsigned kind, unsigned bin,
                                           unsigned fid, unsigned refc, unsigned alpha,
                                           unsigned det, unsigned sup, uint64_t cut,
                                           uint64_t sum, bool sof, bool eof, uint32_t frame,
                                           uint16_t beam) {
  uint64_t w[3] = {0, 0, 0};
  set_field(w, 0, 2, kind);
  set_field(w, 2, 16, bin);
  set_field(w, 18, 16, fid);
  set_field(w, 34, 7, refc);
  set_field(w, 41, 16, alpha);
  set_field(w, 57, 16, det);
  set_field(w, 73, 16, sup);
  set_field(w, 89, 40, cut);
  set_field(w, 129, 47, sum);
  e->w[0] = w[0];
  e->w[1] = w[1];
  e->w[2] = w[2];
  e->frame = frame;
  e->beam = beam;
  e->kind = (uint8_t)kind;
  e->framing = (uint8_t)((sof ? 1u : 0u) | (eof ? 2u : 0u));
}

// An event as two 16-byte stores when the buffer allows it (the layout of
// rd_event: w[3], frame, beam, kind, framing).
__device__ __forceinline__ void store_event(rd_event* d, const rd_event& e, bool v16) {
  if (v16) {
    const unsigned long long tail = (unsigned long long)e.frame |
                                    ((unsigned long long)e.beam << 32) |
                                    ((unsigned long long)e.kind << 48) |
                                    ((unsigned long long)e.framing << 56);
    ulonglong2* q = reinterpret_cast<ulonglong2*>(d);
    q[0] = make_ulonglong2(e.w[0], e.w[1]);
    q[1] = make_ulonglong2(e.w[2], tail);
  } else {
    *d = e;
  }
}

// 32 bits of the zero-padded 192-bit string {w0, w1, w2} starting at signed
// bit s (the words picked by selects, so nothing goes to local memory).
__device__ __forceinline__ uint32_t ext32(uint64_t w0, uint64_t w1, uint64_t w2, int s) {
  if (s >= 192 || s <= -32) return 0u;
  if (s < 0) return (uint32_t)(w0 << (-s));
  const int lo = s >> 6, sh = s & 63;
  const uint64_t a = lo == 0 ? w0 : (lo == 1 ? w1 : w2);
  const uint64_t b = lo == 0 ? w1 : (lo == 1 ? w2 : 0ull);
  uint64_t v = a >> sh;
  if (sh) v |= b << (64 - sh);
  return (uint32_t)v;
}

// One detection packet: the header flit (packet_model.hpp:150-159, sof) and
// payload flits carrying the event LS word first (benchmark_sim_top.sv:
// 1818-1936); flit = data << 5 | eof << 4 | sof << 3 | vc << 1 | odd parity.
// Each 32-bit flit word is cut from the payload bit string with two shifts.
__device__ void write_packet(const rd_event& e, uint32_t* out, unsigned pw, unsigned words,
                             unsigned nfl, unsigned src, unsigned dest, unsigned vc,
                             unsigned seq) {
  const uint64_t hdr = (uint64_t)(dest & 0xFu) | ((uint64_t)(src & 0x1Fu) << 4) |
                       ((uint64_t)(vc & 3u) << 9) | ((uint64_t)0u << 11) |
                       ((uint64_t)(nfl & 0x3Fu) << 14) | ((uint64_t)(seq & 0xFFFFu) << 20);
  const int top = 5 + (int)pw;  // first flit bit past the data
  for (unsigned f = 0; f < nfl; ++f) {
    uint32_t* o = out + (size_t)f * words;
    const uint64_t w0 = f == 0 ? hdr : e.w[0], w1 = f == 0 ? 0ull : e.w[1],
                   w2 = f == 0 ? 0ull : e.w[2];
    const int off = f == 0 ? 0 : (int)((f - 1) * pw);
    // payload bits past this flit's slice belong to the next flit
    const int last = f == 0 ? 36 : (off + (int)pw < 176 ? off + (int)pw : 176);
    const int lim = 5 + (last - off) < top ? 5 + (last - off) : top;  // flit bits in use
    unsigned pop = 0;
    for (unsigned k = 0; k < words; ++k) {
      const int lo = 32 * (int)k;
      uint32_t v = ext32(w0, w1, w2, off + lo - 5);
      if (lo < 5) v &= ~0x1Fu;
      if (lo + 32 > lim) v &= (lim <= lo) ? 0u : ((1u << (lim - lo)) - 1u);
      if (k == 0)
        v |= ((vc & 3u) << 1) | ((f == 0 ? 1u : 0u) << 3) | ((f + 1 == nfl ? 1u : 0u) << 4);
      pop += __popc(v);
      o[k] = v;
    }
    if ((pop & 1u) == 0u) o[0] |= 1u;
  }
}

// write_packet for a packet width fixed at compile time: every word's bit
// offset is a constant, so each word is one funnel shift of the event words
// and a mask. PW = 0 falls back to the general form.
template <unsigned PW>
__device__ __forceinline__ void write_packet_w(const rd_event& e, uint32_t* out, unsigned pw,
                                               unsigned words, unsigned nfl, unsigned src,
                                               unsigned dest, unsigned vc, unsigned seq) {
  if constexpr (PW == 0) {
    write_packet(e, out, pw, words, nfl, src, dest, vc, seq);
  } else {
    constexpr unsigned W = (PW + 5u + 31u) / 32u, NF = 1u + (176u + PW - 1u) / PW;
    constexpr int top = 5 + (int)PW;
    const uint64_t hdr = (uint64_t)(dest & 0xFu) | ((uint64_t)(src & 0x1Fu) << 4) |
                         ((uint64_t)(vc & 3u) << 9) | ((uint64_t)(NF & 0x3Fu) << 14) |
                         ((uint64_t)(seq & 0xFFFFu) << 20);
#pragma unroll
    for (unsigned f = 0; f < NF; ++f) {
      const uint64_t w0 = f == 0 ? hdr : e.w[0], w1 = f == 0 ? 0ull : e.w[1],
                     w2 = f == 0 ? 0ull : e.w[2];
      const int off = f == 0 ? 0 : (int)((f - 1) * PW);
      const int last = f == 0 ? 36 : (off + (int)PW < 176 ? off + (int)PW : 176);
      const int lim = 5 + (last - off) < top ? 5 + (last - off) : top;
      unsigned pop = 0;
      uint32_t first = 0;
#pragma unroll
      for (unsigned k = 0; k < W; ++k) {
        const int lo = 32 * (int)k;
        uint32_t v = ext32(w0, w1, w2, off + lo - 5);
        if (lo < 5) v &= ~0x1Fu;
        if (lo + 32 > lim) v &= (lim <= lo) ? 0u : ((1u << (lim - lo)) - 1u);
        if (k == 0) {
          v |= ((vc & 3u) << 1) | ((f == 0 ? 1u : 0u) << 3) | ((f + 1 == NF ? 1u : 0u) << 4);
          first = v;
        } else {
          out[f * W + k] = v;
        }
        pop += __popc(v);
      }
      out[f * W] = first | ((pop & 1u) ? 0u : 1u);  // odd parity
    }
  }
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// A detection as the emit pass needs it, 16 bytes: cut (40 bits), bin,
// kind, the window sum (47 bits) and the reference count - the fields of the
// 176-bit event that the decision sets (cfar_model.hpp:75-84 widths).
__device__ __forceinline__ uint4 pack_detection(uint64_t cut, unsigned bin, unsigned kind,
                                                uint64_t sum, unsigned refc) {
  cut &= (1ull << 40) - 1ull;
  sum &= (1ull << 47) - 1ull;
  return make_uint4((uint32_t)cut, (uint32_t)(cut >> 32) | ((bin & 0xFFFFu) << 8) | (kind << 24),
                    (uint32_t)sum, (uint32_t)(sum >> 32) | ((refc & 0x7Fu) << 15));
}

// Decides every cell of frame u from its prefix sums (Tp as in warp_prefix;
// the products and comparisons in 64 bits either way): the ballot mask of the
// emitting cells, the detection slots, the frame's counts. Returns the
// frame's event count (detections + SUMMARY) and adds its detections to det.
template <int R, class Tp>
__device__ __forceinline__ unsigned decide_frame(const CfarParams& p, uint64_t u, const Tp* pre,
                                                 bool live, int lo_b, int hi_b, unsigned n_ok,
                                                 unsigned& det) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned words = (p.n + 31u) / 32u;  // at most 4 R
  const unsigned ca_n8 = (p.rl + p.rg) << 8;
  unsigned emitted = 0, mword = 0;
  // unrolled by 4, not fully: 32 copies of the step overflow the instruction
  // cache at 1024 cells (warps then stall on instruction fetch)
#pragma unroll 4
  for (unsigned r = 0; r < 4u * R; ++r) {
    if (r >= words) break;
    const unsigned i = r * 32u + lane;
    bool dt = false;
    Tp cut = 0, sum = 0;  // in Tp: every window sum fits (see warp_prefix)
    unsigned nref = 0;
    const bool ok = live && (int)i >= lo_b && (int)i < hi_b;  // i < n follows
    if (ok) {
      cut = pre[i + 1] - pre[i];
      const Tp sl = pre[i + p.gl + p.rl + 1] - pre[i + p.gl + 1];
      const Tp sg = pre[i - p.gg] - pre[i - p.gg - p.rg];
      uint64_t lhs;
      if (p.go) {
        const bool lead = ((uint64_t)sl * p.rg) >= ((uint64_t)sg * p.rl);
        sum = lead ? sl : sg;
        nref = lead ? p.rl : p.rg;
        lhs = ((uint64_t)cut * nref) << 8;
      } else {
        sum = sl + sg;
        nref = p.rl + p.rg;
        lhs = (uint64_t)cut * ca_n8;
      }
      dt = lhs > (uint64_t)p.alpha * sum;
    }
    bool em = dt;
    unsigned m = __ballot_sync(0xffffffffu, dt);
    det += __popc(m);
    if (p.dense) {  // every cell emits; the detected ones still count
      em = i < p.n;
      m = __ballot_sync(0xffffffffu, em);
      if (em && !ok) cut = pre[i + 1] - pre[i];
    }
    if (lane == (r & 31u)) mword = m;
    if (em) {  // the frame's k-th event, while it fits the frame's slots
      const unsigned k = emitted + __popc(m & ((1u << lane) - 1u));
      if (k < kCfarSlots)
        p.slots[u * kCfarSlots + k] =
            pack_detection((uint64_t)cut, i, dt ? 0u : (!ok ? 2u : 1u), ok ? (uint64_t)sum : 0ull,
                           ok ? nref : 0u);
    }
    emitted += __popc(m);
  }
  if (lane < words) p.mask[u * words + lane] = mword;  // words <= 32
  if (lane == 0) {
    p.counts[u] = emitted + 1u;
    p.detsup[u] = det | ((p.n - n_ok) << 16);  // n <= 1024: both fit 16 bits
  }
  return emitted + 1u;  // + SUMMARY
}

// Persistent: each CTA's 8 warps take 8-frame groups g = blockIdx.x,
// blockIdx.x + gridDim.x, ... (warp w the group's frame w), so warps never
// wait for each other and the grid is one wave; a frame's event count goes
// into its group's total and its 64-group block's total (zeroed before the
// launch) by two atomics, and each warp adds its detected and suppressed
// counts once at the end.
template <int R, class Tc>
__global__ void __launch_bounds__(kCfarWarps * 32, sizeof(Tc) == 4 ? 3 : 2) k_cfar_decide(CfarParams p) {
  extern __shared__ __align__(16) uint64_t s_pre[];
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  // the warp's n + 2 words (on a 16-byte boundary when n is even, as the
  // 16-byte stores need)
  uint64_t* wbase = s_pre + (size_t)warp * (p.n + 2u);
  // cells whose window fits the frame: lo_b <= i < hi_b; only they are
  // evaluable, so the suppressed count is the same for every frame
  const int lo_b = (int)(p.gg + p.rg), hi_b = (int)p.n - (int)(p.gl + p.rl);
  const bool usable = p.go ? (p.rl != 0u && p.rg != 0u) : (p.rl + p.rg) != 0u;
  const bool live = p.enable && usable;
  const unsigned n_ok = live && hi_b > lo_b ? (unsigned)(hi_b - lo_b) : 0u;
  // the emit pass counts from the events before this launch
  if (blockIdx.x == 0 && threadIdx.x == 0) p.stats->scan_scratch[1] = p.stats->events_call;
  unsigned long long det_w = 0, sup_w = 0;
  const uint64_t groups = cfar_groups(p.frames);
  for (uint64_t g = blockIdx.x; g * kCfarWarps < p.frames; g += gridDim.x) {
    const uint64_t u = g * kCfarWarps + warp;
    if (u >= p.frames) break;  // warp-uniform
    unsigned det = 0, count;
    Tc c[R][4];
    load_cells<R>(p, u, p.vec, c);
    // every window sum (and the cell) below 2^32 when the largest cell times
    // the reference cells plus one is: the scan then runs in 32 bits
    Tc mx = 0;
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int k = 0; k < 4; ++k) mx = c[r][k] > mx ? c[r][k] : mx;
    bool narrow = !__any_sync(0xffffffffu, ((uint64_t)mx >> 32) != 0ull);
    if (narrow)
      narrow = (uint64_t)__reduce_max_sync(0xffffffffu, (unsigned)mx) * (p.rl + p.rg + 1u) <=
               0xFFFFFFFFull;
    if (narrow) {  // pre[0] three words past the boundary: pre + 1 on it
      uint32_t* pre = reinterpret_cast<uint32_t*>(wbase) + 3;
      warp_prefix<R>(p, c, pre, p.vec);
      count = decide_frame<R>(p, u, pre, live, lo_b, hi_b, n_ok, det);
    } else {  // pre[0] one word past the boundary
      uint64_t* pre = wbase + 1;
      warp_prefix<R>(p, c, pre, p.vec);
      count = decide_frame<R>(p, u, pre, live, lo_b, hi_b, n_ok, det);
    }
    if (lane == 0) {
      atomicAdd(&p.totals[g], (unsigned long long)count);
      atomicAdd(&p.totals[groups + g / kCfarBlock], (unsigned long long)count);
    }
    det_w += det;
    sup_w += p.n - n_ok;  // every frame has its SUMMARY
    __syncwarp();  // the warp's words are rewritten by its next frame
  }
  if (lane == 0) {
    if (det_w) atomicAdd(&p.stats->cfar_det, det_w);
    if (sup_w) atomicAdd(&p.stats->cfar_sup, sup_w);
  }
}

// Frames of at most 64 cells, several to a warp. A warp pass holds 128 / NP
// frames of NP cells (NP = 16, 32 or 64; a frame's cells past n are zero):
// lane l loads cells 4 (l % (NP / 4)) .. + 3 of frame l / (NP / 4), a scan
// segmented at the frame boundaries writes each frame's prefix sums, and the
// 128 cells are decided 32 a step exactly as k_cfar_decide decides them, each
// frame keeping its own mask words, slots and counts. For NP = 16 a 32-cell
// step spans two frames, whose ballot halves are taken apart by a mask.
template <int NP, class Tp, class Tc>
__device__ __forceinline__ void packed_pass(const CfarParams& p, const Tc (&c)[4], uint64_t u0,
                                            uint64_t* wbase, bool live, int lo_b, int hi_b,
                                            unsigned n_ok, unsigned long long& det_w) {
  constexpr unsigned LPF = NP / 4u;       // lanes a frame holds
  constexpr unsigned STRIDE = NP + 4u;    // prefix words a frame (a multiple of 4)
  constexpr unsigned OFF = sizeof(Tp) == 4 ? 3u : 1u;  // pre + 1 on a 16-byte boundary
  const unsigned lane = threadIdx.x & 31u;
  Tp* base = reinterpret_cast<Tp*>(wbase);
  {  // segmented scan: inclusive prefixes pre[1..n] of lane l's frame
    const unsigned a = lane / LPF, i0 = 4u * (lane % LPF);
    Tp* pre = base + a * STRIDE + OFF;
    const Tp t0 = (Tp)c[0], t1 = t0 + (Tp)c[1], t2 = t1 + (Tp)c[2], t3 = t2 + (Tp)c[3];
    Tp x = t3;
#pragma unroll
    for (unsigned o = 1; o < LPF; o <<= 1) {
      const Tp t = __shfl_up_sync(0xffffffffu, x, o);
      if ((lane % LPF) >= o) x += t;
    }
    const Tp b = x - t3;
    if (i0 == 0u) pre[0] = 0;
    if (p.vec && i0 < p.n) {
      store4(pre + i0 + 1, b + t0, b + t1, b + t2, b + t3);
    } else {
      if (i0 < p.n) pre[i0 + 1] = b + t0;
      if (i0 + 1 < p.n) pre[i0 + 2] = b + t1;
      if (i0 + 2 < p.n) pre[i0 + 3] = b + t2;
      if (i0 + 3 < p.n) pre[i0 + 4] = b + t3;
    }
  }
  __syncwarp();
  const unsigned words = (p.n + 31u) / 32u;  // mask words a frame: 1, or 2 for NP = 64
  const unsigned ca_n8 = (p.rl + p.rg) << 8;
  // this lane's frame's bits of a ballot, and the bits below the lane
  const unsigned fmask = NP >= 32 ? 0xFFFFFFFFu : (0xFFFFu << (lane & 16u));
  const unsigned below = (1u << lane) - 1u;
  unsigned emitted = 0, detf = 0;
#pragma unroll
  for (unsigned r = 0; r < 4u; ++r) {
    const unsigned j = r * 32u + lane;
    const unsigned a = j / NP, i = j % NP;
    const uint64_t u = u0 + a;
    const bool valid = u < p.frames;
    const Tp* pre = base + a * STRIDE + OFF;
    if ((r * 32u) % NP == 0u) emitted = detf = 0;  // a frame starts with this step
    bool dt = false;
    Tp cut = 0, sum = 0;
    unsigned nref = 0;
    const bool ok = live && valid && (int)i >= lo_b && (int)i < hi_b;  // i < n follows
    if (ok) {
      cut = pre[i + 1] - pre[i];
      const Tp sl = pre[i + p.gl + p.rl + 1] - pre[i + p.gl + 1];
      const Tp sg = pre[i - p.gg] - pre[i - p.gg - p.rg];
      uint64_t lhs;
      if (p.go) {
        const bool lead = ((uint64_t)sl * p.rg) >= ((uint64_t)sg * p.rl);
        sum = lead ? sl : sg;
        nref = lead ? p.rl : p.rg;
        lhs = ((uint64_t)cut * nref) << 8;
      } else {
        sum = sl + sg;
        nref = p.rl + p.rg;
        lhs = (uint64_t)cut * ca_n8;
      }
      dt = lhs > (uint64_t)p.alpha * sum;
    }
    bool em = dt;
    const unsigned dm = __ballot_sync(0xffffffffu, dt);
    unsigned m = dm;
    if (lane == 0) det_w += __popc(dm);
    if (p.dense) {  // every cell emits; the detected ones still count
      em = valid && i < p.n;
      m = __ballot_sync(0xffffffffu, em);
      if (em && !ok) cut = pre[i + 1] - pre[i];
    }
    const unsigned mf = m & fmask;
    if (em) {
      const unsigned k = emitted + __popc(mf & below);
      if (k < kCfarSlots)
        p.slots[u * kCfarSlots + k] =
            pack_detection((uint64_t)cut, i, dt ? 0u : (!ok ? 2u : 1u), ok ? (uint64_t)sum : 0ull,
                           ok ? nref : 0u);
    }
    emitted += __popc(mf);
    detf += __popc(dm & fmask);
    const bool first = (i % 32u) == 0u;  // the frame's first lane in this step
    if (valid && first) p.mask[u * words + i / 32u] = NP >= 32 ? mf : mf >> (lane & 16u);
    if (valid && first && ((r * 32u + 32u) % NP == 0u || NP < 32)) {  // the frame's last step
      p.counts[u] = emitted + 1u;
      p.detsup[u] = detf | ((p.n - n_ok) << 16);
      atomicAdd(&p.totals[u / kCfarWarps], (unsigned long long)(emitted + 1u));
      atomicAdd(&p.totals[cfar_groups(p.frames) + u / (kCfarWarps * kCfarBlock)],
                (unsigned long long)(emitted + 1u));
    }
  }
  __syncwarp();  // the warp's words are rewritten by its next pass
}

template <int NP, class Tc>
__global__ void __launch_bounds__(kCfarWarps * 32, 4) k_cfar_decide_packed(CfarParams p) {
  constexpr unsigned RW = 128u / NP;  // frames a warp pass
  constexpr unsigned LPF = NP / 4u;
  __shared__ __align__(16) uint64_t s_pre[kCfarWarps * RW * (NP + 4u)];
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  uint64_t* wbase = s_pre + (size_t)warp * RW * (NP + 4u);
  const int lo_b = (int)(p.gg + p.rg), hi_b = (int)p.n - (int)(p.gl + p.rl);
  const bool usable = p.go ? (p.rl != 0u && p.rg != 0u) : (p.rl + p.rg) != 0u;
  const bool live = p.enable && usable;
  const unsigned n_ok = live && hi_b > lo_b ? (unsigned)(hi_b - lo_b) : 0u;
  if (blockIdx.x == 0 && threadIdx.x == 0) p.stats->scan_scratch[1] = p.stats->events_call;
  unsigned long long det_w = 0, sup_w = 0;
  const uint64_t passes = ((uint64_t)p.frames + RW - 1u) / RW;
  for (uint64_t q = (uint64_t)blockIdx.x * kCfarWarps + warp; q < passes;
       q += (uint64_t)gridDim.x * kCfarWarps) {
    const uint64_t u0 = q * RW;
    const uint64_t ul = u0 + lane / LPF;
    Tc c[4] = {0, 0, 0, 0};
    if (ul < p.frames) cells4(p, ul, 4u * (lane % LPF), p.vec, c);
    Tc mx = c[0] > c[1] ? c[0] : c[1];
    mx = c[2] > mx ? c[2] : mx;
    mx = c[3] > mx ? c[3] : mx;
    bool narrow = !__any_sync(0xffffffffu, ((uint64_t)mx >> 32) != 0ull);
    if (narrow)
      narrow = (uint64_t)__reduce_max_sync(0xffffffffu, (unsigned)mx) * (p.rl + p.rg + 1u) <=
               0xFFFFFFFFull;
    if (narrow)
      packed_pass<NP, uint32_t>(p, c, u0, wbase, live, lo_b, hi_b, n_ok, det_w);
    else
      packed_pass<NP, uint64_t>(p, c, u0, wbase, live, lo_b, hi_b, n_ok, det_w);
    const uint64_t left = p.frames - u0;
    sup_w += (uint64_t)(p.n - n_ok) * (left < RW ? left : RW);  // every frame has its SUMMARY
  }
  if (lane == 0) {
    if (det_w) atomicAdd(&p.stats->cfar_det, det_w);
    if (sup_w) atomicAdd(&p.stats->cfar_sup, sup_w);
  }
}

// The k-th emitted cell of frame u re-decided from the cells themselves (the
// window sums added up directly: the same integers as the prefix
// differences), for frames with more events than their slots.
__device__ uint4 redecide(const CfarParams& p, uint64_t u, unsigned k) {
  const unsigned words = (p.n + 31u) / 32u;
  unsigned i = 0;
  for (unsigned r = 0; r < words; ++r) {
    uint32_t m = p.mask[u * words + r];
    const unsigned c = __popc(m);
    if (k < c) {
      for (unsigned t = 0; t < k; ++t) m &= m - 1u;  // drop the k lower set bits
      i = r * 32u + (unsigned)(__ffs(m) - 1);
      break;
    }
    k -= c;
  }
  const uint64_t cut = cell_at(p, u, i);
  const long long hi = (long long)i + p.gl + p.rl;
  const long long lo = (long long)i - (long long)p.gg - (long long)p.rg;
  const bool ok = hi < (long long)p.n && lo >= 0;
  uint64_t sl = 0, sg = 0;
  if (ok) {
    for (unsigned j = 0; j < p.rl; ++j) sl += cell_at(p, u, i + p.gl + 1u + j);
    for (unsigned j = 0; j < p.rg; ++j) sg += cell_at(p, u, i - p.gg - p.rg + j);
  }
  // the decision on these sums (cfar_model.hpp:295-340)
  uint64_t sum;
  unsigned nref;
  if (p.go) {
    const bool lead = (sl * p.rg) >= (sg * p.rl);
    sum = lead ? sl : sg;
    nref = lead ? p.rl : p.rg;
  } else {
    sum = sl + sg;
    nref = p.rl + p.rg;
  }
  const bool usable = p.go ? (p.rl != 0u && p.rg != 0u) : (p.rl + p.rg) != 0u;
  const bool evaluable = ok && p.enable && usable;
  const bool detected = evaluable && ((cut * nref) << 8) > ((uint64_t)p.alpha * sum);
  return pack_detection(cut, i, detected ? 0u : (!evaluable ? 2u : 1u), evaluable ? sum : 0ull,
                        evaluable ? nref : 0u);
}

// Event j of an emit CTA (frame f of the CTA, its k-th event): the SUMMARY
// from the frame's counts, a detection from the frame's slot (or
// re-decided); the event goes straight out, its packet to `pkt`.
template <unsigned PW, unsigned EF>
__device__ __forceinline__ void emit_one(const CfarParams& p, unsigned long long j,
                                         unsigned long long base, unsigned long long seq0,
                                         size_t pk, uint64_t f0, const unsigned long long* s_fbase,
                                         const unsigned* s_c, uint32_t* pkt) {
  unsigned f = 0;  // the frame holding event j: s_fbase[f] <= j < s_fbase[f + 1]
#pragma unroll
  for (unsigned step = EF / 2; step > 0; step >>= 1)
    if (s_fbase[f + step] <= j) f += step;
  const unsigned k = (unsigned)(j - s_fbase[f]), c = s_c[f];
  const uint64_t u = f0 + f;
  const unsigned u32 = (unsigned)u;  // u < frames < 2^32: 32-bit division
  const unsigned fq = u32 / p.beams;
  const uint64_t frame = p.frame_ids ? p.frame_ids[u] : (p.g0 + fq);
  const unsigned fid = p.frame_ids ? p.frame_ids[u] : (unsigned)(frame & 0xFFFFu);
  const uint16_t beam = (uint16_t)(p.frame_ids ? u32 : (u32 - fq * p.beams));
  const uint64_t idx = base + j;
  if (idx >= p.cap) return;
  rd_event ev;
  if (k + 1u == c) {  // the SUMMARY
    const uint32_t ds = p.detsup[u];
    make_event(&ev, 3u, p.n, fid, 0, p.alpha, ds & 0xFFFFu, ds >> 16, 0, 0, c == 1u, true,
               (uint32_t)frame, beam);
  } else {
    const uint4 e = c - 1u <= kCfarSlots ? p.slots[u * kCfarSlots + k] : redecide(p, u, k);
    const uint64_t cut = (uint64_t)e.x | ((uint64_t)(e.y & 0xFFu) << 32);
    const uint64_t sum = (uint64_t)e.z | ((uint64_t)(e.w & 0x7FFFu) << 32);
    make_event(&ev, e.y >> 24, (e.y >> 8) & 0xFFFFu, fid, (e.w >> 15) & 0x7Fu, p.alpha, 0, 0,
               cut, sum, k == 0u, false, (uint32_t)frame, beam);
  }
  store_event(p.events + idx, ev, p.ev16);
  if (p.flits)
    write_packet_w<PW>(ev, pkt, p.packet_w, p.flit_words, p.nfl, p.src_id, p.dest, p.vc,
                 (unsigned)((seq0 + idx) & 0xFFFFu));
}

// EF frames a CTA: 32, or 256 for frames of at most 64 cells (a frame then
// holds an event or two, and 32 frames would leave most threads idle).
template <unsigned PW, unsigned EF>
__global__ void __launch_bounds__(kCfarWarps * 32) k_cfar_emit(CfarParams p) {
  static_assert(EF % 32u == 0 && EF <= kCfarWarps * 32u, "whole warps of frames, a CTA's at most");
  __shared__ unsigned long long s_part[kCfarWarps], s_wtot[kCfarWarps], s_base, s_fbase[EF + 1];
  __shared__ unsigned s_c[EF];
  const unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u, tid = threadIdx.x;
  const uint64_t f0 = (uint64_t)blockIdx.x * EF;
  // events before this CTA: the launch's base, the totals of the 64-group
  // blocks before its first group's block and of that block's groups before
  // it (read in parallel; G / 128 + 32 words a CTA on average); and this
  // CTA's frames' counts with their exclusive scan (a warp per 32 frames) -
  // both behind one barrier
  {
    const uint64_t g = f0 / kCfarWarps, blk = g / kCfarBlock, groups = cfar_groups(p.frames);
    unsigned long long part = 0;
    for (uint64_t i = tid; i < blk; i += blockDim.x) part += p.totals[groups + i];
    for (uint64_t i = blk * kCfarBlock + tid; i < g; i += blockDim.x) part += p.totals[i];
    part = warp_sum64(part);
    if (lane == 0) s_part[warp] = part;
  }
  if (warp < EF / 32u) {
    const unsigned fl = warp * 32u + lane;
    const unsigned c = f0 + fl < p.frames ? p.counts[f0 + fl] : 0u;
    s_c[fl] = c;
    unsigned long long x = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, x, o);
      if ((int)lane >= o) x += t;
    }
    s_fbase[fl] = x - c;
    if (lane == 31) s_wtot[warp] = x;
  }
  __syncthreads();
  {
    unsigned long long add = 0, all = 0;
#pragma unroll
    for (unsigned w = 0; w < EF / 32u; ++w) {
      add += w < warp ? s_wtot[w] : 0ull;
      all += s_wtot[w];
    }
    if (tid < EF) s_fbase[tid] += add;  // a frame a thread
    if (tid == 0) {
      unsigned long long b = p.stats->scan_scratch[1];
#pragma unroll
      for (unsigned w = 0; w < kCfarWarps; ++w) b += s_part[w];
      s_base = b;
      s_fbase[EF] = all;
    }
  }
  __syncthreads();
  const unsigned long long base = s_base;
  const unsigned long long total = s_fbase[EF];
  if (blockIdx.x == gridDim.x - 1 && tid == 0)  // the launch's last frame is here
    p.stats->events_call = base + total;
  const unsigned long long seq0 = p.stats->events_total;
  const size_t pk = (size_t)p.nfl * p.flit_words;  // words per packet
  // one event a thread, in output order; the round's packets are built in
  // shared memory and leave as one contiguous, coalesced run
  extern __shared__ uint32_t s_pk[];
  for (unsigned long long j0 = 0; j0 < total; j0 += blockDim.x) {
    const unsigned long long j = j0 + tid;
    const unsigned long long end = base + (total < j0 + blockDim.x ? total : j0 + blockDim.x);
    const unsigned long long stop = end < p.cap ? end : p.cap;  // events of the round kept
    if (j < total)
      emit_one<PW, EF>(p, j, base, seq0, pk, f0, s_fbase, s_c, s_pk + (size_t)tid * pk);
    __syncthreads();
    if (p.flits && stop > base + j0) {
      const size_t nw = (size_t)(stop - (base + j0)) * pk;
      uint32_t* dst = p.flits + (size_t)(base + j0) * pk;
      for (size_t w = tid; w < nw; w += blockDim.x) dst[w] = s_pk[w];
    }
    __syncthreads();
  }
}

// Decide: 8 frames x (n + 2) words of shared memory; n <= 1024 needs the
// opt-in above 48 KB, set once per instantiation and device. One wave of
// persistent CTAs (as many as fit an SM, times the SMs), the group totals
// zeroed first.
// CTAs of `kernel` an SM at `sm` bytes of dynamic shared memory, and the
// device's SM count; the occupancy answer is kept per device and shared
// memory size in `memo` (one word per device: sm << 8 | CTAs).
template <class K>
static void decide_fit(K kernel, size_t sm, std::atomic<unsigned long long>* memo, int& per_sm,
                       int& n_sm) {
  int dev = 0;
  per_sm = n_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n_sm = 0;
    return;
  }
  const unsigned long long m = dev >= 0 && dev < 64 ? memo[dev].load(std::memory_order_relaxed) : 0ull;
  if (m && (m >> 8) == (unsigned long long)sm) {
    per_sm = (int)(m & 0xFFull);
    return;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kCfarWarps * 32, sm) !=
      cudaSuccess) {
    cudaGetLastError();
    per_sm = 0;
    return;
  }
  if (dev >= 0 && dev < 64 && per_sm > 0 && per_sm < 256)
    memo[dev].store(((unsigned long long)sm << 8) | (unsigned)per_sm, std::memory_order_relaxed);
}

// The decide grid: one wave (as many CTAs as fit), at most one per `work` unit.
static unsigned decide_grid(unsigned work, int per_sm, int n_sm) {
  const unsigned wave = n_sm > 0 && per_sm > 0 ? (unsigned)(n_sm * per_sm) : work;
  return std::max(1u, std::min(work, wave));
}

template <int R, class Tc>
static void launch_decide(const CfarParams& p, size_t sm, unsigned tiles, cudaStream_t s) {
  static PerDevice attr;
  attr.once([] {
    const int most = (int)((size_t)kCfarWarps * (128u * R + 2u) * sizeof(uint64_t));
    cudaFuncSetAttribute(k_cfar_decide<R, Tc>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  });
  static std::atomic<unsigned long long> memo[64];
  int per_sm, n_sm;
  decide_fit(k_cfar_decide<R, Tc>, sm, memo, per_sm, n_sm);
  const unsigned grid = decide_grid((unsigned)cfar_groups(p.frames), per_sm, n_sm);
  cudaMemsetAsync(p.totals, 0, (size_t)tiles * sizeof(unsigned long long), s);
  k_cfar_decide<R, Tc><<<grid, kCfarWarps * 32, sm, s>>>(p);
}

template <int R>
static void launch_decide_r(const CfarParams& p, cudaStream_t s) {
  const size_t sm = (size_t)kCfarWarps * (p.n + 2u) * sizeof(uint64_t);
  const unsigned tiles = cfar_tiles(p.frames);
  if (p.power_u32)
    launch_decide<R, uint32_t>(p, sm, tiles, s);
  else
    launch_decide<R, uint64_t>(p, sm, tiles, s);
}

// Frames of at most 64 cells: 128 / NP frames a warp pass, persistent as above.
template <int NP, class Tc>
static void launch_decide_packed(const CfarParams& p, cudaStream_t s) {
  const unsigned tiles = cfar_tiles(p.frames);
  static std::atomic<unsigned long long> memo[64];
  int per_sm, n_sm;
  decide_fit(k_cfar_decide_packed<NP, Tc>, 0, memo, per_sm, n_sm);
  const uint64_t passes = ((uint64_t)p.frames + 128u / NP - 1u) / (128u / NP);
  const unsigned grid =
      decide_grid((unsigned)((passes + kCfarWarps - 1u) / kCfarWarps), per_sm, n_sm);
  cudaMemsetAsync(p.totals, 0, (size_t)tiles * sizeof(unsigned long long), s);
  k_cfar_decide_packed<NP, Tc><<<grid, kCfarWarps * 32, 0, s>>>(p);
}

template <int NP>
static void launch_decide_np(const CfarParams& p, cudaStream_t s) {
  if (p.power_u32)
    launch_decide_packed<NP, uint32_t>(p, s);
  else
    launch_decide_packed<NP, uint64_t>(p, s);
}

unsigned cfar_tiles(uint32_t frames) {
  const uint64_t g = cfar_groups(frames);
  return (unsigned)(g + (g + kCfarBlock - 1u) / kCfarBlock);
}

template <unsigned EF>
static void launch_emit(const CfarParams& p, cudaStream_t s) {
  const unsigned emits = (unsigned)((p.frames + EF - 1u) / EF);
  const size_t esm = (size_t)kCfarWarps * 32 * p.nfl * p.flit_words * 4;
  switch (p.packet_w) {  // the common widths with their word layout fixed
    case 64: k_cfar_emit<64, EF><<<emits, kCfarWarps * 32, esm, s>>>(p); break;
    case 128: k_cfar_emit<128, EF><<<emits, kCfarWarps * 32, esm, s>>>(p); break;
    case 256: k_cfar_emit<256, EF><<<emits, kCfarWarps * 32, esm, s>>>(p); break;
    case 512: k_cfar_emit<512, EF><<<emits, kCfarWarps * 32, esm, s>>>(p); break;
    default: k_cfar_emit<0, EF><<<emits, kCfarWarps * 32, esm, s>>>(p); break;
  }
}

void launch_cfar(const CfarParams& p, cudaStream_t s) {
  if (!p.frames) return;
  const unsigned rows = (p.n + 127u) / 128u;
  if (p.n >= 1u && p.n <= 16u) launch_decide_np<16>(p, s);
  else if (p.n >= 1u && p.n <= 32u) launch_decide_np<32>(p, s);
  else if (p.n >= 1u && p.n <= 64u) launch_decide_np<64>(p, s);
  else if (rows <= 1) launch_decide_r<1>(p, s);
  else if (rows <= 2) launch_decide_r<2>(p, s);
  else if (rows <= 4) launch_decide_r<4>(p, s);
  else launch_decide_r<8>(p, s);
  if (p.n <= 64u)
    launch_emit<kCfarWarps * 32u>(p, s);
  else
    launch_emit<kEmitFrames>(p, s);
}

// ---------------------------------------------------------------------------
// Per-block entry points
// ---------------------------------------------------------------------------
__global__ void k_bf_block(uint32_t A, uint32_t B, const uint32_t* w, const uint32_t* x,
                           uint64_t nv, uint32_t* y, long long* acc, uint8_t* flags) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nv * B) return;
  const uint64_t v = i / B;
  const uint32_t b = (uint32_t)(i % B);
  long long ar = 0, ai = 0;
  for (uint32_t a = 0; a < A; ++a) {
    const cplx xv = unpack(x[v * A + a]), wv = unpack(w[(size_t)b * A + a]);
    ar += cmul_re_raw(xv, wv);
    ai += cmul_im_raw(xv, wv);
  }
  unsigned fr = 0, fi = 0;
  const int32_t yr = q15_out64(ar, &fr), yi = q15_out64(ai, &fi);
  y[i] = pack2(yr, yi);
  if (acc) {
    acc[2 * i] = ar;
    acc[2 * i + 1] = ai;
  }
  if (flags) flags[i] = (uint8_t)((fr << 2) | fi);
}
void launch_bf_block(uint32_t n_ant, uint32_t n_beams, const uint32_t* w, const uint32_t* x,
                     uint64_t n_vec, uint32_t* y, long long* acc, uint8_t* flags, cudaStream_t s) {
  const uint64_t n = n_vec * n_beams;
  if (n) k_bf_block<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n_ant, n_beams, w, x, n_vec, y,
                                                                 acc, flags);
}

__global__ void k_power_block(const uint32_t* x, uint64_t n, long long* p) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = (long long)power_u32(unpack(x[i]));
}
void launch_power_block(const uint32_t* x, uint64_t n, long long* p, cudaStream_t s) {
  if (n) k_power_block<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, n, p);
}

__global__ void k_cross_block(const uint32_t* x, const uint32_t* y, uint64_t n, long long* c) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx X = unpack(x[i]), Y = unpack(y[i]);
  const cplx b = {Y.im, Y.re};
  c[2 * i] = cmul_im_raw(X, b);
  c[2 * i + 1] = neg_wrap(cmul_re_raw(X, b));
}
void launch_cross_block(const uint32_t* x, const uint32_t* y, uint64_t n, long long* c,
                        cudaStream_t s) {
  if (n) k_cross_block<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, y, n, c);
}

__global__ void k_packetize(const rd_event* ev, uint64_t n, uint32_t pw, uint32_t src,
                            uint32_t dest, uint32_t vc, uint32_t seq0, uint32_t* flits,
                            uint32_t words, uint32_t nfl) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const rd_event e = ev[i];
  write_packet(e, flits + i * nfl * words, pw, words, nfl, src, dest, vc,
               (unsigned)((seq0 + i) & 0xFFFFu));
}
void launch_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w, uint32_t src,
                      uint32_t dest, uint32_t vc, uint32_t seq0, uint32_t* flits, cudaStream_t s) {
  const uint32_t words = (packet_w + 5u + 31u) / 32u;
  const uint32_t nfl = 1u + (176u + packet_w - 1u) / packet_w;
  if (n) k_packetize<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(ev, n, packet_w, src, dest, vc,
                                                                  seq0, flits, words, nfl);
}

__device__ __forceinline__ unsigned growth_bits(unsigned n) {
  return n <= 1u ? 0u : 32u - __clz(n - 1u);
}

// fxp_ops.hpp:109-177 dispatch over the device primitives
__global__ void k_fxp(const uint32_t* op, const int64_t* a, const int64_t* b, const uint32_t* sh,
                      const uint32_t* wv, uint64_t n, int64_t* y, uint8_t* flags) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long A = a[i], Bv = b[i];
  const unsigned S = sh[i], W = wv[i];
  long long r = 0;
  unsigned f = 0;
  switch (op[i]) {
    case RD_OP_SAT: r = sat64(A, W); f = sat_flags64(A, W); break;
    case RD_OP_TRUNC: r = asr64(A, S); break;
    case RD_OP_ROUND_EVEN:
    case RD_OP_ROUND: r = round_even64(A, S); break;
    case RD_OP_ROUND_HALF_UP: r = round_half_up64(A, S); break;
    case RD_OP_ROUND_SAT: {
      const long long q = round_even64(A, S);
      r = sat64(q, W);
      f = sat_flags64(q, W);
      break;
    }
    case RD_OP_ADD_SAT: r = sat64(add_wrap(A, Bv), W); f = sat_flags64(add_wrap(A, Bv), W); break;
    case RD_OP_SUB_SAT: r = sat64(sub_wrap(A, Bv), W); f = sat_flags64(sub_wrap(A, Bv), W); break;
    case RD_OP_NEG_SAT: r = sat64(neg_wrap(A), W); f = sat_flags64(neg_wrap(A), W); break;
    case RD_OP_MUL_Q15:
      r = (long long)((int32_t)(int16_t)(uint16_t)(A & 0xFFFF) * (int16_t)(uint16_t)(Bv & 0xFFFF));
      break;
    case RD_OP_MUL_Q15_RS: {
      const int32_t pr = (int32_t)(int16_t)(uint16_t)(A & 0xFFFF) * (int16_t)(uint16_t)(Bv & 0xFFFF);
      const int32_t q = rne15_32(pr);
      r = sat16(q);
      f = flags16(q);
      break;
    }
    case RD_OP_CMUL_RE:
    case RD_OP_CMUL_IM: {
      const cplx ca = unpack((uint32_t)(A & 0xFFFFFFFFll)), cb = unpack((uint32_t)(Bv & 0xFFFFFFFFll));
      unsigned fl = 0;
      const cplx o = cmul_q15(ca, cb, &fl);
      // flags of the selected component only
      const long long raw = op[i] == RD_OP_CMUL_RE ? cmul_re_raw(ca, cb) : cmul_im_raw(ca, cb);
      const long long q = rne15_64(raw);
      f = (q > 32767 ? 2u : 0u) | (q < -32768 ? 1u : 0u);
      r = op[i] == RD_OP_CMUL_RE ? o.re : o.im;
      break;
    }
    case RD_OP_ACC_W: r = (long long)(W + growth_bits((uint32_t)(A & 0xFFFFFFFFll))); break;
    case RD_OP_GROWTH_BITS: r = (long long)growth_bits((uint32_t)(A & 0xFFFFFFFFll)); break;
    default: r = 0; break;
  }
  y[i] = r;
  flags[i] = (uint8_t)f;
}
void launch_fxp(const uint32_t* op, const int64_t* a, const int64_t* b, const uint32_t* sh,
                const uint32_t* w, uint64_t n, int64_t* y, uint8_t* flags, cudaStream_t s) {
  if (n) k_fxp<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, a, b, sh, w, n, y, flags);
}

}  // namespace rd
