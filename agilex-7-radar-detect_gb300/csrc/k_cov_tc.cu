// k_cov_tc.cu - the exact block-mode covariance on the tensor cores.
//
// covar::cross_power (covar_model.hpp:119-151) gives, per pair (x, y) and
// frame, R = X conj(Y): re = xr yr + xi yi, im = xi yr - xr yi; the block
// Integrator (covar_model.hpp:204-262) sums it over a window. When no sum can
// saturate (the condition launch_cov states) the window sum is a plain
// integer sum, and for one bin it is a Gram matrix over the window's frames:
//
//   G[x][y] = sum_f X_f[x] conj(X_f[y]),
//
// a GEMM with M = x channels, N = y channels x 6 scale classes, K = frames x
// 4 limb parts. With x = 256 xh + xl (xh in [-128, 127], xl in [0, 255]),
//
//   re: class 16 = xrh yrh + xih yih           im: xih yrh - xrh yih
//       class 8  = xrh yrl + xrl yrh               xih yrl + xil yrh
//                + xih yil + xil yih               - xrh yil - xrl yih
//       class 0  = xrl yrl + xil yil               xil yrl - xrl yil
//
// and per frame every class is at most 4 terms of magnitude <= 128 * 255, so
// over 128 frames every partial sum is an integer below 2^24, exact in the
// fp32 accumulators. The kernel folds them into int64 every 128 frames and at
// the window's end - giving the integers the Integrator adds.
//
// A operand, row x, k = 4f + part: the (re, im) high-limb word of X_f[x] for
// parts 0-1 and the low-limb word for parts 2-3. B operand, column (y, class):
// for parts 0-1 / 2-3 respectively,
//   re16: hi / 0     re8: lo / hi      re0: 0 / lo
//   im16: ns(hi) / 0 im8: ns(lo) / ns(hi)  im0: 0 / ns(lo)
// with ns(a, b) = (-b, a). Three m16n8 tiles cover four y channels, column
// 2t + e of tile j being class 2j + e of channel t (the layout of the tensor
// beamformer), so after the three tiles the accumulator lane with columns
// 2t, 2t+1 holds all six classes of (x, y) for its two x rows. A lane with
// e = g & 1 (its column's class parity) and h = tg & 1 (parts 0-1 or 2-3)
// takes, for tiles 0, 1, 2:
//   (h, e) = (0, 0) and (1, 1): hi, 0, ns(lo)     (0, 1): lo, ns(hi), 0
//   (h, e) = (1, 0):            0, lo, ns(hi)
// The staging writes these three word triples per (frame, channel), so a
// lane's B fragment for all three tiles is one 16-byte load per k half.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "rd_internal.h"
#include "tc.cuh"

namespace rd {

constexpr unsigned kCtFrames = 16u;  // frames per staged chunk
constexpr unsigned kCtLog2 = 4u;     // log2 kCtFrames
constexpr unsigned kCtFold = 8u;     // chunks per fp32 accumulation: 128 frames
constexpr unsigned kCtPre = 8u;      // staged elements per thread per chunk (NB Sp <= 128)

template <int UPW>
__global__ void __launch_bounds__(256, 2) k_cov_tc(CovParams p, CovTcPlan t) {
  extern __shared__ __align__(16) uint32_t sm[];
  const unsigned S = p.S, Sp = t.Sp, NB = t.NB, lsp = t.log2_sp;
  // frame strides (words); FSB = 16 mod 32 keeps the two frames of a B load
  // on different banks
  const unsigned FSA = 2u * Sp + 16u, FSB = 12u * Sp + 16u;
  uint32_t* sA = sm;                                       // [NB][16][FSA]
  uint32_t* sB = sA + NB * kCtFrames * FSA;                // [NB][16][FSB]
  long long* sAcc = reinterpret_cast<long long*>(sB + NB * kCtFrames * FSB);  // [8][UPW][32][4]
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const unsigned g = lane >> 2, tg = lane & 3u;
  const unsigned bin0 = blockIdx.x * NB;
  // this CTA's frames: the open window, one whole window, or the trailing part
  const unsigned z = blockIdx.z, nz = gridDim.z;
  const unsigned first = p.wl - p.count0;
  const unsigned lo = z == 0 ? 0u : first + (z - 1u) * p.wl;
  const unsigned hi_ = z == 0 ? first : first + z * p.wl;
  const unsigned hi = (nz == 1u || hi_ > p.F) ? p.F : hi_;

  uint32_t unit[UPW];
#pragma unroll
  for (int u = 0; u < UPW; ++u) unit[u] = t.units[(blockIdx.y * 8u + warp) * UPW + u];
  float d[UPW][3][4];
#pragma unroll
  for (int u = 0; u < UPW; ++u)
#pragma unroll
    for (int j = 0; j < 3; ++j) d[u][j][0] = d[u][j][1] = d[u][j][2] = d[u][j][3] = 0.f;
  long long* acc = sAcc + ((size_t)warp * UPW * 32u + lane) * 4u;  // + u * 128
#pragma unroll
  for (int u = 0; u < UPW; ++u)
    for (int e = 0; e < 4; ++e) acc[u * 128 + e] = 0;

  // this lane's B word triple (see the header comment): 0 for (h, e) = (0, 0)
  // and (1, 1), 1 for (0, 1), 2 for (1, 0)
  const unsigned bslot = ((g ^ tg) & 1u) == 0u ? 0u : ((tg & 1u) == 0u ? 1u : 2u);

  const unsigned per_chunk = (NB * kCtFrames) << lsp;
  uint32_t pre[kCtPre];
  auto load = [&](unsigned f0) {
#pragma unroll
    for (unsigned j = 0; j < kCtPre; ++j) {
      const unsigned e = tid + j * 256u;
      uint32_t v = 0;
      if (e < per_chunk) {
        const unsigned c = e & (Sp - 1u), r = e >> lsp;
        const unsigned f = f0 + (r & (kCtFrames - 1u)), bin = bin0 + (r >> kCtLog2);
        if (f < hi && bin < p.N && c < S) {
          if (p.src_beam) {
            v = __ldg(p.beams_bn + ((size_t)f * p.N + bin) * S + c);
          } else {
            unsigned slot = p.ring_base + f;
            if (slot >= p.ring_frames) slot -= p.ring_frames;
            v = __ldg(p.ring + ((size_t)slot * p.N + bin) * S + c);
          }
        }
      }
      pre[j] = v;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (unsigned j = 0; j < kCtPre; ++j) {
      const unsigned e = tid + j * 256u;
      if (e < per_chunk) {
        const unsigned c = e & (Sp - 1u), r = e >> lsp;  // r = bl * 16 + frame
        uint32_t h, l;
        limb_words(pre[j], h, l);
        *reinterpret_cast<uint2*>(sA + r * FSA + 2u * c) = make_uint2(h, l);
        const uint32_t nl = negswap(l), nh = negswap(h);
        uint4* b = reinterpret_cast<uint4*>(sB + r * FSB + 12u * c);
        b[0] = make_uint4(h, 0u, nl, 0u);
        b[1] = make_uint4(l, nh, 0u, 0u);
        b[2] = make_uint4(0u, l, nh, 0u);
      }
    }
  };
  auto fold = [&]() {
#pragma unroll
    for (int u = 0; u < UPW; ++u) {
      if (unit[u] != ~0u) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          acc[u * 128 + 2 * h] += fold3(d[u][0][2 * h], d[u][0][2 * h + 1], d[u][1][2 * h]);
          acc[u * 128 + 2 * h + 1] +=
              fold3(d[u][1][2 * h + 1], d[u][2][2 * h], d[u][2][2 * h + 1]);
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) d[u][j][0] = d[u][j][1] = d[u][j][2] = d[u][j][3] = 0.f;
    }
  };

  const unsigned nch = (hi - lo + kCtFrames - 1u) / kCtFrames;
  if (nch) load(lo);
  for (unsigned ci = 0; ci < nch; ++ci) {
    __syncthreads();  // the previous chunk is consumed
    store();
    __syncthreads();
    if (ci + 1u < nch) load(lo + (ci + 1u) * kCtFrames);
#pragma unroll 1
    for (unsigned kk = 0; kk < kCtFrames / 4u; ++kk) {
      uint32_t b00 = 0, b01 = 0, b02 = 0, b10 = 0, b11 = 0, b12 = 0;
#pragma unroll
      for (int u = 0; u < UPW; ++u) {
        const uint32_t un = unit[u];
        if (un == ~0u) continue;
        const unsigned bl = un >> 16, mi = (un >> 8) & 255u, tri = un & 255u;
        const unsigned fr = bl * kCtFrames + 4u * kk + (tg >> 1);  // frame of k = 2 tg
        const uint32_t* pa = sA + fr * FSA + 2u * (16u * mi + g) + (tg & 1u);
        const uint32_t a[4] = {pa[0], pa[16], pa[2u * FSA], pa[2u * FSA + 16u]};
        if (u == 0 || ((un ^ unit[u > 0 ? u - 1 : 0]) & 0xFFFF00FFu) != 0u) {
          const uint32_t* pb = sB + fr * FSB + 12u * (4u * tri + (g >> 1)) + 4u * bslot;
          const uint4 w0 = *reinterpret_cast<const uint4*>(pb);
          const uint4 w1 = *reinterpret_cast<const uint4*>(pb + 2u * FSB);
          b00 = w0.x;
          b01 = w0.y;
          b02 = w0.z;
          b10 = w1.x;
          b11 = w1.y;
          b12 = w1.z;
        }
        mma_f16(d[u][0], a, b00, b10);
        mma_f16(d[u][1], a, b01, b11);
        mma_f16(d[u][2], a, b02, b12);
      }
    }
    if ((ci + 1u) % kCtFold == 0u || ci + 1u == nch) fold();
  }

  // window close / carry (the Integrator's block mode, as k_cov does it)
  const bool carry_in = z == 0u, carry_out = z + 1u == nz;
  const bool closes = z < p.n_windows;
#pragma unroll
  for (int u = 0; u < UPW; ++u) {
    const uint32_t un = unit[u];
    if (un == ~0u) continue;
    const unsigned bin = bin0 + (un >> 16), mi = (un >> 8) & 255u, tri = un & 255u;
    if (bin >= p.N) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const unsigned x = 16u * mi + g + 8u * (unsigned)h, y = 4u * tri + tg;
      if (x >= S || y >= S) continue;
      const int q = t.pq[x * S + y];
      if (q < 0) continue;
      long long re = acc[u * 128 + 2 * h], im = acc[u * 128 + 2 * h + 1];
      const size_t k = (size_t)bin * p.P + (unsigned)q;
      if (carry_in) {
        re += p.acc_re[k];
        im += p.acc_im[k];
      }
      if (closes) {
        long long* o = p.out + (((size_t)z * p.N + bin) * p.P + (unsigned)q) * 2;
        o[0] = re;
        o[1] = im;
        re = im = 0;
      }
      if (carry_out) {
        p.acc_re_out[k] = re;
        p.acc_im_out[k] = im;
      }
    }
  }
}

bool cov_tc_plan(uint32_t S, const uint32_t* px, const uint32_t* py, uint32_t P,
                 CovTcHost* out) {
  if (S == 0 || S > 128u || P == 0) return false;
  out->pq.assign((size_t)S * S, -1);
  std::vector<uint32_t> need;  // tri << 8 | mi
  for (uint32_t q = 0; q < P; ++q) {
    const size_t k = (size_t)px[q] * S + py[q];
    if (px[q] >= S || py[q] >= S || out->pq[k] >= 0) return false;  // a repeated pair
    out->pq[k] = (int32_t)q;
    need.push_back((py[q] / 4u) << 8 | (px[q] / 16u));
  }
  std::sort(need.begin(), need.end());
  need.erase(std::unique(need.begin(), need.end()), need.end());
  uint32_t sp = 16, lsp = 4;
  while (sp < S) sp *= 2, ++lsp;
  const uint32_t U1 = (uint32_t)need.size();
  uint32_t NB = std::max(1u, (16u + U1 - 1u) / U1);
  NB = std::min(NB, std::max(1u, 64u / sp));
  const uint32_t U = NB * U1;
  const uint32_t G = (U + 39u) / 40u, UPW = (U + 8u * G - 1u) / (8u * G);
  out->units.assign((size_t)G * 8u * UPW, ~0u);
  for (uint32_t i = 0; i < U; ++i) {  // sorted by (bin, triple, m-tile): B reuse in a warp
    const uint32_t bl = i / U1, tm = need[i % U1];
    out->units[i] = bl << 16 | (tm & 255u) << 8 | (tm >> 8);
  }
  out->plan.Sp = sp;
  out->plan.log2_sp = lsp;
  out->plan.NB = NB;
  out->plan.UPW = UPW;
  out->plan.G = G;
  return true;
}

size_t cov_tc_smem(const CovTcPlan& t) {
  const size_t fs = (2u * t.Sp + 16u) + (12u * t.Sp + 16u);
  return (size_t)t.NB * kCtFrames * fs * 4u + (size_t)8u * t.UPW * 32u * 4u * 8u;
}

static std::atomic<bool> g_ct_attr[64];

template <int UPW>
static void launch_ct(const CovParams& p, const CovTcPlan& t, dim3 grid, size_t smem,
                      cudaStream_t s) {
  k_cov_tc<UPW><<<grid, 256, smem, s>>>(p, t);
}

void launch_cov_tc(const CovParams& p, const CovTcPlan& t, cudaStream_t s) {
  if (p.P == 0 || p.F == 0) return;
  const unsigned first = p.wl - p.count0;
  const unsigned nz = first >= p.F ? 1u : 1u + (p.F - first + p.wl - 1u) / p.wl;
  const dim3 grid((p.N + t.NB - 1u) / t.NB, t.G, nz);
  const size_t smem = cov_tc_smem(t);
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !g_ct_attr[dev].load()) {
    const int mx = 200 * 1024;
    cudaFuncSetAttribute(k_cov_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_cov_tc<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_cov_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_cov_tc<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_cov_tc<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (dev >= 0 && dev < 64) g_ct_attr[dev].store(true);
  }
  switch (t.UPW) {
    case 1: launch_ct<1>(p, t, grid, smem, s); break;
    case 2: launch_ct<2>(p, t, grid, smem, s); break;
    case 3: launch_ct<3>(p, t, grid, smem, s); break;
    case 4: launch_ct<4>(p, t, grid, smem, s); break;
    default: launch_ct<5>(p, t, grid, smem, s); break;
  }
}

}  // namespace rd
