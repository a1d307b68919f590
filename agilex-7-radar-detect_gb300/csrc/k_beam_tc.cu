// k_beam_tc.cu - beamforming on the tensor cores, exact.
//
// Y[r][b] = sum_a X[r][a] W[b][a] (bf::dot, beamformer_model.hpp:162-179) as a
// real fp16 GEMM with fp32 accumulation that is exact by construction:
//
//   x = 256 xh + xl,  w = 256 wh + wl,  xh, wh in [-128, 127], xl, wl in [0, 255]
//
// every limb is an integer of magnitude <= 256, exact in fp16; every product
// is an integer of magnitude < 2^16, exact in fp32; and the three scale
// classes of the complex product
//
//   class 16: xh*wh          class 8: xh*wl + xl*wh          class 0: xl*wl
//
// each sum at most 4 C terms of magnitude <= 128 * 255, which for C <= 128 is
// below 2^24: every partial sum the tensor core forms, in any order, is an
// integer that fp32 holds exactly. The epilogue recombines
// acc = 2^16 c16 + 2^8 c8 + c0 in int64 - the integer bf::dot sums - then
// round_sat and covar::power (covar_model.hpp:99-102).
//
// GEMM: rows r = (frame, bin) of the spectrum ring; K = 4 limb parts x C
// channels, k = 4a + {xre_hi, xim_hi, xre_lo, xim_lo}; N = 6 columns per beam
// {re16, re8, re0, im16, im8, im0}. Three m16n8 tiles cover four beams, laid
// out so that column 2t + e of tile j is class 2j + e of beam t: the lane of
// the accumulator fragment that holds columns 2t, 2t+1 then holds all six
// classes of beam t for its two rows after the three tiles, and every lane
// finishes two outputs without exchanging data. The weight matrix is built on
// the host in mma fragment order (set_weights). mma.sync m16n8k16 f16 -> f32.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "fxp.cuh"
#include "rd_internal.h"
#include "tc.cuh"

namespace rd {

constexpr unsigned kTcRows = 128u;  // rows per CTA: 8 warps x 16
constexpr unsigned kTcBeams = 16u;  // beams per group: 4 tile triples
constexpr unsigned kTcTiles = 12u;  // m16n8 tiles per group

// ---- host: weight operand -----------------------------------------------------
static int wlimb(const uint32_t* w, uint32_t C, uint32_t B, uint32_t b, uint32_t a, int part) {
  if (b >= B || a >= C) return 0;
  const uint32_t v = w[(size_t)b * C + a];
  const int re = (int16_t)(uint16_t)(v & 0xFFFFu), im = (int16_t)(uint16_t)(v >> 16);
  switch (part) {
    case 0: return re >> 8;    // wrh
    case 1: return im >> 8;    // wih
    case 2: return re & 255;   // wrl
    default: return im & 255;  // wil
  }
}

// W'[k = 4a + part][class] of beam b, class in {re16, re8, re0, im16, im8, im0}:
// re = xr wr - xi wi, im = xr wi + xi wr, split by limb scale.
static int wprime(const uint32_t* w, uint32_t C, uint32_t B, uint32_t b, uint32_t k, int cls) {
  const uint32_t a = k / 4;
  const int part = (int)(k % 4);  // 0 xrh, 1 xih, 2 xrl, 3 xil
  const int wrh = wlimb(w, C, B, b, a, 0), wih = wlimb(w, C, B, b, a, 1);
  const int wrl = wlimb(w, C, B, b, a, 2), wil = wlimb(w, C, B, b, a, 3);
  switch (cls) {
    case 0: return part == 0 ? wrh : part == 1 ? -wih : 0;                       // re16
    case 1: return part == 0 ? wrl : part == 1 ? -wil : part == 2 ? wrh : -wih;  // re8
    case 2: return part == 2 ? wrl : part == 3 ? -wil : 0;                       // re0
    case 3: return part == 0 ? wih : part == 1 ? wrh : 0;                        // im16
    case 4: return part == 0 ? wil : part == 1 ? wrl : part == 2 ? wih : wrh;    // im8
    default: return part == 2 ? wil : part == 3 ? wrl : 0;                       // im0
  }
}

// IEEE binary16 bits of an integer |v| <= 2048 (exact)
static uint16_t host_f16(int v) {
  if (v == 0) return 0;
  const unsigned sign = v < 0 ? 0x8000u : 0u;
  const unsigned m = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((m >> (e + 1)) != 0) ++e;  // m in [2^e, 2^(e+1))
  const unsigned mant = (m << (10 - e)) & 0x3FFu;
  return (uint16_t)(sign | (unsigned)(e + 15) << 10 | mant);
}

uint32_t beam_tc_fragment_words(uint32_t C, uint32_t B) {
  const uint32_t KS = (C + 3u) / 4u, G = (B + kTcBeams - 1u) / kTcBeams;
  return G * KS * kTcTiles * 64u;
}

// Fragment order: [group][k-step][tile j][lane] x 2 words. Lane (g', t') of
// tile j holds B[k = 2t' + {0,1}][n = g'] and B[k = 2t' + 8 + {0,1}][n = g'];
// column n of tile j (triple j / 3, sub-tile j % 3) is class 2 (j % 3) +
// (n & 1) of beam 16 group + 4 (j / 3) + (n >> 1).
void beam_tc_fragments(const uint32_t* w, uint32_t C, uint32_t B, uint32_t* out) {
  const uint32_t KS = (C + 3u) / 4u, G = (B + kTcBeams - 1u) / kTcBeams;
  for (uint32_t g = 0; g < G; ++g)
    for (uint32_t kk = 0; kk < KS; ++kk)
      for (uint32_t j = 0; j < kTcTiles; ++j)
        for (uint32_t l = 0; l < 32; ++l) {
          const uint32_t n = l >> 2, tig = l & 3;
          const uint32_t b = g * kTcBeams + (j / 3) * 4 + (n >> 1);
          const int cls = (int)(2 * (j % 3) + (n & 1));
          uint32_t* o = out + (((size_t)(g * KS + kk) * kTcTiles + j) * 64 + l * 2);
          for (int h = 0; h < 2; ++h) {
            const uint32_t k0 = kk * 16 + tig * 2 + (uint32_t)h * 8;
            const uint16_t lo = host_f16(wprime(w, C, B, b, k0, cls));
            const uint16_t hi = host_f16(wprime(w, C, B, b, k0 + 1, cls));
            o[h] = (uint32_t)lo | ((uint32_t)hi << 16);
          }
        }
}

// The products and the epilogue of one tile held in shared memory as limb
// words (row stride S, ks k16 steps): this lane's rows are rr0 and rr0 + 8 of
// the tile (global rows r0 + rr0, + 8; chunk frames f0, f1; bins bin0, bin1),
// each written only when valid (ok0, ok1).
__device__ __forceinline__ void tile_products(const BeamParams& p, const uint32_t* s_x, unsigned S,
                                              unsigned ks, uint64_t r0, unsigned rr0, bool ok0,
                                              bool ok1, unsigned f0, unsigned bin0, unsigned f1,
                                              unsigned bin1, unsigned& fl_any,
                                              unsigned long long& nsat) {
  const unsigned B = p.B, N = p.N;
  const unsigned lane = threadIdx.x & 31u, tig = lane & 3u;
  const uint32_t* xa0 = s_x + rr0 * S + tig;
  const uint32_t* xa1 = xa0 + 8u * S;
  const unsigned G = (B + kTcBeams - 1u) / kTcBeams;
  // output rows: beam b's power cell at pw + b N, its beam word at bn + b
  uint32_t* const pw0 = p.power ? p.power + ((uint64_t)f0 * B) * N + bin0 : nullptr;
  uint32_t* const pw1 = p.power ? p.power + ((uint64_t)f1 * B) * N + bin1 : nullptr;
  uint32_t* const bn0 = p.beams_bn ? p.beams_bn + ((uint64_t)f0 * N + bin0) * B : nullptr;
  uint32_t* const bn1 = p.beams_bn ? p.beams_bn + ((uint64_t)f1 * N + bin1) * B : nullptr;
  for (unsigned grp = 0; grp < G; ++grp) {
    float d[kTcTiles][4];
#pragma unroll
    for (int j = 0; j < (int)kTcTiles; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
    const uint2* wf = reinterpret_cast<const uint2*>(p.w_frag) +
                      (size_t)grp * ks * kTcTiles * 32u + lane;
#pragma unroll 1
    for (unsigned kk = 0; kk < ks; ++kk) {
      const uint32_t af[4] = {xa0[8u * kk], xa1[8u * kk], xa0[8u * kk + 4u], xa1[8u * kk + 4u]};
      const uint2* wk = wf + (size_t)kk * kTcTiles * 32u;
#pragma unroll
      for (int j = 0; j < (int)kTcTiles; ++j) {
        const uint2 bw = __ldg(wk + j * 32);
        mma_f16(d[j], af, bw.x, bw.y);
      }
    }
    // epilogue: lane t of each quad holds beam 4 t3 + t of the group for
    // rows g (h = 0) and g + 8 (h = 1). The fp32 estimate of a sum is off by
    // less than 2^8 + 2^-24 of itself, so a sum estimated below 1e9 in
    // magnitude is below 2^31 - 2^15: recombined modulo 2^32 it is exact, and
    // rounds in 32 bits
#pragma unroll
    for (int t3 = 0; t3 < 4; ++t3) {
      const unsigned b = grp * kTcBeams + (unsigned)t3 * 4u + tig;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float* c0 = d[3 * t3];
        const float* c1 = d[3 * t3 + 1];
        const float* c2 = d[3 * t3 + 2];
        const float cr16 = c0[2 * h], cr8 = c0[2 * h + 1], cr0 = c1[2 * h];
        const float ci16 = c1[2 * h + 1], ci8 = c2[2 * h], ci0 = c2[2 * h + 1];
        if (b < B && (h ? ok1 : ok0)) {
          unsigned fr = 0, fi = 0;
          long long re_v, im_v;
          int32_t yr, yi;
          const float est = fmaxf(fabsf(fmaf(cr16, 65536.f, fmaf(cr8, 256.f, cr0))),
                                  fabsf(fmaf(ci16, 65536.f, fmaf(ci8, 256.f, ci0))));
          if (est < 1.0e9f) {
            const int32_t re32 = (int32_t)((uint32_t)__float2int_rn(cr16) * 65536u +
                                           (uint32_t)__float2int_rn(cr8) * 256u +
                                           (uint32_t)__float2int_rn(cr0));
            const int32_t im32 = (int32_t)((uint32_t)__float2int_rn(ci16) * 65536u +
                                           (uint32_t)__float2int_rn(ci8) * 256u +
                                           (uint32_t)__float2int_rn(ci0));
            yr = q15_out32(re32, &fr);
            yi = q15_out32(im32, &fi);
            re_v = re32;
            im_v = im32;
          } else {
            re_v = fold3(cr16, cr8, cr0);
            im_v = fold3(ci16, ci8, ci0);
            yr = q15_out64(re_v, &fr);
            yi = q15_out64(im_v, &fi);
          }
          if (fr | fi) {
            fl_any |= fr | fi;
            ++nsat;
          }
          const uint32_t y = pack2(yr, yi);
          if (p.power) (h ? pw1 : pw0)[b * N] = power_u32(unpack(y));
          if (p.beams_bn) (h ? bn1 : bn0)[b] = y;
          const uint64_t r = r0 + rr0 + 8u * (unsigned)h;
          if (p.y_rows) p.y_rows[r * B + b] = y;
          if (p.acc_rows) {
            p.acc_rows[(r * B + b) * 2] = re_v;
            p.acc_rows[(r * B + b) * 2 + 1] = im_v;
          }
          if (p.flag_rows) p.flag_rows[r * B + b] = (uint8_t)((fr << 2) | fi);
        }
      }
    }
  }
}

// ---- device ---------------------------------------------------------------------
// One CTA: 128 rows of the ring, all beams in groups of 16. The rows are
// converted once into fp16 limb words in shared memory, row stride S = 8 ks
// + 4 words (ks = ceil(C / 4) k16 steps): word 2a of a row holds channel a's
// (re, im) high limbs and word 2a + 1 its low limbs, so the A fragment of
// k-step kk is words 8 kk + t and 8 kk + 4 + t, bank-conflict free.
__global__ void __launch_bounds__(256, 2) k_beam_tc(BeamParams p) {
  extern __shared__ __align__(16) uint32_t sm[];
  const unsigned C = p.C, N = p.N;
  const unsigned ks = (C + 3u) / 4u;
  const unsigned S = 8u * ks + 4u;
  uint32_t* s_x = sm;                                                      // [128][S]
  unsigned long long* s_off = reinterpret_cast<unsigned long long*>(sm + kTcRows * S);
  uint32_t* s_f = reinterpret_cast<uint32_t*>(s_off + kTcRows);            // chunk frame
  uint32_t* s_bin = s_f + kTcRows;
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const unsigned gid = lane >> 2;
  const uint64_t rows = (uint64_t)p.F * N;
  const uint64_t r0 = (uint64_t)blockIdx.x * kTcRows;

  if (tid < kTcRows) {
    const uint64_t r = r0 + tid;
    unsigned long long off = ~0ull;
    unsigned f = 0, bin = 0;
    if (r < rows) {
      f = (unsigned)(r / N);
      bin = (unsigned)(r - (uint64_t)f * N);
      unsigned slot = p.ring_base + f;
      if (slot >= p.ring_frames) slot -= p.ring_frames;
      off = ((unsigned long long)slot * N + bin) * C;
    }
    s_off[tid] = off;
    s_f[tid] = f;
    s_bin[tid] = bin;
  }
  __syncthreads();
  // stage: 4 channels per item (channels >= C and rows >= rows read as 0,
  // whose limbs are 0). With C a multiple of 4, every thread issues eight
  // quad loads, then converts them, so the loads overlap instead of each
  // waiting on the last
  const bool vec = (C & 3u) == 0u;
  constexpr unsigned kBatch = 8u;  // quads in flight per thread
  for (unsigned k0 = 0; vec && k0 < kTcRows * ks; k0 += kBatch * 256u) {
    uint4 t[kBatch];
#pragma unroll
    for (unsigned q = 0; q < kBatch; ++q) {
      const unsigned k = k0 + tid + q * 256u;
      t[q] = make_uint4(0u, 0u, 0u, 0u);
      if (k < kTcRows * ks) {
        const unsigned rr = k / ks, j = k - rr * ks;
        const unsigned long long off = s_off[rr];
        if (off != ~0ull) t[q] = __ldg(reinterpret_cast<const uint4*>(p.ring + off) + j);
      }
    }
#pragma unroll
    for (unsigned q = 0; q < kBatch; ++q) {
      const unsigned k = k0 + tid + q * 256u;
      if (k < kTcRows * ks) {
        const unsigned rr = k / ks, j = k - rr * ks;
        uint4 w0, w1;
        limb_words(t[q].x, w0.x, w0.y);
        limb_words(t[q].y, w0.z, w0.w);
        limb_words(t[q].z, w1.x, w1.y);
        limb_words(t[q].w, w1.z, w1.w);
        uint4* dst = reinterpret_cast<uint4*>(s_x + rr * S + 8u * j);
        dst[0] = w0;
        dst[1] = w1;
      }
    }
  }
  for (unsigned k = tid; !vec && k < kTcRows * ks; k += 256u) {
    const unsigned rr = k / ks, j = k - rr * ks;
    const unsigned long long off = s_off[rr];
    uint32_t v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    if (off != ~0ull) {
      {
        const unsigned a = 4u * j;
        v0 = p.ring[off + a];
        if (a + 1u < C) v1 = p.ring[off + a + 1u];
        if (a + 2u < C) v2 = p.ring[off + a + 2u];
        if (a + 3u < C) v3 = p.ring[off + a + 3u];
      }
    }
    uint4 w0, w1;
    limb_words(v0, w0.x, w0.y);
    limb_words(v1, w0.z, w0.w);
    limb_words(v2, w1.x, w1.y);
    limb_words(v3, w1.z, w1.w);
    uint4* dst = reinterpret_cast<uint4*>(s_x + rr * S + 8u * j);
    dst[0] = w0;
    dst[1] = w1;
  }
  __syncthreads();

  const unsigned rr0 = warp * 16u + gid;
  unsigned fl_any = 0;
  unsigned long long nsat = 0;
  tile_products(p, s_x, S, ks, r0, rr0, s_off[rr0] != ~0ull, s_off[rr0 + 8u] != ~0ull, s_f[rr0],
                s_bin[rr0], s_f[rr0 + 8u], s_bin[rr0 + 8u], fl_any, nsat);
  const unsigned a = __reduce_or_sync(0xffffffffu, fl_any);
  for (int o = 16; o > 0; o >>= 1) nsat += __shfl_xor_sync(0xffffffffu, nsat, o);
  if (lane == 0u && p.stats) {
    if (a) atomicOr(&p.stats->bf_flags, a);
    if (nsat) atomicAdd(&p.stats->bf_sat, nsat);
  }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Tiles of 128 rows that are one contiguous run of the ring (N a multiple of
// 128: 128 bins of one frame, C a multiple of 4, C <= 64): a persistent CTA
// copies tile t + grid into a raw buffer with cp.async while it multiplies
// tile t, so the spectrum reads overlap the tensor work. The raw samples are
// converted into limb words in shared memory as in k_beam_tc.
__global__ void __launch_bounds__(256, 2) k_beam_tc_pipe(BeamParams p, unsigned n_tiles) {
  extern __shared__ __align__(16) uint32_t sm[];
  const unsigned C = p.C, N = p.N;
  const unsigned ks = C / 4u, S = 8u * ks + 4u, RS = C + 4u;
  uint32_t* s_x = sm;                  // [128][S] limb words of tile t
  uint32_t* s_raw = sm + kTcRows * S;  // [128][RS] samples of the next tile
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u, gid = lane >> 2;
  const unsigned q4 = kTcRows * ks;    // 16-byte pieces of a tile
  auto fetch = [&](unsigned t) {
    const uint64_t row0 = (uint64_t)t * kTcRows;
    const unsigned f = (unsigned)(row0 / N), bin0 = (unsigned)(row0 - (uint64_t)f * N);
    unsigned slot = p.ring_base + f;
    if (slot >= p.ring_frames) slot -= p.ring_frames;
    const uint32_t* src = p.ring + ((size_t)slot * N + bin0) * C;
    for (unsigned i = tid; i < q4; i += 256u) {
      const unsigned rr = i / ks, j = i - rr * ks;
      cp_async16(s_raw + rr * RS + 4u * j, src + 4u * i);
    }
    cp_async_commit();
  };
  unsigned fl_any = 0;
  unsigned long long nsat = 0;
  unsigned t = blockIdx.x;
  if (t < n_tiles) fetch(t);
  for (; t < n_tiles; t += gridDim.x) {
    cp_async_wait_all();
    __syncthreads();  // tile t landed for every thread; the last tile's products are done
    // row-fastest, so that both the padded raw rows (stride C + 4) and the
    // limb rows (stride 8 ks + 4) put a quarter-warp's 16-byte accesses on
    // distinct banks
    for (unsigned i = tid; i < q4; i += 256u) {
      const unsigned rr = i & (kTcRows - 1u), j = i / kTcRows;
      const uint4 v = *reinterpret_cast<const uint4*>(s_raw + rr * RS + 4u * j);
      uint4 w0, w1;
      limb_words(v.x, w0.x, w0.y);
      limb_words(v.y, w0.z, w0.w);
      limb_words(v.z, w1.x, w1.y);
      limb_words(v.w, w1.z, w1.w);
      uint4* dst = reinterpret_cast<uint4*>(s_x + rr * S + 8u * j);
      dst[0] = w0;
      dst[1] = w1;
    }
    __syncthreads();  // the limb words are ready; the raw buffer is free
    if (t + gridDim.x < n_tiles) fetch(t + gridDim.x);
    const uint64_t row0 = (uint64_t)t * kTcRows;
    const unsigned f = (unsigned)(row0 / N), binb = (unsigned)(row0 - (uint64_t)f * N);
    const unsigned rr0 = warp * 16u + gid;
    tile_products(p, s_x, S, ks, row0, rr0, true, true, f, binb + rr0, f, binb + rr0 + 8u,
                  fl_any, nsat);
  }
  const unsigned a = __reduce_or_sync(0xffffffffu, fl_any);
  for (int o = 16; o > 0; o >>= 1) nsat += __shfl_xor_sync(0xffffffffu, nsat, o);
  if (lane == 0u && p.stats) {
    if (a) atomicOr(&p.stats->bf_flags, a);
    if (nsat) atomicAdd(&p.stats->bf_sat, nsat);
  }
}

size_t beam_tc_smem(uint32_t C) {
  const size_t S = 8u * ((C + 3u) / 4u) + 4u;
  return (kTcRows * S + 4u * kTcRows) * sizeof(uint32_t);
}

static size_t pipe_smem(uint32_t C) {
  return (kTcRows * (8u * (C / 4u) + 4u) + (size_t)kTcRows * (C + 4u)) * sizeof(uint32_t);
}

// the dynamic shared-memory opt-in is per device
static std::atomic<bool> g_tc_attr[64];

void launch_beam_tc(const BeamParams& p, cudaStream_t s) {
  const uint64_t rows = (uint64_t)p.F * p.N;
  if (!rows) return;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !g_tc_attr[dev].load()) {
    cudaFuncSetAttribute(k_beam_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)beam_tc_smem(RD_TC_MAX_CHAN));
    cudaFuncSetAttribute(k_beam_tc_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)pipe_smem(64));
    if (dev >= 0 && dev < 64) g_tc_attr[dev].store(true);
  }
  if (p.N % kTcRows == 0u && p.C % 4u == 0u && p.C <= 64u && p.ring_frames >= 1u) {
    int n_sm = 0;
    if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      n_sm = 0;
    }
    const uint64_t tiles = rows / kTcRows;  // N a multiple of 128: every tile full
    const uint64_t grid = n_sm > 0 ? std::min<uint64_t>(tiles, 2ull * (unsigned)n_sm) : tiles;
    k_beam_tc_pipe<<<(unsigned)grid, 256, pipe_smem(p.C), s>>>(p, (unsigned)tiles);
    return;
  }
  k_beam_tc<<<(unsigned)((rows + kTcRows - 1u) / kTcRows), 256, beam_tc_smem(p.C), s>>>(p);
}

}  // namespace rd
