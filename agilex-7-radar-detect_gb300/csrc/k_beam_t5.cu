// k_beam_t5.cu - beamforming on the 5th-generation tensor cores (tcgen05,
// TMEM accumulators), exact.
//
// Y[r][b] = sum_a X[r][a] W[b][a] (bf::dot, beamformer_model.hpp:162-179) with
// both int16 operands split into balanced 8-bit limbs held exactly in fp16,
//
//   x = 256 xh + xl,  w = 256 wh + wl,  xl, wl in [-128, 127], xh, wh in [-128, 128]
//
// (xl the sign-extended low byte, xh = (x >> 8) + bit 7 of x),
// and the complex product organised as three real GEMMs over the real
// embedding of the channels (K = 2C: k = 2a + {re, im}) and of the beams
// (N = 2 per beam: n = 2b + {re, im}):
//
//   D16 = Xh Whi^T,   D0 = Xl Wlo^T,   D8 = Xh Wlo^T + Xl Whi^T
//
// where Whi[(b, re)][(a, re), (a, im)] = (wh_re, -wh_im) and
// Whi[(b, im)][...] = (wh_im, wh_re), and Wlo the same with the low limbs.
// Then re/im of bf::dot's int64 sum is 2^16 D16 + 2^8 D8 + D0. Every limb
// product is an integer of magnitude <= 2^14, and every partial sum the
// tensor core forms (at most 4C terms in D8, 2C in D16 and D0) is an integer
// of magnitude <= 2^22 for C <= 64, so the fp32 accumulators hold them exactly
// in any order. (The limbs and their negations are integers of magnitude <=
// 128: exact in fp16.) An integer v with |v| <= 2^22 turns into an int by one
// fp32 add: v + 1.5 x 2^23 lies where fp32's spacing is 1, so its bit pattern
// is that of 1.5 x 2^23 plus v - no conversion instruction. When |D16| <=
// 16351, |2^16 D16 + 2^8 D8 + D0| <= 2^31 - 2^15 - 1, so the sum recombines
// and rounds in 32 bits; other outputs take the 64-bit path.
//
// Kernel: persistent, one CTA per SM, warp-specialised (512 threads):
//   warp 0      allocates TMEM and issues the MMAs (one thread);
//   warps 1-7   convert 128-row tiles of the spectrum ring into Xh / Xl in
//               shared memory (double-buffered); a thread loads its share of
//               tile i + 1 into registers before it waits for the buffer, so
//               the loads' latency overlaps the wait;
//   warps 8-15  read the accumulators back (warp 8 + e: TMEM lanes 32 (e % 4)
//               .. + 31, i.e. tile rows; e / 4 picks half of the beam
//               columns) and finish round_sat, power and the outputs.
// The weight operands of every beam group (32 beams, N = 64) stay in shared
// memory for the whole launch; each group's three accumulators (3 x N fp32
// columns) alternate between two TMEM buffers, so the epilogue of one group
// overlaps the MMAs of the next. mbarriers order the roles; every wait is
// bounded, and a wait that gives up sets DevStats::dev_timeout, makes every
// role leave its loop, lets this CTA's issued MMAs finish and frees the TMEM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "fxp.cuh"
#include "rd_internal.h"
#include "tc.cuh"
#include "tc5.cuh"

namespace rd {

namespace {

constexpr unsigned kRows = 128u;     // M: rows per tile, one TMEM lane each
constexpr unsigned kProd = 7u;       // producer warps (1 .. 7)
constexpr unsigned kEpi0 = 8u;       // first epilogue warp (8 .. 15)
constexpr unsigned kEpi = 8u;        // epilogue warps: two per TMEM lane quadrant
constexpr unsigned kThreads = 512u;
// 16-byte items (4 channels of one row) a producer thread converts per tile:
// 128 rows x at most 16 items a row, over the producer threads
constexpr unsigned kItemsMax = (kRows * 16u + kProd * 32u - 1u) / (kProd * 32u);

struct Geo5 {
  unsigned Kp;   // fp16 per operand row: 2C rounded up to a multiple of 16
  unsigned nch;  // 16-byte chunks per row (4 channels each)
  unsigned NB;   // beams per group (a multiple of 8, <= 32)
  unsigned N;    // MMA N = 2 NB
  unsigned G;    // groups
  unsigned CS;   // TMEM columns per accumulator class
};

__host__ __device__ inline Geo5 geo5(unsigned C, unsigned B) {
  Geo5 g;
  g.Kp = (2u * C + 15u) & ~15u;
  g.nch = g.Kp / 8u;
  const unsigned b8 = (B + 7u) & ~7u;
  g.NB = b8 < 32u ? b8 : 32u;
  g.N = 2u * g.NB;
  g.G = (B + g.NB - 1u) / g.NB;
  g.CS = g.N;
  return g;
}

// shared-memory plan (bytes): [A: 2 buffers x (Xh, Xl)] [W: G x (hi, lo)]
// [mbarriers] [TMEM address]
__host__ __device__ inline unsigned a_bytes(const Geo5& g) { return kRows * g.Kp * 2u; }
__host__ __device__ inline unsigned w_bytes(const Geo5& g) { return g.N * g.Kp * 2u; }
__host__ __device__ inline unsigned bar_off(const Geo5& g) {
  return 4u * a_bytes(g) + 2u * g.G * w_bytes(g);
}
// TMEM columns: two buffers of three classes, rounded up to a power of two
__host__ __device__ inline unsigned tmem_cols(const Geo5& g) {
  unsigned need = 6u * g.CS, c = 32u;
  while (c < need) c <<= 1;
  return c;
}

// The host-built weight operand in the canonical layout, element (n, k) of
// matrix (group, hi/lo). Limbs of beams >= B and channels >= C are zero.
int w5_value(const uint32_t* w, unsigned C, unsigned B, const Geo5& g, unsigned grp, int lo,
             unsigned n, unsigned k) {
  const unsigned b = grp * g.NB + n / 2u, a = k / 2u;
  if (b >= B || a >= C) return 0;
  const uint32_t v = w[(size_t)b * C + a];
  const int re = (int16_t)(uint16_t)(v & 0xFFFFu), im = (int16_t)(uint16_t)(v >> 16);
  // balanced limbs: the low one the sign-extended low byte, the high one the
  // rest divided by 256
  auto lo8 = [](int v) { return ((v & 255) ^ 128) - 128; };
  auto hi8 = [](int v) { return (v >> 8) + ((v >> 7) & 1); };
  const int wr = lo ? lo8(re) : hi8(re), wi = lo ? lo8(im) : hi8(im);
  const bool out_im = (n & 1u) != 0u, in_im = (k & 1u) != 0u;
  // re row: x_re wr - x_im wi; im row: x_re wi + x_im wr
  if (!out_im) return in_im ? -wi : wr;
  return in_im ? wr : wi;
}

uint16_t host_f16(int v) {  // IEEE binary16 of an integer |v| <= 2048
  if (v == 0) return 0;
  const unsigned sign = v < 0 ? 0x8000u : 0u;
  const unsigned m = (unsigned)(v < 0 ? -v : v);
  int e = 0;
  while ((m >> (e + 1)) != 0) ++e;
  const unsigned mant = (m << (10 - e)) & 0x3FFu;
  return (uint16_t)(sign | (unsigned)(e + 15) << 10 | mant);
}

}  // namespace

bool beam_t5_ok(uint32_t C, uint32_t B) {
  if (C == 0 || C > 64 || B == 0 || B > 128) return false;
  const Geo5 g = geo5(C, B);
  return bar_off(g) + 128u <= 200u * 1024u;
}

uint32_t beam_t5_operand_words(uint32_t C, uint32_t B) {
  const Geo5 g = geo5(C, B);
  return g.G * 2u * w_bytes(g) / 4u;
}

void beam_t5_operand(const uint32_t* w, uint32_t C, uint32_t B, uint32_t* out) {
  const Geo5 g = geo5(C, B);
  uint16_t* o = reinterpret_cast<uint16_t*>(out);
  const unsigned sbo = 16u * g.Kp;  // bytes per 8-row group
  for (unsigned grp = 0; grp < g.G; ++grp)
    for (int lo = 0; lo < 2; ++lo) {
      uint16_t* m = o + ((size_t)grp * 2u + (unsigned)lo) * (w_bytes(g) / 2u);
      for (unsigned n = 0; n < g.N; ++n)
        for (unsigned k = 0; k < g.Kp; ++k) {
          const size_t byte = (size_t)(n / 8u) * sbo + (k / 8u) * t5::kLbo + (n % 8u) * 16u +
                              (k % 8u) * 2u;
          m[byte / 2u] = host_f16(w5_value(w, C, B, g, grp, lo, n, k));
        }
    }
}

size_t beam_t5_smem(uint32_t C, uint32_t B) {
  const Geo5 g = geo5(C, B);
  // at least 120 KB, so that two CTAs never share an SM (and its TMEM)
  return std::max<size_t>(bar_off(g) + 128u, 120u * 1024u);
}

__global__ void __launch_bounds__(kThreads, 1) k_beam_t5(BeamParams p, unsigned n_tiles) {
  extern __shared__ __align__(1024) uint8_t sm5[];
  __shared__ uint32_t s_abort;
  const unsigned C = p.C, B = p.B, N = p.N;
  const Geo5 g = geo5(C, B);
  const unsigned sbo = 16u * g.Kp;
  const unsigned ab = a_bytes(g), wb = w_bytes(g);
  uint8_t* sA = sm5;                    // [2 buffers][Xh, Xl]
  uint8_t* sW = sm5 + 4u * ab;          // [G][hi, lo]
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm5 + bar_off(g));
  uint64_t* a_full = bars;              // [2] producers -> MMA
  uint64_t* a_empty = bars + 2;         // [2] MMA commit -> producers
  uint64_t* t_full = bars + 4;          // [2] MMA commit -> epilogue
  uint64_t* t_empty = bars + 6;         // [2] epilogue -> MMA
  uint64_t* done = bars + 8;            // MMA commit at the end
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const uint64_t rows = (uint64_t)p.F * N;
  const unsigned ncols = tmem_cols(g);

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      t5::bar_init(&a_full[i], kProd * 32u);
      t5::bar_init(&a_empty[i], 1);
      t5::bar_init(&t_full[i], 1);
      t5::bar_init(&t_empty[i], kEpi * 32u);
    }
    t5::bar_init(done, 1);
    t5::bar_init_fence();
    s_abort = 0;
  }
  // the weight operands of every group, copied once
  {
    const uint4* src = reinterpret_cast<const uint4*>(p.w_t5);
    uint4* dst = reinterpret_cast<uint4*>(sW);
    const unsigned n16 = 2u * g.G * wb / 16u;
    for (unsigned i = tid; i < n16; i += kThreads) dst[i] = __ldg(src + i);
  }
  t5::fence_proxy_async();
  __syncwarp();
  if (warp == 0) t5::tmem_alloc(tslot, ncols);
  t5::fence_before();
  __syncthreads();
  t5::fence_after();
  const uint32_t tmem = *tslot;
  volatile uint32_t* abort = &s_abort;
  const unsigned n_local = blockIdx.x < n_tiles ? (n_tiles - 1u - blockIdx.x) / gridDim.x + 1u : 0u;

  if (warp == 0) {
    // ---- MMA issue (one thread) ----
    if (lane == 0) {
      const uint32_t idesc = t5::idesc_f16(kRows, g.N);
      const unsigned ks = g.Kp / 16u;
      const uint32_t a0 = t5::saddr(sA), w0 = t5::saddr(sW);
      unsigned u = 0;  // groups issued so far
      for (unsigned i = 0; i < n_local && !*abort; ++i) {
        const unsigned s = i & 1u;
        if (!t5::bar_wait(&a_full[s], (i >> 1) & 1u, abort)) break;
        t5::fence_after();
        const uint32_t xh = a0 + s * 2u * ab, xl = xh + ab;
        bool ok = true;
        for (unsigned grp = 0; grp < g.G; ++grp, ++u) {
          const unsigned tb = u & 1u;
          if (!t5::bar_wait(&t_empty[tb], ((u >> 1) & 1u) ^ 1u, abort)) {
            ok = false;
            break;
          }
          t5::fence_after();
          const uint32_t whi = w0 + grp * 2u * wb, wlo = whi + wb;
          const uint32_t d16 = tmem + tb * 3u * g.CS, d8 = d16 + g.CS, d0 = d8 + g.CS;
          for (unsigned kk = 0; kk < ks; ++kk) {
            const uint32_t off = kk * 256u;
            const uint64_t dxh = t5::desc(xh + off, sbo), dxl = t5::desc(xl + off, sbo);
            const uint64_t dwh = t5::desc(whi + off, sbo), dwl = t5::desc(wlo + off, sbo);
            t5::mma_f16(d16, dxh, dwh, idesc, kk > 0u);
            t5::mma_f16(d0, dxl, dwl, idesc, kk > 0u);
            t5::mma_f16(d8, dxh, dwl, idesc, kk > 0u);
            t5::mma_f16(d8, dxl, dwh, idesc, 1u);
          }
          t5::commit(&t_full[tb]);
        }
        if (!ok) break;
        t5::commit(&a_empty[s]);
      }
      // every MMA this thread issued is done before the TMEM is given back
      t5::commit(done);
      if (!t5::bar_wait_own(done, 0u)) *abort = 1u;
    }
    __syncwarp();
  } else if (warp <= kProd) {
    // ---- producers: tile rows -> Xh, Xl ----
    const unsigned pt = tid - 32u;  // 0 .. 32 kProd - 1
    const unsigned items = kRows * g.nch;
    const bool vec = (C & 3u) == 0u;
    // The items of this thread are the same in every tile: item m is
    // 16-byte chunk j (channels 4j .. 4j + 3) of row `row`, stored at shared
    // byte offset soff[m]; eight consecutive items are the 8 rows of one core
    // matrix. grow[m] = row << 16 | 4j, or ~0 for an item that is all padding.
    uint32_t soff[kItemsMax], grow[kItemsMax];
#pragma unroll
    for (unsigned m = 0; m < kItemsMax; ++m) {
      const unsigned it = pt + m * kProd * 32u;
      const unsigned q8 = it >> 3, rr = it & 7u;
      const unsigned rg = q8 / g.nch, j = q8 - rg * g.nch;
      soff[m] = rg * sbo + j * t5::kLbo + rr * 16u;
      grow[m] = (it < items && 4u * j < C) ? ((rg * 8u + rr) << 16 | 4u * j) : ~0u;
    }
    for (unsigned i = 0; i < n_local && !*abort; ++i) {
      const unsigned s = i & 1u;
      const uint64_t r0 = (uint64_t)(blockIdx.x + i * gridDim.x) * kRows;
      // rows r0 .. r0 + last of this tile; row k is (frame f0, bin b0 + k)
      // wrapped into later frames
      const unsigned last = (unsigned)std::min<uint64_t>(kRows - 1u, rows - 1u - r0);
      const uint64_t f0 = r0 / N;
      const unsigned b0 = (unsigned)(r0 - f0 * N);
      auto pos = [&](unsigned row) {  // ring position (slot * N + bin) of a tile row
        const unsigned add = b0 + row;
        const unsigned df = add / N;
        uint64_t slot = p.ring_base + f0 + df;
        while (slot >= p.ring_frames) slot -= p.ring_frames;
        return slot * N + (add - df * N);
      };
      // the tile's rows are consecutive ring rows unless it crosses the
      // ring's end (then every row is located on its own)
      const uint64_t pos0 = pos(0u);
      const bool contig = pos(last) == pos0 + last;
      const uint32_t* base = p.ring + pos0 * C;
      // every load of this thread's items first, then the wait for the buffer
      uint4 v[kItemsMax];
#pragma unroll
      for (unsigned m = 0; m < kItemsMax; ++m) {
        v[m] = make_uint4(0u, 0u, 0u, 0u);
        const unsigned row = grow[m] >> 16, a = grow[m] & 0xFFFFu;
        if (grow[m] == ~0u || row > last) continue;
        const uint32_t* src = (contig ? base + row * C : p.ring + pos(row) * C) + a;
        if (vec) {
          v[m] = __ldg(reinterpret_cast<const uint4*>(src));
        } else {
          v[m].x = __ldg(src);
          if (a + 1u < C) v[m].y = __ldg(src + 1);
          if (a + 2u < C) v[m].z = __ldg(src + 2);
          if (a + 3u < C) v[m].w = __ldg(src + 3);
        }
      }
      if (!t5::bar_wait(&a_empty[s], ((i >> 1) & 1u) ^ 1u, abort)) break;
      uint8_t* xh = sA + s * 2u * ab;
      uint8_t* xl = xh + ab;
#pragma unroll
      for (unsigned m = 0; m < kItemsMax; ++m) {
        if (pt + m * kProd * 32u >= items) continue;
        uint4 h, l;
        limb_words_bal(v[m].x, h.x, l.x);
        limb_words_bal(v[m].y, h.y, l.y);
        limb_words_bal(v[m].z, h.z, l.z);
        limb_words_bal(v[m].w, h.w, l.w);
        *reinterpret_cast<uint4*>(xh + soff[m]) = h;
        *reinterpret_cast<uint4*>(xl + soff[m]) = l;
      }
      t5::fence_proxy_async();
      t5::bar_arrive(&a_full[s]);
    }
  } else {
    // ---- epilogue: accumulators -> outputs ----
    const unsigned e = warp - kEpi0;
    const unsigned q = e & 3u, half = e >> 2;  // TMEM lane quadrant, column half
    const unsigned row = 32u * q + lane;
    unsigned fl_any = 0;
    unsigned nsat = 0;
    unsigned u = 0;
    for (unsigned i = 0; i < n_local && !*abort; ++i) {
      const uint64_t r = (uint64_t)(blockIdx.x + i * gridDim.x) * kRows + row;
      const bool live = r < rows;
      const uint64_t f = live ? r / N : 0, bin = live ? r - f * N : 0;
      // this row's outputs: beam b at pw[b N], bn[b], yr[b], ar[2 b], fr[b]
      uint32_t* pw = p.power ? p.power + f * B * N + bin : nullptr;
      uint32_t* bn = p.beams_bn ? p.beams_bn + (f * N + bin) * B : nullptr;
      uint32_t* yr_row = p.y_rows ? p.y_rows + r * B : nullptr;
      long long* ar_row = p.acc_rows ? p.acc_rows + r * B * 2 : nullptr;
      uint8_t* fr_row = p.flag_rows ? p.flag_rows + r * B : nullptr;
      bool ok = true;
      for (unsigned grp = 0; grp < g.G; ++grp, ++u) {
        const unsigned tb = u & 1u;
        // every lane waits, and the warp goes on only together: the loads
        // below are warp-collective
        const bool got = t5::bar_wait(&t_full[tb], (u >> 1) & 1u, abort);
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        t5::fence_after();
        const uint32_t tq = tmem + ((32u * q) << 16) + tb * 3u * g.CS;
        for (unsigned c8 = half; c8 < g.NB / 8u; c8 += 2u) {
          uint32_t v16[16], v8[16], v0[16];
          t5::tmem_ld3x16(tq + 16u * c8, tq + g.CS + 16u * c8, tq + 2u * g.CS + 16u * c8, v16, v8,
                          v0);
          // the eight beams of the chunk without branches: the 32-bit path for
          // every output, and a bit per output that needs the 64-bit path or
          // saturates (both rare), which a second pass redoes
          constexpr int32_t kBias = 0x4B400000;          // bits of 1.5 x 2^23
          constexpr uint32_t kFold = (uint32_t)kBias * 65793u;
          auto mg = [](uint32_t u) {  // bits of 1.5 x 2^23 + v, |v| <= 2^22
            return (int32_t)__float_as_uint(__fadd_rn(__uint_as_float(u), 12582912.f));
          };
          uint32_t y[8], pv[8];
          unsigned slow = 0;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int32_t r16 = mg(v16[2 * k]), i16 = mg(v16[2 * k + 1]);
            const int32_t r8 = mg(v8[2 * k]), i8 = mg(v8[2 * k + 1]);
            const int32_t r0 = mg(v0[2 * k]), i0 = mg(v0[2 * k + 1]);
            // 2^16 D16 + 2^8 D8 + D0 modulo 2^32, the biases folded into one
            // constant; exact when |D16| <= 16351
            const int32_t re32 = (int32_t)(((uint32_t)r16 << 16) + ((uint32_t)r8 << 8) +
                                           (uint32_t)r0 - kFold);
            const int32_t im32 = (int32_t)(((uint32_t)i16 << 16) + ((uint32_t)i8 << 8) +
                                           (uint32_t)i0 - kFold);
            // round_sat(v, 15, 16) in 32 bits (q15_out32)
            const int32_t yr = (re32 + 0x3FFF + ((re32 >> 15) & 1)) >> 15;
            const int32_t yi = (im32 + 0x3FFF + ((im32 >> 15) & 1)) >> 15;
            const bool fits = ((uint32_t)(r16 - kBias + 16351) <= 32702u) &&
                              ((uint32_t)(i16 - kBias + 16351) <= 32702u);
            const bool in16 = ((uint32_t)(yr + 32768) | (uint32_t)(yi + 32768)) <= 65535u;
            slow |= (fits && in16) ? 0u : (1u << k);
            y[k] = pack2(yr, yi);
            pv[k] = (uint32_t)(yr * yr) + (uint32_t)(yi * yi);
          }
          unsigned flk[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          long long accr[8], acci[8];
          const bool want_acc = ar_row != nullptr;
          if (want_acc) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              accr[k] = ((long long)(mg(v16[2 * k]) - kBias) << 16) +
                        ((long long)(mg(v8[2 * k]) - kBias) << 8) + (long long)(mg(v0[2 * k]) - kBias);
              acci[k] = ((long long)(mg(v16[2 * k + 1]) - kBias) << 16) +
                        ((long long)(mg(v8[2 * k + 1]) - kBias) << 8) +
                        (long long)(mg(v0[2 * k + 1]) - kBias);
            }
          }
          if (slow) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              if (!((slow >> k) & 1u)) continue;
              const long long re_v = ((long long)(mg(v16[2 * k]) - kBias) << 16) +
                                     ((long long)(mg(v8[2 * k]) - kBias) << 8) +
                                     (long long)(mg(v0[2 * k]) - kBias);
              const long long im_v = ((long long)(mg(v16[2 * k + 1]) - kBias) << 16) +
                                     ((long long)(mg(v8[2 * k + 1]) - kBias) << 8) +
                                     (long long)(mg(v0[2 * k + 1]) - kBias);
              unsigned fr = 0, fi = 0;
              const int32_t yr = q15_out64(re_v, &fr), yi = q15_out64(im_v, &fi);
              if (fr | fi) {
                fl_any |= fr | fi;
                ++nsat;
              }
              flk[k] = (fr << 2) | fi;
              y[k] = pack2(yr, yi);
              pv[k] = (uint32_t)(yr * yr) + (uint32_t)(yi * yi);
            }
          }
          if (live) {
            const unsigned bc = grp * g.NB + 8u * c8;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const unsigned b = bc + (unsigned)k;
              if (b >= B) break;
              if (pw) pw[b * N] = pv[k];
              if (bn) bn[b] = y[k];
              if (yr_row) yr_row[b] = y[k];
              if (want_acc) {
                ar_row[2u * b] = accr[k];
                ar_row[2u * b + 1u] = acci[k];
              }
              if (fr_row) fr_row[b] = (uint8_t)flk[k];
            }
          }
        }
        t5::fence_before();
        t5::bar_arrive(&t_empty[tb]);
      }
      if (!ok) break;
    }
    const unsigned a = __reduce_or_sync(0xffffffffu, fl_any);
    const unsigned ns = __reduce_add_sync(0xffffffffu, nsat);
    if (lane == 0u && p.stats) {
      if (a) atomicOr(&p.stats->bf_flags, a);
      if (ns) atomicAdd(&p.stats->bf_sat, (unsigned long long)ns);
    }
  }
  if (tid == 0 && *abort && p.stats) atomicOr(&p.stats->dev_timeout, 1u);
  t5::fence_before();
  __syncthreads();
  t5::fence_after();
  if (warp == 0) {
    __syncwarp();
    t5::tmem_dealloc(tmem, ncols);
  }
}

static PerDevice g_t5_attr;

void launch_beam_t5(const BeamParams& p, cudaStream_t s) {
  const uint64_t rows = (uint64_t)p.F * p.N;
  if (!rows) return;
  const uint64_t tiles = (rows + kRows - 1u) / kRows;
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n_sm = 1;
  }
  g_t5_attr.once([] {
    cudaFuncSetAttribute(k_beam_t5, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)(n_sm > 0 ? n_sm : 1));
  k_beam_t5<<<grid, kThreads, beam_t5_smem(p.C, p.B), s>>>(p, (unsigned)tiles);
}

}  // namespace rd
