// k_cov_t5.cu - the exact block-mode covariance on the 5th-generation tensor
// cores (tcgen05, TMEM accumulators).
//
// covar::cross_power (covar_model.hpp:119-151) gives, per pair (x, y) and
// frame, R = X conj(Y): re = xr yr + xi yi, im = xi yr - xr yi; the block
// Integrator (covar_model.hpp:204-262) sums it over a window. When no sum can
// saturate (the condition launch_cov states) the window sum is a plain
// integer sum, and for one bin it is a Gram matrix over the window's frames.
// With u_c = (c_re, c_im) and v_c = (-c_im, c_re) per frame,
//
//   re(x, y) = sum_f u_y . u_x,   im(x, y) = sum_f v_y . u_x,
//
// a GEMM whose A rows are [U; V] (the channels' u rows, then their v rows),
// whose B rows are U, and whose depth K is 2 per frame. Several bins of fewer
// channels share one tile: A rows 0-63 hold U of 64 / Sp bins (Sp channels
// each, a power of two >= 16, padded with zeros), rows 64-127 their V, and B
// is A's first 64 rows (the same shared memory); only the diagonal blocks
// (a bin's rows against its own columns) are used.
//
// Both operands are split into balanced 8-bit limbs (u = 256 uh + ul, ul the
// sign-extended low byte in [-128, 127], uh in [-128, 128]) held exactly in
// fp16, and the three scale classes accumulate in TMEM:
//
//   D16 = Ah Bh^T,   D0 = Al Bl^T,   D8 = Ah Bl^T + Al Bh^T,
//
// every limb product an integer of magnitude <= 2^14 and every class at most
// 4 such terms a frame, so over a window segment of at most 256 frames every
// partial sum is an integer of magnitude <= 2^24: exact in the fp32
// accumulators. The epilogue recombines 2^16 D16 + 2^8 D8 + D0 in int64 - the
// integer the Integrator adds - then adds the carried-in sum (first segment
// of the launch), writes each window that closes, and the carried-out sum.
//
// Kernel: persistent, one CTA per SM, warp-specialised (384 threads): warp 0
// allocates TMEM and issues the MMAs; warps 1-7 stage 64-frame chunks of the
// spectrum (double-buffered in shared memory, and in two register sets, so a
// thread's loads of the next chunk are in flight while it converts this
// one); warps 8-11 read the accumulators back (warp 8 + q: TMEM lanes 32q ..
// 32q + 31 = A rows) and finish the sums. A work unit is
// (window segment, bin group); its accumulators alternate between two TMEM
// buffers. Every wait is bounded (DevStats::dev_timeout on a timeout).
#include <cuda_runtime.h>

#include <algorithm>

#include "rd_internal.h"
#include "tc.cuh"
#include "tc5.cuh"

namespace rd {

namespace {

constexpr unsigned kRowsC = 128u;   // M: [U; V] rows
constexpr unsigned kColsC = 64u;    // N: U rows
constexpr unsigned kChunk = 64u;    // frames per staged chunk (K = 128)
constexpr unsigned kKp = 2u * kChunk;
constexpr unsigned kSboC = 16u * kKp;               // bytes per 8-row group
constexpr unsigned kMatC = kRowsC * kKp * 2u;       // one limb matrix: 32 KB
constexpr unsigned kProdC = 7u;                     // producer warps 1 .. 7
constexpr unsigned kEpiC = 8u;                      // epilogue warps 8 .. 11
constexpr unsigned kThreadsC = 384u;
// items (row, 4-frame quad) of a chunk per producer thread
constexpr unsigned kItemsC = (kColsC * (kChunk / 4u) + kProdC * 32u - 1u) / (kProdC * 32u);

__host__ __device__ inline unsigned sp_of(unsigned S) {
  unsigned sp = 16u;
  while (sp < S) sp <<= 1;
  return sp;
}

}  // namespace

// One producer thread's items of one 64-frame chunk: item m is A row r
// (bin bin0 + r / Sp, channel r % Sp) and 4-frame quad fq; consecutive threads
// take consecutive rows (the 8 rows of a core matrix, and consecutive channels
// in memory). Loads them into v (zero outside the chunk, the bins, the
// channels).
__device__ __forceinline__ void c5_load(const CovParams& p, unsigned pt, unsigned Sp, bool ok,
                                        unsigned f0, unsigned hi, unsigned bin0,
                                        uint32_t (&v)[kItemsC][4]) {
  const uint32_t* src = p.src_beam ? p.beams_bn : p.ring;
#pragma unroll
  for (unsigned m = 0; m < kItemsC; ++m) {
    const unsigned it = pt + m * kProdC * 32u;
    const unsigned r = it & (kColsC - 1u), fq = it / kColsC;
    const unsigned ch = r & (Sp - 1u), bin = bin0 + r / Sp;
    const bool rok = ok && fq < kChunk / 4u && ch < p.S && bin < p.N;
#pragma unroll
    for (unsigned e = 0; e < 4u; ++e) {
      const unsigned f = f0 + 4u * fq + e;
      uint32_t x = 0u;
      if (rok && f < hi) {
        unsigned slot = p.src_beam ? f : p.ring_base + f;
        if (!p.src_beam && slot >= p.ring_frames) slot -= p.ring_frames;
        x = __ldg(src + ((size_t)slot * p.N + bin) * p.S + ch);
      }
      v[m][e] = x;
    }
  }
}

// The same items as [U; V] balanced limb words into one chunk buffer: row r
// (U) and row 64 + r (V) of the high- and low-limb matrices, K chunk fq
// (frames 4 fq .. 4 fq + 3).
__device__ __forceinline__ void c5_store(unsigned pt, uint8_t* ah, uint8_t* al,
                                         const uint32_t (&v)[kItemsC][4]) {
#pragma unroll
  for (unsigned m = 0; m < kItemsC; ++m) {
    const unsigned it = pt + m * kProdC * 32u;
    const unsigned r = it & (kColsC - 1u), fq = it / kColsC;
    if (fq >= kChunk / 4u) continue;
    uint4 uh, ul;
    limb_words_bal(v[m][0], uh.x, ul.x);
    limb_words_bal(v[m][1], uh.y, ul.y);
    limb_words_bal(v[m][2], uh.z, ul.z);
    limb_words_bal(v[m][3], uh.w, ul.w);
    const uint4 vh = make_uint4(negswap(uh.x), negswap(uh.y), negswap(uh.z), negswap(uh.w));
    const uint4 vl = make_uint4(negswap(ul.x), negswap(ul.y), negswap(ul.z), negswap(ul.w));
    const unsigned ou = (r >> 3) * kSboC + fq * t5::kLbo + (r & 7u) * 16u;
    const unsigned ov = ou + 8u * kSboC;
    *reinterpret_cast<uint4*>(ah + ou) = uh;
    *reinterpret_cast<uint4*>(al + ou) = ul;
    *reinterpret_cast<uint4*>(ah + ov) = vh;
    *reinterpret_cast<uint4*>(al + ov) = vl;
  }
}

bool cov_t5_ok(uint32_t S, uint32_t wl) { return S >= 1 && S <= 64 && wl >= 64 && wl <= 256; }

size_t cov_t5_smem(uint32_t S) {
  // two chunk buffers (high, low limbs), the pair map, barriers; at least
  // 120 KB so that two CTAs never share an SM (and its TMEM)
  const size_t need = 4u * kMatC + (size_t)S * S * 4u + 128u;
  return std::max<size_t>(need, 120u * 1024u);
}

__global__ void __launch_bounds__(kThreadsC, 1) k_cov_t5(CovParams p, const int32_t* pq,
                                                          unsigned n_groups, unsigned nz) {
  extern __shared__ __align__(1024) uint8_t smc[];
  __shared__ uint32_t s_abort;
  const unsigned S = p.S, Sp = sp_of(S), Pb = kColsC / Sp;  // channels padded, bins per tile
  uint8_t* sA = smc;                                   // [2 buffers][hi, lo]
  int32_t* s_pq = reinterpret_cast<int32_t*>(smc + 4u * kMatC);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smc + 4u * kMatC + ((S * S * 4u + 15u) & ~15u));
  uint64_t* a_full = bars;        // [2]
  uint64_t* a_empty = bars + 2;   // [2]
  uint64_t* t_full = bars + 4;    // [2]
  uint64_t* t_empty = bars + 6;   // [2]
  uint64_t* done = bars + 8;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
  const unsigned tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  constexpr unsigned kCols = 512u;  // 2 buffers x 3 classes x 64 columns, rounded up

  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      t5::bar_init(&a_full[i], kProdC * 32u);
      t5::bar_init(&a_empty[i], 1);
      t5::bar_init(&t_full[i], 1);
      t5::bar_init(&t_empty[i], 128u);
    }
    t5::bar_init(done, 1);
    t5::bar_init_fence();
    s_abort = 0;
  }
  for (unsigned i = tid; i < S * S; i += kThreadsC) s_pq[i] = __ldg(pq + i);
  __syncwarp();
  if (warp == 0) t5::tmem_alloc(tslot, kCols);
  t5::fence_before();
  __syncthreads();
  t5::fence_after();
  const uint32_t tmem = *tslot;
  volatile uint32_t* abort = &s_abort;
  // work units: (segment z, bin group), z-major; segment z covers frames
  // [lo, hi): the open window, then whole windows, then the trailing part
  const unsigned n_units = nz * n_groups;
  const unsigned n_local =
      blockIdx.x < n_units ? (n_units - 1u - blockIdx.x) / gridDim.x + 1u : 0u;
  const unsigned first = p.wl - p.count0;
  auto seg = [&](unsigned z, unsigned& lo, unsigned& hi) {
    lo = z == 0 ? 0u : first + (z - 1u) * p.wl;
    const unsigned h = z == 0 ? first : first + z * p.wl;
    hi = (nz == 1u || h > p.F) ? p.F : h;
  };

  if (warp == 0) {
    // ---- MMA issue (one thread) ----
    if (lane == 0) {
      const uint32_t idesc = t5::idesc_f16(kRowsC, kColsC);
      const uint32_t a0 = t5::saddr(sA);
      unsigned c = 0;  // chunks consumed so far
      for (unsigned i = 0; i < n_local && !*abort; ++i) {
        const unsigned unit = blockIdx.x + i * gridDim.x, z = unit / n_groups;
        unsigned lo, hi;
        seg(z, lo, hi);
        const unsigned tb = i & 1u;
        if (!t5::bar_wait(&t_empty[tb], ((i >> 1) & 1u) ^ 1u, abort)) break;
        t5::fence_after();
        const uint32_t d16 = tmem + tb * 3u * kColsC, d8 = d16 + kColsC, d0 = d8 + kColsC;
        bool ok = true, started = false;
        for (unsigned f0 = lo; f0 < hi; f0 += kChunk, ++c) {
          const unsigned s = c & 1u;
          if (!t5::bar_wait(&a_full[s], (c >> 1) & 1u, abort)) {
            ok = false;
            break;
          }
          t5::fence_after();
          const uint32_t ah = a0 + s * 2u * kMatC, al = ah + kMatC;
          const unsigned nf = hi - f0 < kChunk ? hi - f0 : kChunk;
          const unsigned ksteps = (nf + 7u) / 8u;  // 8 frames a step
          for (unsigned kk = 0; kk < ksteps; ++kk) {
            const uint32_t off = kk * 256u;
            const uint64_t dah = t5::desc(ah + off, kSboC), dal = t5::desc(al + off, kSboC);
            const uint32_t acc = started ? 1u : 0u;
            t5::mma_f16(d16, dah, dah, idesc, acc);  // B = the first 64 rows of A
            t5::mma_f16(d0, dal, dal, idesc, acc);
            t5::mma_f16(d8, dah, dal, idesc, acc);
            t5::mma_f16(d8, dal, dah, idesc, 1u);
            started = true;
          }
          t5::commit(&a_empty[s]);
        }
        if (!ok) break;
        t5::commit(&t_full[tb]);
      }
      t5::commit(done);
      if (!t5::bar_wait_own(done, 0u)) *abort = 1u;
    }
    __syncwarp();
  } else if (warp <= kProdC) {
    // ---- producers: 64-frame chunks of the unit's bins -> [U; V] limbs ----
    // The CTA's chunk sequence: unit i's frames [lo, hi) in 64-frame chunks,
    // units one after another. Chunk c + 1's loads are issued before chunk c
    // is converted (two register sets), so they overlap the conversion and
    // the wait for the buffer.
    const unsigned pt = tid - 32u;
    unsigned i_a = 0, f_a = 0, hi_a = 0, b_a = 0, i_b = 0, f_b = 0, hi_b = 0, b_b = 0;
    bool ok_a = false, ok_b = false;
    auto unit_start = [&](unsigned i, unsigned& f0, unsigned& hi, unsigned& bin0) {
      if (i >= n_local) return false;
      const unsigned unit = blockIdx.x + i * gridDim.x, z = unit / n_groups;
      seg(z, f0, hi);
      bin0 = (unit - z * n_groups) * Pb;
      return true;
    };
    ok_a = unit_start(0u, f_a, hi_a, b_a);
    uint32_t va[kItemsC][4], vb[kItemsC][4];
    c5_load(p, pt, Sp, ok_a, f_a, hi_a, b_a, va);
    for (unsigned c = 0; ok_a && !*abort; c += 2u) {
      // chunk c + 1 follows chunk c (a)
      i_b = i_a;
      f_b = f_a + kChunk;
      hi_b = hi_a;
      b_b = b_a;
      ok_b = f_b < hi_b || (i_b = i_a + 1u, unit_start(i_b, f_b, hi_b, b_b));
      c5_load(p, pt, Sp, ok_b, f_b, hi_b, b_b, vb);
      if (!t5::bar_wait(&a_empty[c & 1u], ((c >> 1) & 1u) ^ 1u, abort)) break;
      c5_store(pt, sA + (c & 1u) * 2u * kMatC, sA + (c & 1u) * 2u * kMatC + kMatC, va);
      t5::fence_proxy_async();
      t5::bar_arrive(&a_full[c & 1u]);
      if (!ok_b) break;
      // chunk c + 2 follows chunk c + 1 (b)
      i_a = i_b;
      f_a = f_b + kChunk;
      hi_a = hi_b;
      b_a = b_b;
      ok_a = f_a < hi_a || (i_a = i_b + 1u, unit_start(i_a, f_a, hi_a, b_a));
      c5_load(p, pt, Sp, ok_a, f_a, hi_a, b_a, va);
      const unsigned c1 = c + 1u;
      if (!t5::bar_wait(&a_empty[c1 & 1u], ((c1 >> 1) & 1u) ^ 1u, abort)) break;
      c5_store(pt, sA + (c1 & 1u) * 2u * kMatC, sA + (c1 & 1u) * 2u * kMatC + kMatC, vb);
      t5::fence_proxy_async();
      t5::bar_arrive(&a_full[c1 & 1u]);
    }
  } else {
    // ---- epilogue: D rows -> window sums of the pairs ----
    const unsigned q = warp - kEpiC, row = 32u * q + lane;
    const unsigned comp = row >> 6, rl = row & 63u;  // 0: re rows (U), 1: im rows (V)
    const unsigned bl = rl / Sp, y = rl & (Sp - 1u);
    // A TMEM load takes one column address for the whole warp, and the
    // warp's 32 rows may belong to two bins (Sp = 16): the warp loads the
    // columns of every bin among its rows, and each lane uses its own bin's
    const unsigned wcol0 = (((32u * q) & 63u) / Sp) * Sp;
    const unsigned wcols = Sp < 32u ? 32u : Sp;
    for (unsigned i = 0; i < n_local && !*abort; ++i) {
      const unsigned unit = blockIdx.x + i * gridDim.x, z = unit / n_groups;
      const unsigned bin = (unit - z * n_groups) * Pb + bl;
      const unsigned tb = i & 1u;
      const bool got = t5::bar_wait(&t_full[tb], (i >> 1) & 1u, abort);
      if (!__all_sync(0xffffffffu, got)) break;
      t5::fence_after();
      const bool carry_in = z == 0u, carry_out = z + 1u == nz, closes = z < p.n_windows;
      const uint32_t tq = tmem + ((32u * q) << 16) + tb * 3u * kColsC + wcol0;
      for (unsigned x0 = 0; x0 < wcols; x0 += 16u) {
        uint32_t c16[16], c8[16], c0[16];
        t5::tmem_ld3x16(tq + x0, tq + kColsC + x0, tq + 2u * kColsC + x0, c16, c8, c0);
        // this chunk's columns wcol0 + x0 .. + 15 against the lane's bin's
        // columns bl Sp .. bl Sp + Sp - 1
        const int xb = (int)(wcol0 + x0) - (int)(bl * Sp);
        if (y >= S || bin >= p.N || xb < 0 || xb >= (int)Sp) continue;
#pragma unroll
        for (unsigned k = 0; k < 16u; ++k) {
          const unsigned x = (unsigned)xb + k;
          if (x >= S) break;
          const int pi = s_pq[x * S + y];
          if (pi < 0) continue;
          long long v = (long long)__float2int_rn(__uint_as_float(c16[k])) * 65536 +
                        (long long)__float2int_rn(__uint_as_float(c8[k])) * 256 +
                        (long long)__float2int_rn(__uint_as_float(c0[k]));
          const size_t kq = (size_t)bin * p.P + (unsigned)pi;
          if (carry_in) v += comp ? p.acc_im[kq] : p.acc_re[kq];
          if (closes) {
            p.out[(((size_t)z * p.N + bin) * p.P + (unsigned)pi) * 2u + comp] = v;
            v = 0;
          }
          if (carry_out) (comp ? p.acc_im_out : p.acc_re_out)[kq] = v;
        }
      }
      t5::fence_before();
      t5::bar_arrive(&t_empty[tb]);
    }
  }
  if (tid == 0 && *abort && p.stats) atomicOr(&p.stats->dev_timeout, 1u);
  t5::fence_before();
  __syncthreads();
  t5::fence_after();
  if (warp == 0) {
    __syncwarp();
    t5::tmem_dealloc(tmem, kCols);
  }
}

static PerDevice g_c5_attr;

void launch_cov_t5(const CovParams& p, const int32_t* pq, cudaStream_t s) {
  if (p.P == 0 || p.F == 0) return;
  const unsigned first = p.wl - p.count0;
  const unsigned nz = first >= p.F ? 1u : 1u + (p.F - first + p.wl - 1u) / p.wl;
  const unsigned Pb = kColsC / sp_of(p.S);
  const unsigned n_groups = (p.N + Pb - 1u) / Pb;
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    n_sm = 1;
  }
  g_c5_attr.once([] {
    cudaFuncSetAttribute(k_cov_t5, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  });
  const unsigned units = nz * n_groups;
  const unsigned grid = std::min<unsigned>(units, (unsigned)(n_sm > 0 ? n_sm : 1));
  k_cov_t5<<<grid, kThreadsC, cov_t5_smem(p.S), s>>>(p, pq, n_groups, nz);
}

}  // namespace rd
