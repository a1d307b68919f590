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
// integer the Integrator adds, each class read off its fp32 value with adds
// (exact_int24) - then adds the carried-in sum (first segment of the
// launch), writes each window that closes, and the carried-out sum.
//
// Kernel: persistent, one CTA per SM, warp-specialised (544 threads): warp 0
// allocates TMEM and issues the MMAs; warps 1-8 stage 64-frame chunks of the
// spectrum (16-byte cp.async copies of 4 channels a frame into a ring of raw
// stages, three chunks ahead, then converted into double-buffered operand
// tiles); warps 9-16 read the accumulators
// back (warp w: TMEM lanes 32 (w % 4) .. + 31 = A rows, half of the columns)
// and finish the sums.
// A work unit is (window segment, bin group); its accumulators alternate
// between two TMEM buffers. Every wait is bounded (DevStats::dev_timeout on a
// timeout).
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
// bytes per 8-row group: the group's 16 core matrices (2 KB) and a 16-byte
// skew, so that the 8 row groups a quarter-warp's stores touch (rows 4 g + j,
// g = 0 .. 7) start in 8 different 16-byte bank slots
constexpr unsigned kSboC = 16u * kKp + 16u;
constexpr unsigned kMatC = 16u * kSboC;             // one limb matrix (128 rows)
constexpr unsigned kProdC = 8u;                     // producer warps 1 .. 8
constexpr unsigned kEpiC = 9u;                      // epilogue warps 9 .. 16
constexpr unsigned kThreadsC = 544u;
// a chunk's items: (4-row group g, 4-frame quad) = 16 x 16, one per producer
constexpr unsigned kItemsC = 16u * (kChunk / 4u);
static_assert(kItemsC == kProdC * 32u, "one item per producer thread");
constexpr unsigned kStages = 4u;                    // chunks of raw words in flight
constexpr unsigned kStageBytes = kItemsC * 4u * 16u;  // 16 KB: [frame e][item] uint4

__host__ __device__ inline unsigned sp_of(unsigned S) {
  unsigned sp = 16u;
  while (sp < S) sp <<= 1;
  return sp;
}

}  // namespace

// One producer thread's item of one 64-frame chunk: A rows 4 g .. 4 g + 3
// (bin bin0 + 4 g / Sp, channels 4 g % Sp ..) over frames 4 fq .. 4 fq + 3,
// g = pt % 16 and fq = pt / 16, so a warp's 16-byte copies of one frame cover
// 64 consecutive rows (256 contiguous bytes when S = Sp). Copies frame
// 4 fq + e of the 4 channels to stage word [e][pt] with cp.async, zero-filled
// outside the chunk, the bins, the channels. vec: S is a multiple of 4 and the
// source 16-byte aligned, so a group of 4 channels is whole and aligned.
__device__ __forceinline__ void c5_issue(const CovParams& p, unsigned pt, unsigned Sp, bool vec,
                                         unsigned f0, unsigned hi, unsigned bin0, uint32_t stage) {
  const uint32_t* src = p.src_beam ? p.beams_bn : p.ring;
  const unsigned r0 = 4u * (pt & 15u), fq = pt >> 4;
  const unsigned ch0 = r0 & (Sp - 1u), bin = bin0 + r0 / Sp;
  const bool rok = ch0 < p.S && bin < p.N;
#pragma unroll
  for (unsigned e = 0; e < 4u; ++e) {
    const unsigned f = f0 + 4u * fq + e;
    const bool fok = rok && f < hi;
    const uint32_t* a = src;  // any valid address when nothing is read
    if (fok) {
      unsigned slot = p.src_beam ? f : p.ring_base + f;
      if (!p.src_beam && slot >= p.ring_frames) slot -= p.ring_frames;
      a = src + ((size_t)slot * p.N + bin) * p.S + ch0;
    }
    const uint32_t d = stage + (e * kItemsC + pt) * 16u;
    if (vec) {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(a),
                   "r"(fok ? 16 : 0)
                   : "memory");
    } else {
#pragma unroll
      for (unsigned j = 0; j < 4u; ++j) {
        const bool ok = fok && ch0 + j < p.S;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d + 4u * j),
                     "l"(ok ? a + j : src), "r"(ok ? 4 : 0)
                     : "memory");
      }
    }
  }
}

// Channel j of the four frames as one 16-byte row of each limb matrix: row
// r = 4 g + j (U) and 64 + r (V), K chunk fq (frames 4 fq .. 4 fq + 3).
__device__ __forceinline__ void c5_row(uint8_t* ah, uint8_t* al, unsigned r, unsigned fq,
                                       uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3) {
  uint4 uh, ul;
  limb_words_bal(w0, uh.x, ul.x);
  limb_words_bal(w1, uh.y, ul.y);
  limb_words_bal(w2, uh.z, ul.z);
  limb_words_bal(w3, uh.w, ul.w);
  const uint4 vh = make_uint4(negswap(uh.x), negswap(uh.y), negswap(uh.z), negswap(uh.w));
  const uint4 vl = make_uint4(negswap(ul.x), negswap(ul.y), negswap(ul.z), negswap(ul.w));
  const unsigned ou = (r >> 3) * kSboC + fq * t5::kLbo + (r & 7u) * 16u;
  const unsigned ov = ou + 8u * kSboC;
  *reinterpret_cast<uint4*>(ah + ou) = uh;
  *reinterpret_cast<uint4*>(al + ou) = ul;
  *reinterpret_cast<uint4*>(ah + ov) = vh;
  *reinterpret_cast<uint4*>(al + ov) = vl;
}

// The item as [U; V] balanced limb words into one chunk buffer.
__device__ __forceinline__ void c5_store(unsigned pt, uint8_t* ah, uint8_t* al,
                                         const uint4 (&v)[4]) {
  const unsigned r0 = 4u * (pt & 15u), fq = pt >> 4;
  c5_row(ah, al, r0 + 0u, fq, v[0].x, v[1].x, v[2].x, v[3].x);
  c5_row(ah, al, r0 + 1u, fq, v[0].y, v[1].y, v[2].y, v[3].y);
  c5_row(ah, al, r0 + 2u, fq, v[0].z, v[1].z, v[2].z, v[3].z);
  c5_row(ah, al, r0 + 3u, fq, v[0].w, v[1].w, v[2].w, v[3].w);
}

bool cov_t5_ok(uint32_t S, uint32_t wl) { return S >= 1 && S <= 64 && wl >= 64 && wl <= 256; }

size_t cov_t5_smem(uint32_t S) {
  // two chunk buffers (high, low limbs), the raw-word stages, the pair map,
  // barriers; at least 120 KB so that two CTAs never share an SM (and its
  // TMEM)
  const size_t need = 4u * kMatC + kStages * kStageBytes + (size_t)S * S * 4u + 128u;
  return std::max<size_t>(need, 120u * 1024u);
}

__global__ void __launch_bounds__(kThreadsC, 1) k_cov_t5(CovParams p, const int32_t* pq,
                                                          unsigned n_groups, unsigned nz,
                                                          unsigned vec) {
  extern __shared__ __align__(1024) uint8_t smc[];
  __shared__ uint32_t s_abort;
  const unsigned S = p.S, Sp = sp_of(S), Pb = kColsC / Sp;  // channels padded, bins per tile
  uint8_t* sA = smc;                                   // [2 buffers][hi, lo]
  uint8_t* sStg = smc + 4u * kMatC;                    // [kStages] raw words
  int32_t* s_pq = reinterpret_cast<int32_t*>(sStg + kStages * kStageBytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sStg + kStages * kStageBytes +
                                               ((S * S * 4u + 15u) & ~15u));
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
      t5::bar_init(&t_empty[i], 256u);
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
    // units one after another. Each thread copies its item of chunk
    // c + kStages - 1 (cp.async, one commit group a chunk) before it converts
    // chunk c from the stage its own copies filled, so kStages - 1 chunks of
    // loads are in flight while it converts and waits for a buffer.
    const unsigned pt = tid - 32u;
    const uint32_t stg0 = t5::saddr(sStg);
    unsigned ii = 0, f_i = 0, hi_i = 0, b_i = 0;  // the next chunk to copy
    auto unit_start = [&](unsigned i) {
      if (i >= n_local) return false;
      const unsigned unit = blockIdx.x + i * gridDim.x, z = unit / n_groups;
      seg(z, f_i, hi_i);
      b_i = (unit - z * n_groups) * Pb;
      return true;
    };
    bool more = unit_start(0u);
    unsigned n_issued = 0;
    auto issue_next = [&]() {
      if (more) {
        c5_issue(p, pt, Sp, vec != 0u, f_i, hi_i, b_i, stg0 + (n_issued % kStages) * kStageBytes);
        ++n_issued;
        f_i += kChunk;
        if (f_i >= hi_i) more = unit_start(++ii);
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
#pragma unroll 1
    for (unsigned d = 0; d + 1u < kStages; ++d) issue_next();
#pragma unroll 1
    for (unsigned c = 0; c < n_issued && !*abort; ++c) {
      issue_next();
      // groups committed: c + kStages; chunk c's is complete when at most
      // kStages - 1 are pending
      asm volatile("cp.async.wait_group %0;\n" ::"n"(kStages - 1u) : "memory");
      const uint8_t* st = sStg + (c % kStages) * kStageBytes + pt * 16u;
      uint4 v[4];
#pragma unroll
      for (unsigned e = 0; e < 4u; ++e) v[e] = *reinterpret_cast<const uint4*>(st + e * kItemsC * 16u);
      if (!t5::bar_wait(&a_empty[c & 1u], ((c >> 1) & 1u) ^ 1u, abort)) break;
      c5_store(pt, sA + (c & 1u) * 2u * kMatC, sA + (c & 1u) * 2u * kMatC + kMatC, v);
      t5::fence_proxy_async();
      t5::bar_arrive(&a_full[c & 1u]);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
  } else {
    // ---- epilogue: D rows -> window sums of the pairs ----
    // warp w reads TMEM lanes 32 (w % 4) .. + 31; two warps share a lane
    // quarter, each taking half of the columns
    const unsigned q = warp & 3u, half = (warp - kEpiC) >> 2, row = 32u * q + lane;
    const unsigned comp = row >> 6, rl = row & 63u;  // 0: re rows (U), 1: im rows (V)
    const unsigned bl = rl / Sp, y = rl & (Sp - 1u);
    // A TMEM load takes one column address for the whole warp, and the
    // warp's 32 rows may belong to two bins (Sp = 16): the warp loads the
    // columns of every bin among its rows, and each lane uses its own bin's
    const unsigned wcol0 = (((32u * q) & 63u) / Sp) * Sp;
    const unsigned wcols = Sp < 32u ? 32u : Sp;
    const unsigned xa = half * (wcols / 2u), xe = xa + wcols / 2u;
    for (unsigned i = 0; i < n_local && !*abort; ++i) {
      const unsigned unit = blockIdx.x + i * gridDim.x, z = unit / n_groups;
      const unsigned bin = (unit - z * n_groups) * Pb + bl;
      const unsigned tb = i & 1u;
      const bool got = t5::bar_wait(&t_full[tb], (i >> 1) & 1u, abort);
      if (!__all_sync(0xffffffffu, got)) break;
      t5::fence_after();
      const bool carry_in = z == 0u, carry_out = z + 1u == nz, closes = z < p.n_windows;
      const bool lane_ok = y < S && bin < p.N;
      // the unit's rows of the carried-in and carried-out sums and of the
      // window output (pair pi at [pi], [pi], [2 pi])
      const size_t kb = (size_t)bin * p.P;
      const long long* acc_in = (comp ? p.acc_im : p.acc_re) + kb;
      long long* acc_out = (comp ? p.acc_im_out : p.acc_re_out) + kb;
      long long* outw = p.out + ((size_t)z * p.N * p.P + kb) * 2u + comp;
      const uint32_t tq = tmem + ((32u * q) << 16) + tb * 3u * kColsC + wcol0;
      for (unsigned x0 = xa; x0 < xe; x0 += 8u) {
        // columns wcol0 + x0 .. + 7 against the lane's bin's columns
        // bl Sp .. bl Sp + Sp - 1: their pair indices, and the block is
        // skipped when no lane of the warp has a pair in it
        const int xb = (int)(wcol0 + x0) - (int)(bl * Sp);
        const bool blk_ok = lane_ok && xb >= 0 && xb < (int)Sp;
        int pis[8];
        bool any = false;
#pragma unroll
        for (unsigned k = 0; k < 8u; ++k) {
          const unsigned x = (unsigned)xb + k;
          pis[k] = blk_ok && x < S ? s_pq[x * S + y] : -1;
          any |= pis[k] >= 0;
        }
        if (!__any_sync(0xffffffffu, any)) continue;
        // carried-in sums loaded all at once, ahead of the stores (which may
        // alias them for the compiler), and in flight during the TMEM load
        long long cin[8];
#pragma unroll
        for (unsigned k = 0; k < 8u; ++k)
          cin[k] = carry_in && pis[k] >= 0 ? __ldg(acc_in + pis[k]) : 0ll;
        uint32_t c16[8], c8[8], c0[8];
        t5::tmem_ld3x8(tq + x0, tq + kColsC + x0, tq + 2u * kColsC + x0, c16, c8, c0);
#pragma unroll
        for (unsigned k = 0; k < 8u; ++k) {
          const int pi = pis[k];
          if (pi < 0) continue;
          long long v = fold3_24(__uint_as_float(c16[k]), __uint_as_float(c8[k]),
                                 __uint_as_float(c0[k])) +
                        cin[k];
          if (closes) {
            outw[2 * pi] = v;
            v = 0;
          }
          if (carry_out) acc_out[pi] = v;
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
  // the opt-in covers the largest channel count; with the kernel's static
  // shared memory it stays within the 227 KB a block may have
  g_c5_attr.once([] {
    cudaFuncSetAttribute(k_cov_t5, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cov_t5_smem(64));
  });
  const unsigned units = nz * n_groups;
  const unsigned grid = std::min<unsigned>(units, (unsigned)(n_sm > 0 ? n_sm : 1));
  // 16-byte loads when every group of 4 channels starts on a 16-byte boundary
  const void* src = p.src_beam ? (const void*)p.beams_bn : (const void*)p.ring;
  const unsigned vec = (p.S % 4u == 0u && reinterpret_cast<uintptr_t>(src) % 16u == 0u) ? 1u : 0u;
  k_cov_t5<<<grid, kThreadsC, cov_t5_smem(p.S), s>>>(p, pq, n_groups, nz, vec);
}

}  // namespace rd
