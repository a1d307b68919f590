// tc5.cuh - the 5th-generation tensor core (tcgen05) on sm_103a: operand
// descriptors, the f16 MMA into TMEM, commits, mbarriers with bounded waits,
// TMEM allocation and loads. Inline PTX only.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices (8 fp16 of 8 rows, 128 contiguous
// bytes); element (r, k) of a matrix with Kp fp16 per row is at byte
//   (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2
// with LBO = 128 (core matrices adjacent along K are contiguous) and
// SBO = 16 * Kp (8-row groups one after another). One MMA step consumes
// K = 16, two core matrices along K: the next step starts 256 bytes further.
#pragma once

#include <stdint.h>

namespace rd {
namespace t5 {

constexpr uint32_t kLbo = 128u;

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (64 bits): start address >> 4 in bits
// 0-13, LBO >> 4 in 16-29, SBO >> 4 in 32-45, the fixed value 1 in 46-47,
// base offset 0, no swizzle (bits 61-63 zero).
__device__ __forceinline__ uint64_t desc(uint32_t addr, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16 (32 bits): D fp32 (bits 4-5 = 1), A and
// B fp16 (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t m, uint32_t n) {
  return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// D[tmem] (+)= A * B^T, one thread issues it
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// the mbarrier's phase completes once every MMA this thread issued before is done
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          saddr(bar))
      : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(saddr(bar))
               : "memory");
}
// One try: the thread may sleep in hardware up to the hint (10 ms) and wakes
// when the phase completes, so a waiting warp takes no issue slots.
__device__ __forceinline__ bool bar_try(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(saddr(bar)), "r"(parity), "r"(10000000u)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Every wait gives up after 2 s of wall-clock time (or 2^24 tries, whichever
// comes first): a stage that long overdue means a fault, not a slow GPU.
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr uint32_t kMaxTries = 1u << 24;

// Waits for the phase of parity `parity` to complete; gives up early when
// *abort is set, and on a timeout sets *abort. Returns whether the phase
// completed.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, volatile uint32_t* abort) {
  if (bar_try(bar, parity)) return true;
  const uint64_t t0 = now_ns();
  for (uint32_t it = 0; it < kMaxTries; ++it) {
    if (bar_try(bar, parity)) return true;
    if (*abort) return false;
    if (now_ns() - t0 > kWaitNs) break;
  }
  *abort = 1u;
  return false;
}

// The same without the early exit: the wait for this CTA's own MMAs before
// its TMEM is given back, which must not be cut short by an abort.
__device__ __forceinline__ bool bar_wait_own(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = now_ns();
  for (uint32_t it = 0; it < kMaxTries; ++it) {
    if (bar_try(bar, parity)) return true;
    if (now_ns() - t0 > kWaitNs) break;
  }
  return false;
}

// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Warp-collective (.sync.aligned): the whole warp, converged.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   saddr(slot)), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}

// Warp-collective: three runs of 16 consecutive 32-bit TMEM columns of this
// thread's lane (the warp's lane quadrant), and the wait for them in the same
// statement, so no use of the registers can move above the wait. The column
// addresses must be the same in every lane of the warp: the load uses one.
__device__ __forceinline__ void tmem_ld3x16(uint32_t ta, uint32_t tb, uint32_t tc,
                                            uint32_t (&a)[16], uint32_t (&b)[16],
                                            uint32_t (&c)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%48];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
      "%28,%29,%30,%31}, [%49];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,"
      "%44,%45,%46,%47}, [%50];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]),
        "=r"(a[7]), "=r"(a[8]), "=r"(a[9]), "=r"(a[10]), "=r"(a[11]), "=r"(a[12]), "=r"(a[13]),
        "=r"(a[14]), "=r"(a[15]), "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]),
        "=r"(b[5]), "=r"(b[6]), "=r"(b[7]), "=r"(b[8]), "=r"(b[9]), "=r"(b[10]), "=r"(b[11]),
        "=r"(b[12]), "=r"(b[13]), "=r"(b[14]), "=r"(b[15]), "=r"(c[0]), "=r"(c[1]), "=r"(c[2]),
        "=r"(c[3]), "=r"(c[4]), "=r"(c[5]), "=r"(c[6]), "=r"(c[7]), "=r"(c[8]), "=r"(c[9]),
        "=r"(c[10]), "=r"(c[11]), "=r"(c[12]), "=r"(c[13]), "=r"(c[14]), "=r"(c[15])
      : "r"(ta), "r"(tb), "r"(tc)
      : "memory");
}

// The same for 8 columns of each of three accumulators.
__device__ __forceinline__ void tmem_ld3x8(uint32_t ta, uint32_t tb, uint32_t tc,
                                           uint32_t (&a)[8], uint32_t (&b)[8],
                                           uint32_t (&c)[8]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%24];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%25];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%26];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]),
        "=r"(a[7]), "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]), "=r"(b[5]),
        "=r"(b[6]), "=r"(b[7]), "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3]), "=r"(c[4]),
        "=r"(c[5]), "=r"(c[6]), "=r"(c[7])
      : "r"(ta), "r"(tb), "r"(tc)
      : "memory");
}

}  // namespace t5
}  // namespace rd
