// fabric.cu - egress aggregation of many streams' detection packets into
// per-port DMA rings, and the packet fabric's deterministic route.
//
// Every egress port is fed by one round-robin arbiter over the sources that
// target it, the arbiter design the reference fabric uses at every level
// (rtl/packet/pkt_rr_arb.sv:1-150): grant the lowest requesting index at or
// after the pointer, then move the pointer one past the grant. With every
// source's packets queued that grants the port's sources in cyclic order and
// skips those whose queue has run dry, so packet r of source s leaves port d
// at position
//     sum over sources t of port d of min(n_t, r)  +  #{t < s of port d : n_t > r}
// and each source's packets leave in their own order - the per-(src, VC,
// dest) ordering property the reference's scoreboard checks
// (model/cpp/packet/packet_model.hpp:475-500). The kernel places every packet
// at that position directly, all packets in parallel; a warp moves 32 packets
// together so that its loads and stores run over whole packets.
#include <cuda_runtime.h>

#include "rd_internal.h"

namespace {

struct EgressSrc {
  const uint32_t* flits;
  const unsigned long long* count;  // device counter, or null
  unsigned long long n;             // packets, or the most *count may give
  uint32_t dest;
  uint32_t pad;
};

struct EgressParams {
  EgressSrc src[RD_EGRESS_MAX_SRC];
  uint32_t n_src, words, n_ports;
  unsigned long long cap;           // packets per port ring
  uint32_t* ring;                   // [n_ports][cap][words]
  uint32_t* src_of;                 // [n_ports][cap] or null
  unsigned long long* port_count;   // [n_ports]
};

constexpr uint32_t kThreads = 512;
static_assert(RD_EGRESS_MAX_SRC <= kThreads, "one staging thread per source");

__global__ void __launch_bounds__(kThreads) k_egress_merge(const __grid_constant__ EgressParams p) {
  __shared__ unsigned long long s_n[RD_EGRESS_MAX_SRC], s_pre[RD_EGRESS_MAX_SRC + 1];
  __shared__ const uint32_t* s_ptr[RD_EGRESS_MAX_SRC];
  __shared__ uint32_t s_dest[RD_EGRESS_MAX_SRC];
  __shared__ unsigned long long s_warp[kThreads / 32];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, wid = tid >> 5;

  // packets per source, and their exclusive prefix (a block scan)
  unsigned long long n = 0;
  if (tid < p.n_src) {
    const EgressSrc& e = p.src[tid];
    n = e.n;
    if (e.count) n = min(*e.count, n);
    s_n[tid] = n;
    s_ptr[tid] = e.flits;
    s_dest[tid] = e.dest;
  }
  unsigned long long incl = n;
  for (uint32_t o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  unsigned long long before = 0;
  for (uint32_t w = 0; w < wid; ++w) before += s_warp[w];
  if (tid < p.n_src) s_pre[tid] = before + incl - n;
  if (tid == kThreads - 1) s_pre[p.n_src] = before + incl;
  __syncthreads();
  const unsigned long long total = s_pre[p.n_src];

  if (blockIdx.x == 0)
    for (uint32_t d = tid; d < p.n_ports; d += kThreads) {
      unsigned long long c = 0;
      for (uint32_t t = 0; t < p.n_src; ++t)
        if (s_dest[t] == d) c += s_n[t];
      p.port_count[d] = c;
    }

  const uint32_t W = p.words;
  const unsigned long long n_warps = (unsigned long long)gridDim.x * (kThreads / 32);
  for (unsigned long long base = ((unsigned long long)blockIdx.x * (kThreads / 32) + wid) * 32;
       base < total; base += n_warps * 32) {
    const unsigned long long i = base + lane;
    bool ok = i < total;
    uint32_t s = 0;
    unsigned long long r = 0, out = 0;
    if (ok) {
      // the source holding packet i: the last s with s_pre[s] <= i (it has
      // s_pre[s + 1] > i, so it is not empty)
      uint32_t lo = 0, hi = p.n_src;  // s_pre[lo] <= i < s_pre[hi]
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_pre[mid] <= i) lo = mid; else hi = mid;
      }
      s = lo;
      r = i - s_pre[s];
      const uint32_t d = s_dest[s];
      unsigned long long pos = 0;
      for (uint32_t t = 0; t < p.n_src; ++t) {
        if (s_dest[t] != d) continue;
        const unsigned long long m = s_n[t];
        pos += m < r ? m : r;
        if (t < s && m > r) ++pos;
      }
      ok = pos < p.cap;
      out = (unsigned long long)d * p.cap + pos;
      if (ok && p.src_of) p.src_of[out] = s;
    }
    // 32 packets, W words each, moved by the whole warp: every lane runs the
    // same W iterations
    for (uint32_t j = lane; j < 32u * W; j += 32u) {
      const uint32_t q = j / W, w = j - q * W;
      const uint32_t sq = __shfl_sync(0xffffffffu, s, q);
      const unsigned long long rq = __shfl_sync(0xffffffffu, r, q);
      const unsigned long long oq = __shfl_sync(0xffffffffu, out, q);
      const int okq = __shfl_sync(0xffffffffu, (int)ok, q);
      if (okq) p.ring[oq * W + w] = __ldg(s_ptr[sq] + rq * W + w);
    }
  }
}

}  // namespace

namespace rd {

rd_status egress_merge(const rd_egress_source* src, uint32_t n_src, uint32_t packet_w,
                       uint32_t n_ports, uint32_t* ring_dev, uint64_t cap_per_port,
                       uint32_t* src_of_dev, uint64_t* port_count_dev, cudaStream_t st) {
  if (!src || !ring_dev || !port_count_dev || n_src == 0 || n_ports == 0)
    return set_error(RD_EINVAL, "rd_egress_merge: bad argument");
  if (n_src > RD_EGRESS_MAX_SRC)
    return set_error(RD_EINVAL, "rd_egress_merge: %u sources, at most %u", n_src,
                     RD_EGRESS_MAX_SRC);
  if (packet_w < 64 || packet_w > 512 || packet_w % 32)
    return set_error(RD_EINVAL, "rd_egress_merge: packet_w %u", packet_w);
  // ring word offsets (port x cap + position) x words must stay far inside
  // 64 bits
  const uint32_t words = rd_detection_flits(packet_w) * rd_flit_words(packet_w);
  if (cap_per_port > (~0ull >> 8) / n_ports / words)
    return set_error(RD_EINVAL, "rd_egress_merge: ring too large");
  EgressParams p{};  // 16 KB, copied into the launch
  for (uint32_t s = 0; s < n_src; ++s) {
    if (!src[s].flits && (src[s].n_packets || src[s].count_dev))
      return set_error(RD_EINVAL, "rd_egress_merge: source %u has no flits", s);
    if (src[s].dest >= n_ports)
      return set_error(RD_EINVAL, "rd_egress_merge: source %u targets port %u of %u", s,
                       src[s].dest, n_ports);
    p.src[s] = EgressSrc{src[s].flits, (const unsigned long long*)src[s].count_dev,
                         src[s].n_packets, src[s].dest, 0};
  }
  p.n_src = n_src;
  p.words = words;
  p.n_ports = n_ports;
  p.cap = cap_per_port;
  p.ring = ring_dev;
  p.src_of = src_of_dev;
  p.port_count = (unsigned long long*)port_count_dev;
  static int n_sm = 0;
  if (!n_sm) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return set_error(RD_EDEVICE, "rd_egress_merge: no usable CUDA device");
  }
  // two resident blocks per SM cover any packet count by striding
  k_egress_merge<<<2 * n_sm, kThreads, 0, st>>>(p);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? RD_OK
                          : set_error(RD_EDEVICE, "rd_egress_merge: %s", cudaGetErrorString(e));
}

}  // namespace rd

extern "C" rd_status rd_egress_merge(const rd_egress_source* src, uint32_t n_src,
                                     uint32_t packet_w, uint32_t n_ports, uint32_t* ring_dev,
                                     uint64_t cap_per_port, uint32_t* src_of_dev,
                                     uint64_t* port_count_dev, void* stream) {
  if (!rd_device_ok()) return rd::set_error(RD_EDEVICE, "rd_egress_merge: no usable CUDA device");
  return rd::egress_merge(src, n_src, packet_w, n_ports, ring_dev, cap_per_port, src_of_dev,
                          port_count_dev, stream ? (cudaStream_t)stream : cudaStreamLegacy);
}

// The wires a packet from `src` to `dest` occupies in a `stages`-stage
// radix-`radix` butterfly (packet_model.hpp:266-303): path[0] = src and
// path[s + 1] = the wire out of stage s. Stage s switches on digit
// stages - 1 - s: the switch is the current wire with that digit removed,
// and its output is the switch with the destination's digit put back there.
// After the last stage every digit is the destination's, so the route ends at
// dest from every source.
extern "C" rd_status rd_route_path(uint32_t src, uint32_t dest, uint32_t radix, uint32_t stages,
                                   uint32_t* path) {
  if (!path || radix < 2 || stages == 0 || stages > 32)
    return rd::set_error(RD_EINVAL, "rd_route_path: bad argument");
  uint64_t ports = 1;
  for (uint32_t i = 0; i < stages && ports <= 0xFFFFFFFFull; ++i) ports *= radix;
  if (ports > 0xFFFFFFFFull || src >= ports || dest >= ports)
    return rd::set_error(RD_EINVAL, "rd_route_path: port out of range");
  uint32_t cur = src;
  path[0] = src;
  for (uint32_t s = 0; s < stages; ++s) {
    uint32_t scale = 1;
    for (uint32_t i = 0; i < stages - 1 - s; ++i) scale *= radix;
    const uint32_t sw = cur / (scale * radix) * scale + cur % scale;
    const uint32_t digit = dest / scale % radix;
    cur = sw / scale * scale * radix + digit * scale + sw % scale;
    path[s + 1] = cur;
  }
  return RD_OK;
}
