// cfar_static.cu - rd_cfar_run_static: the CFAR detector on caller-provided
// device buffers, with every piece of scratch in a file-scope static device
// array instead of an allocation.
//
// Who needs it: callers that are handed device memory but may not allocate
// any themselves - code running inside another framework's memory pool, a
// real-time loop where cudaMalloc/cudaFree would synchronise the device or
// miss a deadline, or a process whose allocator is locked down after start-up.
// Such a caller passes its cells, frame ids and event buffer; this entry point
// calls no cudaMalloc, cudaFree or allocating library routine.
//
// Limits and sharing: the scratch holds at most RD_STATIC_CFAR_MAX_FRAMES
// frames of at most RD_STATIC_CFAR_MAX_CELLS cells (about 1.6 MB, held by
// every GPU that loads the library until the process exits). Every call on a
// device uses the same array and leaves its contents behind; the per-call
// counters are cleared at the start of each call. Two calls whose work
// overlaps on the GPU (different streams, no ordering between them) race on
// the array and give wrong results.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress, with that device current. In host code the
// array's name is only a host-side stand-in, never a device address. Make the
// first call on a device before any stream capture.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "rd_internal.h"

namespace {

struct StaticCfarScratch {
  rd::DevStats stats;
  unsigned long long totals[RD_STATIC_CFAR_MAX_FRAMES];
  uint32_t counts[RD_STATIC_CFAR_MAX_FRAMES];
  uint32_t detsup[RD_STATIC_CFAR_MAX_FRAMES];
  uint32_t mask[RD_STATIC_CFAR_MAX_FRAMES * (RD_STATIC_CFAR_MAX_CELLS / 32)];
  uint4 slots[RD_STATIC_CFAR_MAX_FRAMES * rd::kCfarSlots];
};

std::mutex g_mu;
constexpr int kMaxDevices = 64;
StaticCfarScratch* g_addr[kMaxDevices] = {};

}  // namespace

static __device__ __align__(256) unsigned char g_cfar_scratch[sizeof(StaticCfarScratch)];

namespace {

__global__ void k_static_count_out(const rd::DevStats* st, unsigned long long* n_events) {
  *n_events = st->events_call;
}

// Device address of the scratch on the current device (looked up once).
cudaError_t scratch_address(StaticCfarScratch** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cfar_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<StaticCfarScratch*>(p);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" rd_status rd_cfar_run_static(const int64_t* cells, uint32_t n, uint32_t frames,
                                        const rd_config* cfg, const uint32_t* frame_ids,
                                        rd_event* events, uint64_t cap, uint64_t* n_events,
                                        void* stream) {
  if (!cells || !cfg || !frame_ids || !events || !n_events)
    return rd::set_error(RD_EINVAL, "rd_cfar_run_static: null argument");
  if (n == 0 || n > RD_STATIC_CFAR_MAX_CELLS)
    return rd::set_error(RD_EINVAL, "rd_cfar_run_static: %u cells per frame, the static scratch "
                         "holds 1..%u", n, RD_STATIC_CFAR_MAX_CELLS);
  if (frames > RD_STATIC_CFAR_MAX_FRAMES)
    return rd::set_error(RD_EINVAL, "rd_cfar_run_static: %u frames, the static scratch holds at "
                         "most %u", frames, RD_STATIC_CFAR_MAX_FRAMES);
  StaticCfarScratch* sc = nullptr;
  cudaError_t e = scratch_address(&sc);
  if (e != cudaSuccess)
    return rd::set_error(RD_EDEVICE, "rd_cfar_run_static: cudaGetSymbolAddress failed: %s",
                         cudaGetErrorString(e));
  cudaStream_t s = (cudaStream_t)stream;
  // the counters the kernels accumulate start at zero each call
  e = cudaMemsetAsync(&sc->stats, 0, sizeof(rd::DevStats), s);
  if (e != cudaSuccess)
    return rd::set_error(RD_EDEVICE, "rd_cfar_run_static: %s", cudaGetErrorString(e));
  rd::CfarParams p{};
  p.cells_i64 = cells;
  p.frames = frames;
  p.n = n;
  p.beams = 1;
  p.frame_ids = frame_ids;
  p.enable = cfg->cfar_enable != 0;
  p.go = cfg->cfar_mode == RD_CFAR_GO;
  p.dense = cfg->cfar_out_mode == RD_CFAR_DENSE;
  p.gl = cfg->guard_lead < cfg->max_guard ? cfg->guard_lead : cfg->max_guard;
  p.gg = cfg->guard_lag < cfg->max_guard ? cfg->guard_lag : cfg->max_guard;
  p.rl = cfg->ref_lead < cfg->max_ref ? cfg->ref_lead : cfg->max_ref;
  p.rg = cfg->ref_lag < cfg->max_ref ? cfg->ref_lag : cfg->max_ref;
  p.alpha = cfg->alpha;
  p.counts = sc->counts;
  p.detsup = sc->detsup;
  p.mask = sc->mask;
  p.totals = sc->totals;
  p.slots = sc->slots;
  p.vec = (n % 4u) == 0 && reinterpret_cast<uintptr_t>(cells) % 16u == 0;
  p.ev16 = reinterpret_cast<uintptr_t>(events) % 16u == 0;
  p.events = events;
  p.cap = cap;
  p.stats = &sc->stats;
  if (frames) rd::launch_cfar(p, s);
  k_static_count_out<<<1, 1, 0, s>>>(&sc->stats, reinterpret_cast<unsigned long long*>(n_events));
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return rd::set_error(RD_EDEVICE, "rd_cfar_run_static: launch failed: %s",
                         cudaGetErrorString(e));
  return RD_OK;
}
