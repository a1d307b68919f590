// batch.cu - rd_batch_*: many independent scenarios of uneven geometry run
// together. Each scenario is a chain (the same launch sequence a single
// stream uses); a run resets every chain and processes one input per
// scenario. The scenarios are spread largest-first over concurrent streams
// so that small ones fill the SMs the large ones leave idle, and the whole
// run - resets, launches, cross-stream ordering - is captured once into a
// CUDA graph and replayed, so the host issues one launch per run. The
// autotuner times the (streams, frames-per-launch) candidates with graph
// replays and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "rd_internal.h"

namespace {

#define BK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return rd::set_error(RD_EDEVICE, "%s failed: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

#define BS(call)                      \
  do {                                \
    rd_status s_ = (call);            \
    if (s_ != RD_OK) return s_;       \
  } while (0)

}  // namespace

struct rd_batch {
  std::vector<rd_chain*> chains;
  std::vector<rd_config> cfgs;
  rd_batch_options opt{};
  std::vector<cudaStream_t> streams;  // worker streams (32 at most)
  cudaStream_t root = nullptr;        // capture origin
  cudaEvent_t ev = nullptr;
  cudaGraphExec_t exec = nullptr;
  // what the graph was captured with
  std::vector<const rd_cplx16*> cap_adc;
  std::vector<uint64_t> cap_n;
  rd_batch_options cap_opt{};
  uint64_t cap_out_gen = 0;
  bool warmed = false;
  cudaStream_t last = nullptr;        // the stream of the last run
  // results exported by every run (rd_batch_set_outputs): the caller's
  // buffers, the events' and flits' device views, and per scenario a mapped
  // header (event count, timeout) and page-locked window flags
  std::vector<rd_output> outs;
  std::vector<rd_event*> out_ev;
  std::vector<uint32_t*> out_fl;
  rd::ExportHdr* hdr = nullptr;       // mapped, one per scenario
  rd::ExportHdr* hdr_dev = nullptr;
  unsigned* wflags = nullptr;         // page-locked, wf_off[i] + cap_cov_windows
  std::vector<size_t> wf_off;
  uint64_t out_gen = 0;
};

namespace {

constexpr uint32_t kMaxStreams = 32;

void drop_graph(rd_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

// A chain's frames per launch for the option's launch_frames, which counts
// frames of a 1024-point FFT: an N-point scenario takes launch_frames x 1024 /
// N frames (the same samples per launch), capped by its max_frames; 0 takes
// max_frames.
uint32_t scaled_frames(const rd_config& c, uint32_t launch_frames) {
  if (!launch_frames) return std::max(1u, c.max_frames);
  const uint64_t f = (uint64_t)launch_frames * 1024u / std::max(1u, c.n_fft);
  return (uint32_t)std::max<uint64_t>(1u, std::min<uint64_t>(f, c.max_frames));
}

// Scenario i's results into its registered host buffers, on s after its
// launches (rd::chain_export: the events and flits by a kernel through the
// mapped views, the window flags and sums by copies).
rd_status export_one(rd_batch* b, uint32_t i, cudaStream_t s) {
  const rd_output& o = b->outs[i];
  const rd_config& c = b->cfgs[i];
  const uint32_t nfl = rd_detection_flits(c.packet_w);
  uint64_t cap = o.cap_events;
  if (b->out_fl[i]) cap = std::min<uint64_t>(cap, o.cap_flits / nfl);
  const rd::ExportDst d{b->hdr_dev + i,         b->out_ev[i], b->out_fl[i],
                        cap,                    b->wflags + b->wf_off[i],
                        o.cap_cov_windows,      o.cov_acc,
                        o.cov_acc ? (size_t)o.cap_cov_windows * rd::chain_window_words(b->chains[i])
                                  : 0u};
  return rd::chain_export(b->chains[i], d, s);
}

// Enqueues one full run on `root`: fork to the worker streams, reset and
// process every scenario on its stream (exporting its results when outputs
// are registered), join back.
rd_status enqueue(rd_batch* b, const rd_cplx16* const* adc, const uint64_t* n, cudaStream_t root,
                  const rd_batch_options& o) {
  const uint32_t ns = std::max(1u, std::min<uint32_t>(o.n_streams, (uint32_t)b->streams.size()));
  for (size_t i = 0; i < b->chains.size(); ++i)
    BS(rd_chain_set_launch_frames(b->chains[i], scaled_frames(b->cfgs[i], o.launch_frames)));
  // largest first onto the least-loaded stream (cost ~ samples x channels x beams)
  std::vector<uint32_t> order(b->chains.size());
  std::iota(order.begin(), order.end(), 0u);
  auto cost = [&](uint32_t i) {
    const rd_config& c = b->cfgs[i];
    return (double)n[i] * c.n_chan * (1.0 + c.n_beams / 16.0);
  };
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return cost(a) > cost(c); });
  std::vector<double> load(ns, 0.0);
  std::vector<std::vector<uint32_t>> per(ns);
  for (uint32_t i : order) {
    const uint32_t k = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
    load[k] += cost(i);
    per[k].push_back(i);
  }
  BK(cudaEventRecord(b->ev, root));
  for (uint32_t k = 0; k < ns; ++k) BK(cudaStreamWaitEvent(b->streams[k], b->ev, 0));
  for (uint32_t k = 0; k < ns; ++k)
    for (uint32_t i : per[k]) {
      BS(rd_chain_reset(b->chains[i], b->streams[k]));
      BS(rd_chain_process_device(b->chains[i], adc[i], n[i], n[i], b->streams[k]));
      if (!b->outs.empty()) BS(export_one(b, i, b->streams[k]));
    }
  for (uint32_t k = 0; k < ns; ++k) {
    BK(cudaEventRecord(b->ev, b->streams[k]));
    BK(cudaStreamWaitEvent(root, b->ev, 0));
  }
  return RD_OK;
}

rd_status capture(rd_batch* b, const rd_cplx16* const* adc, const uint64_t* n,
                  const rd_batch_options& o) {
  drop_graph(b);
  cudaGraph_t g = nullptr;
  BK(cudaStreamBeginCapture(b->root, cudaStreamCaptureModeRelaxed));
  rd_status st = enqueue(b, adc, n, b->root, o);
  cudaError_t e = cudaStreamEndCapture(b->root, &g);
  if (st != RD_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess)
    return rd::set_error(RD_EDEVICE, "graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return rd::set_error(RD_EDEVICE, "graph instantiation failed: %s", cudaGetErrorString(e));
  }
  b->cap_adc.assign(adc, adc + b->chains.size());
  b->cap_n.assign(n, n + b->chains.size());
  b->cap_opt = o;
  b->cap_out_gen = b->out_gen;
  return RD_OK;
}

bool same_inputs(const rd_batch* b, const rd_cplx16* const* adc, const uint64_t* n) {
  for (size_t i = 0; i < b->chains.size(); ++i)
    if (b->cap_adc[i] != adc[i] || b->cap_n[i] != n[i]) return false;
  return true;
}

// One run with options o on stream s (graph or eager); the first run of a
// batch is eager so that every chain sizes its buffers outside a capture.
rd_status run_with(rd_batch* b, const rd_cplx16* const* adc, const uint64_t* n, cudaStream_t s,
                   const rd_batch_options& o) {
  rd::NvtxRange range("rd_batch_run");
  BK(cudaEventRecord(b->ev, s));
  BK(cudaStreamWaitEvent(b->root, b->ev, 0));
  if (!o.use_graph || !b->warmed) {
    BS(enqueue(b, adc, n, b->root, o));
    b->warmed = true;
    drop_graph(b);
  } else {
    const bool reuse = b->exec && same_inputs(b, adc, n) && b->cap_opt.n_streams == o.n_streams &&
                       b->cap_opt.launch_frames == o.launch_frames &&
                       b->cap_out_gen == b->out_gen;
    if (!reuse) BS(capture(b, adc, n, o));
    BK(cudaGraphLaunch(b->exec, b->root));
  }
  BK(cudaEventRecord(b->ev, b->root));
  BK(cudaStreamWaitEvent(s, b->ev, 0));
  b->last = s;
  return RD_OK;
}

}  // namespace

rd_status rd_batch_create(uint32_t n, const rd_config* cfgs, const rd_cplx16* const* coeff,
                          const rd_cplx16* const* weights, const rd_batch_options* opt,
                          rd_batch** out) {
  if (!out || !cfgs || !coeff || !weights || n == 0)
    return rd::set_error(RD_EINVAL, "rd_batch_create: bad argument");
  *out = nullptr;
  rd_batch* b = new rd_batch();
  b->opt = opt ? *opt : rd_batch_options{0, 0, 1};
  if (b->opt.n_streams == 0) b->opt.n_streams = 16;
  b->cfgs.assign(cfgs, cfgs + n);
  for (uint32_t i = 0; i < n; ++i) {
    rd_chain* ch = nullptr;
    rd_status st = rd_chain_create(&cfgs[i], &ch);
    if (st == RD_OK) st = rd_chain_set_coeff(ch, coeff[i]);
    if (st == RD_OK) st = rd_chain_set_weights(ch, weights[i]);
    if (st != RD_OK) {
      if (ch) rd_chain_destroy(ch);
      rd_batch_destroy(b);
      return st;
    }
    b->chains.push_back(ch);
  }
  b->streams.resize(kMaxStreams);
  for (cudaStream_t& s : b->streams)
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      s = nullptr;
      rd_batch_destroy(b);
      return rd::set_error(RD_EDEVICE, "rd_batch_create: stream creation failed");
    }
  if (cudaStreamCreateWithFlags(&b->root, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess) {
    rd_batch_destroy(b);
    return rd::set_error(RD_EDEVICE, "rd_batch_create: stream creation failed");
  }
  *out = b;
  return RD_OK;
}

namespace {

void free_outputs(rd_batch* b) {
  if (b->hdr) cudaFreeHost(b->hdr);
  if (b->wflags) cudaFreeHost(b->wflags);
  b->hdr = b->hdr_dev = nullptr;
  b->wflags = nullptr;
  b->outs.clear();
  b->out_ev.clear();
  b->out_fl.clear();
  b->wf_off.clear();
}

}  // namespace

void rd_batch_destroy(rd_batch* b) {
  if (!b) return;
  if (b->root) cudaStreamSynchronize(b->root);
  if (b->last) cudaStreamSynchronize(b->last);
  drop_graph(b);
  free_outputs(b);
  for (rd_chain* ch : b->chains) rd_chain_destroy(ch);
  for (cudaStream_t s : b->streams)
    if (s) cudaStreamDestroy(s);
  if (b->root) cudaStreamDestroy(b->root);
  if (b->ev) cudaEventDestroy(b->ev);
  delete b;
}

rd_status rd_batch_run(rd_batch* b, const rd_cplx16* const* adc_dev, const uint64_t* n_samples,
                       void* stream) {
  if (!b || !adc_dev || !n_samples) return rd::set_error(RD_EINVAL, "rd_batch_run: bad argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  return run_with(b, adc_dev, n_samples, s, b->opt);
}

rd_status rd_batch_run_sequential(rd_batch* b, const rd_cplx16* const* adc_dev,
                                  const uint64_t* n_samples, void* stream) {
  if (!b || !adc_dev || !n_samples)
    return rd::set_error(RD_EINVAL, "rd_batch_run_sequential: bad argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  for (size_t i = 0; i < b->chains.size(); ++i) {
    BS(rd_chain_set_launch_frames(b->chains[i], b->cfgs[i].max_frames));
    BS(rd_chain_reset(b->chains[i], s));
    BS(rd_chain_process_device(b->chains[i], adc_dev[i], n_samples[i], n_samples[i], s));
  }
  b->last = s;
  return RD_OK;
}

rd_status rd_batch_set_outputs(rd_batch* b, const rd_output* outs) {
  if (!b) return rd::set_error(RD_EINVAL, "rd_batch_set_outputs: null batch");
  if (b->last) BK(cudaStreamSynchronize(b->last));  // no run still writes the old ones
  drop_graph(b);
  free_outputs(b);
  ++b->out_gen;
  if (!outs) return RD_OK;
  const size_t n = b->chains.size();
  std::vector<rd_event*> ev(n, nullptr);
  std::vector<uint32_t*> fl(n, nullptr);
  std::vector<size_t> off(n + 1, 0);
  for (size_t i = 0; i < n; ++i) {
    const rd_output& o = outs[i];
    void* d = nullptr;
    if (!o.events || cudaHostGetDevicePointer(&d, o.events, 0) != cudaSuccess) {
      cudaGetLastError();
      return rd::set_error(RD_EINVAL, "rd_batch_set_outputs: scenario %zu: events are not "
                           "mapped page-locked memory", i);
    }
    ev[i] = static_cast<rd_event*>(d);
    if (o.flits) {
      if (cudaHostGetDevicePointer(&d, o.flits, 0) != cudaSuccess) {
        cudaGetLastError();
        return rd::set_error(RD_EINVAL, "rd_batch_set_outputs: scenario %zu: flits are not "
                             "mapped page-locked memory", i);
      }
      fl[i] = static_cast<uint32_t*>(d);
    }
    if (o.cov_acc) {
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, o.cov_acc) != cudaSuccess || a.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        return rd::set_error(RD_EINVAL, "rd_batch_set_outputs: scenario %zu: cov_acc is not "
                             "page-locked memory", i);
      }
    }
    off[i + 1] = off[i] + std::max<uint32_t>(o.cap_cov_windows, 1u);
  }
  void* h = nullptr;
  BK(cudaHostAlloc(&h, n * sizeof(rd::ExportHdr), cudaHostAllocMapped));
  b->hdr = static_cast<rd::ExportHdr*>(h);
  std::memset(b->hdr, 0, n * sizeof(rd::ExportHdr));
  void* hd = nullptr;
  if (cudaHostGetDevicePointer(&hd, h, 0) != cudaSuccess) {
    free_outputs(b);
    return rd::set_error(RD_EDEVICE, "rd_batch_set_outputs: no device view of the headers");
  }
  b->hdr_dev = static_cast<rd::ExportHdr*>(hd);
  void* w = nullptr;
  if (cudaHostAlloc(&w, off[n] * sizeof(unsigned), cudaHostAllocDefault) != cudaSuccess) {
    free_outputs(b);
    return rd::set_error(RD_EDEVICE, "rd_batch_set_outputs: page-locked allocation failed");
  }
  b->wflags = static_cast<unsigned*>(w);
  b->outs.assign(outs, outs + n);
  b->out_ev = ev;
  b->out_fl = fl;
  b->wf_off.assign(off.begin(), off.end() - 1);
  return RD_OK;
}

rd_status rd_batch_results(rd_batch* b, uint32_t i, rd_output* out) {
  if (!b || !out || i >= b->chains.size())
    return rd::set_error(RD_EINVAL, "rd_batch_results: bad argument");
  if (b->outs.empty()) return rd::set_error(RD_EINVAL, "rd_batch_results: no outputs registered");
  if (b->last) BK(cudaStreamSynchronize(b->last));
  const rd::ExportHdr h = b->hdr[i];
  if (h.dev_timeout)
    return rd::set_error(RD_ETIMEOUT, "a bounded wait inside a tensor-core kernel gave up; "
                         "results invalid");
  const rd_config& c = b->cfgs[i];
  const rd_output& o = b->outs[i];
  const uint32_t nfl = rd_detection_flits(c.packet_w);
  uint64_t kept = std::min<uint64_t>(h.n_events, rd::chain_call_cap(b->chains[i]));
  kept = std::min<uint64_t>(kept, o.cap_events);
  if (o.flits) kept = std::min<uint64_t>(kept, o.cap_flits / nfl);
  out->n_events = h.n_events;
  out->n_flits = h.n_events * nfl;
  out->flit_words = rd_flit_words(c.packet_w);
  out->n_frames = rd::chain_call_frames(b->chains[i]);
  const std::vector<rd_cov_window>& w = rd::chain_call_windows(b->chains[i]);
  out->n_cov_windows = (uint32_t)w.size();
  const uint32_t nw = std::min<uint32_t>((uint32_t)w.size(), out->cap_cov_windows);
  if (out->cov_windows)
    for (uint32_t k = 0; k < nw; ++k) {
      out->cov_windows[k] = w[k];
      out->cov_windows[k].sat_flags = (uint8_t)b->wflags[b->wf_off[i] + k];
    }
  const bool trunc = kept < h.n_events || nw < w.size();
  return trunc ? rd::set_error(RD_ETRUNC, "output capacity exceeded") : RD_OK;
}

rd_status rd_batch_fetch(rd_batch* b, uint32_t i, rd_output* out) {
  if (!b || i >= b->chains.size()) return rd::set_error(RD_EINVAL, "rd_batch_fetch: bad index");
  if (b->last) BK(cudaStreamSynchronize(b->last));
  return rd_chain_fetch(b->chains[i], out);
}

rd_status rd_batch_tune(rd_batch* b, const rd_cplx16* const* adc_dev, const uint64_t* n_samples,
                        uint32_t reps, rd_batch_options* chosen, double* best_ms) {
  if (!b || !adc_dev || !n_samples) return rd::set_error(RD_EINVAL, "rd_batch_tune: bad argument");
  if (reps == 0) reps = 3;
  // candidates in frames of a 1024-point FFT, up to the largest any chain takes
  uint64_t maxf = 1;
  for (const rd_config& c : b->cfgs)
    maxf = std::max<uint64_t>(maxf, ((uint64_t)c.max_frames * c.n_fft + 1023u) / 1024u);
  const uint32_t n = (uint32_t)b->chains.size();
  std::vector<uint32_t> stream_c, frame_c;
  for (uint32_t s : {1u, 4u, 8u, 16u, 32u})
    if (s <= std::max(1u, n)) stream_c.push_back(s);
  for (uint32_t f : {32u, 64u, 128u, 256u, 512u, 1024u, 4096u})
    if (f <= maxf) frame_c.push_back(f);
  if (frame_c.empty() || frame_c.back() < maxf) frame_c.push_back((uint32_t)std::min<uint64_t>(maxf, 1u << 30));
  cudaEvent_t t0, t1;
  BK(cudaEventCreate(&t0));
  BK(cudaEventCreate(&t1));
  cudaStream_t s = b->root;
  rd_batch_options best = b->opt;
  double best_t = 1e30;
  if (!b->warmed) {  // size every chain's buffers before the first capture
    rd_batch_options o = b->opt;
    o.use_graph = 0;
    BS(run_with(b, adc_dev, n_samples, s, o));
  }
  for (uint32_t ns : stream_c)
    for (uint32_t lf : frame_c) {
      rd_batch_options o{ns, lf, 1};
      BS(run_with(b, adc_dev, n_samples, s, o));  // capture + first replay
      std::vector<float> ts;
      for (uint32_t r = 0; r < reps; ++r) {
        BK(cudaEventRecord(t0, s));
        BS(run_with(b, adc_dev, n_samples, s, o));
        BK(cudaEventRecord(t1, s));
        BK(cudaEventSynchronize(t1));
        float ms = 0;
        BK(cudaEventElapsedTime(&ms, t0, t1));
        ts.push_back(ms);
      }
      std::sort(ts.begin(), ts.end());
      const double med = ts[ts.size() / 2];
      if (med < best_t) {
        best_t = med;
        best = o;
      }
    }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  b->opt = best;
  drop_graph(b);
  if (chosen) *chosen = best;
  if (best_ms) *best_ms = best_t;
  return RD_OK;
}

namespace {

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  return h;
}

// What the tuner's choice depends on: the device, this library, and every
// scenario's configuration and sample count (rd_config is all 32-bit fields,
// no padding).
uint64_t tune_key(const rd_batch* b, const uint64_t* n_samples) {
  uint64_t h = 1469598103934665603ull;
  int dev = 0;
  cudaDeviceProp pr{};
  if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&pr, dev) == cudaSuccess) {
    h = fnv1a(h, pr.name, strnlen(pr.name, sizeof(pr.name)));
    h = fnv1a(h, &pr.multiProcessorCount, sizeof(int));
    h = fnv1a(h, &pr.major, sizeof(int));
    h = fnv1a(h, &pr.minor, sizeof(int));
  } else {
    cudaGetLastError();
  }
  const char* v = rd_version();
  h = fnv1a(h, v, strlen(v));
  const uint32_t n = (uint32_t)b->cfgs.size();
  h = fnv1a(h, &n, sizeof(n));
  for (uint32_t i = 0; i < n; ++i) {
    h = fnv1a(h, &b->cfgs[i], sizeof(rd_config));
    h = fnv1a(h, &n_samples[i], sizeof(uint64_t));
  }
  return h;
}

}  // namespace

rd_status rd_batch_tune_cached(rd_batch* b, const rd_cplx16* const* adc_dev,
                               const uint64_t* n_samples, uint32_t reps, const char* cache_path,
                               rd_batch_options* chosen, double* best_ms, int* hit) {
  if (!b || !adc_dev || !n_samples || !cache_path)
    return rd::set_error(RD_EINVAL, "rd_batch_tune_cached: bad argument");
  if (hit) *hit = 0;
  const uint64_t key = tune_key(b, n_samples);
  // one line per tuned batch: key, streams, frames per launch, milliseconds;
  // the last line of a key wins
  bool found = false;
  unsigned f_ns = 0, f_lf = 0;
  double f_ms = 0;
  if (FILE* f = std::fopen(cache_path, "r")) {
    char line[256];
    while (std::fgets(line, sizeof(line), f)) {
      unsigned long long k = 0;
      unsigned ns = 0, lf = 0;
      double ms = 0;
      if (std::sscanf(line, "%llx %u %u %lf", &k, &ns, &lf, &ms) == 4 && k == key && ns >= 1 &&
          ns <= kMaxStreams && lf >= 1) {
        found = true;
        f_ns = ns;
        f_lf = lf;
        f_ms = ms;
      }
    }
    std::fclose(f);
  }
  if (found) {
    b->opt = rd_batch_options{f_ns, f_lf, 1};
    drop_graph(b);
    if (chosen) *chosen = b->opt;
    if (best_ms) *best_ms = f_ms;
    if (hit) *hit = 1;
    return RD_OK;
  }
  rd_batch_options o{};
  double ms = 0;
  const rd_status st = rd_batch_tune(b, adc_dev, n_samples, reps, &o, &ms);
  if (st != RD_OK) return st;
  // a cache that cannot be written costs the next caller a tuning, nothing more
  if (FILE* f = std::fopen(cache_path, "a")) {
    std::fprintf(f, "%016llx %u %u %.4f\n", (unsigned long long)key, o.n_streams,
                 o.launch_frames, ms);
    std::fclose(f);
  }
  if (chosen) *chosen = o;
  if (best_ms) *best_ms = ms;
  return RD_OK;
}

rd_status rd_batch_egress(rd_batch* b, uint32_t n_ports, uint32_t* ring_dev, uint64_t cap_per_port,
                          uint32_t* src_of_dev, uint64_t* port_count_dev, void* stream) {
  if (!b) return rd::set_error(RD_EINVAL, "rd_batch_egress: bad argument");
  if (!b->last) return rd::set_error(RD_EINVAL, "rd_batch_egress: the batch has not run");
  const uint32_t n = (uint32_t)b->chains.size();
  std::vector<rd_egress_source> src(n);
  const uint32_t pw = rd::chain_packet_w(b->chains[0]);
  for (uint32_t i = 0; i < n; ++i) {
    if (rd::chain_packet_w(b->chains[i]) != pw)
      return rd::set_error(RD_EINVAL, "rd_batch_egress: scenario %u has another packet width", i);
    src[i] = rd::chain_egress_source(b->chains[i]);
  }
  return rd::egress_merge(src.data(), n, pw, n_ports, ring_dev, cap_per_port, src_of_dev,
                          port_count_dev, stream ? (cudaStream_t)stream : cudaStreamLegacy);
}
