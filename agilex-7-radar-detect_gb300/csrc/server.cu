// server.cu - rd_server_*: a request loop over many streams whose chain state
// stays on the device between requests.
//
// Admission. The server reserves its request slots (one device input buffer
// each) against the HBM budget at create; a stream is admitted at open when
// its chain's footprint (rd_chain_footprint) fits what is left, else
// RD_ENOMEM; close returns it.
//
// Scheduling. Submitted requests wait in one FIFO. A request starts when its
// stream has no request on the device and a slot is free: its samples go
// host -> slot over the stream's CUDA stream, the chain runs after the copy,
// and an event marks the end. Requests of different streams therefore
// overlap on the device and are admitted the moment a slot frees, without
// waiting for a batch to drain (continuous batching); requests of one stream
// run in order, because each one continues the stream's state. Polling
// collects finished requests and starts whatever can start next.
//
// Outputs. Behind each request's launches its stream also exports the
// outputs into host memory (rd::chain_export): the event count and up to
// kExpEvents events and packets into a mapped page-locked block, the closed
// windows' sums by DMA into a page-locked block, so that polling reads counts
// from host memory and never waits on a copy. A request with more events
// than a block holds is read with synchronous copies instead (its stream
// starts nothing before it is collected, so the chain still holds them).
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <deque>
#include <utility>
#include <unordered_map>
#include <vector>

#include "rd_internal.h"

namespace {

#define SK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return rd::set_error(RD_EDEVICE, "%s failed: %s", #call, cudaGetErrorString(e_));   \
  } while (0)

// A vector whose resize leaves new elements uninitialised (the outputs are
// written by the device copy right after).
template <typename T>
struct NoInit {
  using value_type = T;
  NoInit() = default;
  template <typename U>
  NoInit(const NoInit<U>&) {}
  T* allocate(size_t n) { return static_cast<T*>(::operator new(n * sizeof(T))); }
  void deallocate(T* p, size_t) { ::operator delete(p); }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    if constexpr (sizeof...(A) > 0) ::new ((void*)p) U(std::forward<A>(a)...);
  }
  template <typename U>
  bool operator==(const NoInit<U>&) const { return true; }
  template <typename U>
  bool operator!=(const NoInit<U>&) const { return false; }
};
template <typename T>
using RawVec = std::vector<T, NoInit<T>>;

// A page-locked block for a request's covariance window sums: they are the
// one large output (34 MB for a full-scale window), and a page-locked
// destination takes them by DMA instead of through a staging copy.
struct PinnedBuf {
  int64_t* p = nullptr;
  size_t cap = 0;  // int64 words
  size_t len = 0;
};

// A mapped page-locked block a request's events and packets are exported
// into: header, kExpEvents events, their packets at the widest packet format,
// kExpWindows window flags.
constexpr uint64_t kExpEvents = 4096;
constexpr uint32_t kExpWindows = 1024;
constexpr uint32_t kExpPkWords = 34;  // detection packet words at 512-bit flits, the most
struct ExportBlock {
  void* host = nullptr;
  rd::ExportHdr* hdr = nullptr;  // host views
  rd_event* ev = nullptr;
  uint32_t* fl = nullptr;
  unsigned* wf = nullptr;
  rd::ExportHdr* d_hdr = nullptr;  // device views
  rd_event* d_ev = nullptr;
  uint32_t* d_fl = nullptr;
};
constexpr size_t kExpHdrBytes = 256;
constexpr size_t kExpEvBytes = kExpEvents * sizeof(rd_event);
constexpr size_t kExpFlBytes = kExpEvents * kExpPkWords * 4;
constexpr size_t kExpBytes = kExpHdrBytes + kExpEvBytes + kExpFlBytes + kExpWindows * 4;

struct Request {
  uint64_t id = 0;
  uint32_t stream = 0;
  uint64_t n = 0;
  int host_buf = -1;
  int slot = -1;
  double t_submit = 0, t_start = 0, t_done = 0;
  rd_status status = RD_OK;
  bool done = false;
  RawVec<rd_event> events;
  RawVec<uint32_t> flits;
  RawVec<rd_cov_window> windows;
  PinnedBuf cov;
  ExportBlock* xb = nullptr;  // the exported outputs (null: read synchronously)
  uint64_t n_events = 0, n_flits = 0, n_kept = 0;
  uint32_t n_windows = 0, flit_words = 0;
};

// Output buffers of a finished request, kept (capacity included) for the
// next one, so that steady serving allocates nothing.
struct OutBufs {
  RawVec<rd_event> events;
  RawVec<uint32_t> flits;
  RawVec<rd_cov_window> windows;
};

struct StreamState {
  rd_chain* ch = nullptr;
  rd_config cfg{};
  cudaStream_t cs = nullptr;
  uint64_t footprint = 0;
  uint32_t n_pairs = 0;
  bool open = false;
  bool busy = false;
  uint32_t outstanding = 0;
};

struct Slot {
  rd_cplx16* dev = nullptr;
  cudaEvent_t done = nullptr;
  uint64_t req = 0;
  bool used = false;
};

}  // namespace

struct rd_server {
  rd_server_config cfg{};
  uint64_t used = 0;
  size_t slot_words = 0;
  std::vector<StreamState> streams;
  std::vector<Slot> slots;
  std::vector<rd_cplx16*> host;   // pinned staging, queue_cap buffers
  std::vector<int> free_host;
  std::unordered_map<uint64_t, Request> reqs;
  std::vector<OutBufs> pool;      // output buffers of finished requests, reused
  std::vector<PinnedBuf> cov_pool;  // page-locked window-sum blocks, reused
  std::vector<ExportBlock*> xpool;  // mapped export blocks, reused
  std::deque<uint64_t> waiting;   // submitted, not started (submission order)
  std::vector<rd_completion> finished;
  uint64_t next_id = 1;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now() const {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

// Removes request `it`, keeping its output buffers (capacity included) for
// later requests.
void retire(rd_server* s, std::unordered_map<uint64_t, Request>::iterator it) {
  if (it == s->reqs.end()) return;
  Request& r = it->second;
  const size_t keep = (size_t)s->cfg.queue_cap + s->cfg.max_inflight;
  if (s->pool.size() < keep)
    s->pool.push_back(OutBufs{std::move(r.events), std::move(r.flits), std::move(r.windows)});
  if (r.cov.p) {
    if (s->cov_pool.size() < keep) s->cov_pool.push_back(PinnedBuf{r.cov.p, r.cov.cap, 0});
    else cudaFreeHost(r.cov.p);
  }
  if (r.xb) {
    if (s->xpool.size() < keep) {
      s->xpool.push_back(r.xb);
    } else {
      cudaFreeHost(r.xb->host);
      delete r.xb;
    }
  }
  s->reqs.erase(it);
}

ExportBlock* take_xblock(rd_server* s) {
  if (!s->xpool.empty()) {
    ExportBlock* b = s->xpool.back();
    s->xpool.pop_back();
    return b;
  }
  ExportBlock* b = new ExportBlock();
  if (cudaHostAlloc(&b->host, kExpBytes, cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return nullptr;
  }
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, b->host, 0) != cudaSuccess) {
    cudaGetLastError();
    cudaFreeHost(b->host);
    delete b;
    return nullptr;
  }
  char* h = static_cast<char*>(b->host);
  char* g = static_cast<char*>(d);
  b->hdr = reinterpret_cast<rd::ExportHdr*>(h);
  b->d_hdr = reinterpret_cast<rd::ExportHdr*>(g);
  b->ev = reinterpret_cast<rd_event*>(h + kExpHdrBytes);
  b->d_ev = reinterpret_cast<rd_event*>(g + kExpHdrBytes);
  b->fl = reinterpret_cast<uint32_t*>(h + kExpHdrBytes + kExpEvBytes);
  b->d_fl = reinterpret_cast<uint32_t*>(g + kExpHdrBytes + kExpEvBytes);
  b->wf = reinterpret_cast<unsigned*>(h + kExpHdrBytes + kExpEvBytes + kExpFlBytes);
  return b;
}

// A page-locked block of at least `need` words for the request's window
// sums: a kept block that holds it (the smallest), else a new one.
rd_status take_cov(rd_server* s, Request& r, size_t need) {
  if (need <= r.cov.cap) return RD_OK;
  size_t best = s->cov_pool.size();
  for (size_t k = 0; k < s->cov_pool.size(); ++k)
    if (s->cov_pool[k].cap >= need &&
        (best == s->cov_pool.size() || s->cov_pool[k].cap < s->cov_pool[best].cap))
      best = k;
  PinnedBuf b{};
  if (best < s->cov_pool.size()) {
    b = s->cov_pool[best];
    s->cov_pool.erase(s->cov_pool.begin() + (ptrdiff_t)best);
  } else if (cudaMallocHost(&b.p, need * sizeof(int64_t)) == cudaSuccess) {
    b.cap = need;
  } else {
    cudaGetLastError();
    return rd::set_error(RD_ENOMEM, "rd_server: no page-locked memory for window sums");
  }
  if (r.cov.p) s->cov_pool.push_back(PinnedBuf{r.cov.p, r.cov.cap, 0});
  r.cov = b;
  return RD_OK;
}

rd_status start_ready(rd_server* s) {
  for (auto it = s->waiting.begin(); it != s->waiting.end();) {
    Request& r = s->reqs[*it];
    StreamState& st = s->streams[r.stream];
    if (st.busy) {
      ++it;
      continue;
    }
    int slot = -1;
    for (size_t k = 0; k < s->slots.size(); ++k)
      if (!s->slots[k].used) {
        slot = (int)k;
        break;
      }
    if (slot < 0) break;
    Slot& sl = s->slots[slot];
    rd::NvtxRange range("rd_server request start");
    const size_t words = (size_t)st.cfg.n_chan * r.n;
    SK(cudaMemcpyAsync(sl.dev, s->host[r.host_buf], words * 4, cudaMemcpyHostToDevice, st.cs));
    rd_status rs = rd_chain_process_device(st.ch, sl.dev, r.n, r.n, st.cs);
    if (rs != RD_OK) return rs;
    // the outputs follow the launches into host memory (see the top of the
    // file); without a block the request is read synchronously when it ends
    {
      const std::vector<rd_cov_window>& w = rd::chain_call_windows(st.ch);
      const size_t per = rd::chain_window_words(st.ch);
      const uint32_t pk = rd_detection_flits(st.cfg.packet_w) * rd_flit_words(st.cfg.packet_w);
      ExportBlock* xb = w.size() <= kExpWindows && pk <= kExpPkWords ? take_xblock(s) : nullptr;
      if (xb && take_cov(s, r, w.size() * per) == RD_OK) {
        r.windows.assign(w.begin(), w.end());
        r.cov.len = w.size() * per;
        rd::ExportDst d{xb->d_hdr, xb->d_ev, xb->d_fl, kExpEvents, xb->wf, kExpWindows,
                        r.cov.p, r.cov.cap};
        rs = rd::chain_export(st.ch, d, st.cs);
        if (rs != RD_OK) {
          s->xpool.push_back(xb);
          return rs;
        }
        r.xb = xb;
      } else if (xb) {
        s->xpool.push_back(xb);
      }
    }
    SK(cudaEventRecord(sl.done, st.cs));
    sl.used = true;
    sl.req = r.id;
    r.slot = slot;
    r.t_start = s->now();
    st.busy = true;
    it = s->waiting.erase(it);
  }
  return RD_OK;
}

// Outputs of a finished request, read from its chain: the counts first
// (no buffers), then the outputs into buffers of exactly that size.
rd_status collect(rd_server* s, Request& r) {
  StreamState& st = s->streams[r.stream];
  const rd_config& c = st.cfg;
  const uint32_t nfl = rd_detection_flits(c.packet_w), words = rd_flit_words(c.packet_w);
  rd_output q{};
  rd_status rs = rd_chain_fetch(st.ch, &q);
  if (rs != RD_OK && rs != RD_ETRUNC) return rs;
  const size_t per = (size_t)c.n_fft * std::max(st.n_pairs, 1u) * 2;
  r.events.resize(q.n_events);
  r.flits.resize(q.n_events * nfl * words);
  r.windows.resize(q.n_cov_windows);
  const size_t need = (size_t)q.n_cov_windows * per;
  if (need > r.cov.cap) {  // a kept block that holds it, else a new one
    size_t best = s->cov_pool.size();
    for (size_t k = 0; k < s->cov_pool.size(); ++k)
      if (s->cov_pool[k].cap >= need && (best == s->cov_pool.size() ||
                                         s->cov_pool[k].cap < s->cov_pool[best].cap))
        best = k;
    PinnedBuf b{};
    if (best < s->cov_pool.size()) {
      b = s->cov_pool[best];
      s->cov_pool.erase(s->cov_pool.begin() + (ptrdiff_t)best);
    } else if (cudaMallocHost(&b.p, need * sizeof(int64_t)) == cudaSuccess) {
      b.cap = need;
    } else {
      return rd::set_error(RD_ENOMEM, "rd_server: no page-locked memory for window sums");
    }
    if (r.cov.p) s->cov_pool.push_back(PinnedBuf{r.cov.p, r.cov.cap, 0});
    r.cov = b;
  }
  r.cov.len = need;
  rd_output o{};
  o.events = r.events.data();
  o.cap_events = q.n_events;
  o.flits = r.flits.data();
  o.cap_flits = q.n_events * nfl;
  o.cov_windows = r.windows.data();
  o.cov_acc = r.cov.p;
  o.cap_cov_windows = q.n_cov_windows;
  rs = rd_chain_fetch(st.ch, &o);
  r.n_events = o.n_events;
  r.n_flits = o.n_flits;
  r.n_windows = o.n_cov_windows;
  r.flit_words = o.flit_words;
  return rs;  // RD_ETRUNC: the chain's own event buffer overflowed
}

// A finished request whose outputs were exported: counts from host memory;
// more events than the block kept means the synchronous read after all.
rd_status finish_export(rd_server* s, Request& r) {
  StreamState& st = s->streams[r.stream];
  const rd_config& c = st.cfg;
  const rd::ExportHdr h = *r.xb->hdr;
  if (h.dev_timeout)
    return rd::set_error(RD_ETIMEOUT, "a bounded wait inside a tensor-core kernel gave up; "
                         "results invalid");
  const uint64_t cap = rd::chain_call_cap(st.ch);
  const uint64_t avail = std::min<uint64_t>(h.n_events, cap);
  if (avail > kExpEvents) {
    s->xpool.push_back(r.xb);
    r.xb = nullptr;
    return collect(s, r);
  }
  const uint32_t nfl = rd_detection_flits(c.packet_w);
  r.n_events = h.n_events;
  r.n_flits = h.n_events * nfl;
  r.n_kept = avail;
  r.flit_words = rd_flit_words(c.packet_w);
  r.n_windows = (uint32_t)r.windows.size();
  for (uint32_t w = 0; w < r.n_windows; ++w) r.windows[w].sat_flags = (uint8_t)r.xb->wf[w];
  return h.n_events > cap ? rd::set_error(RD_ETRUNC, "output capacity exceeded") : RD_OK;
}

}  // namespace

rd_status rd_server_create(const rd_server_config* cfg, rd_server** out) {
  if (!cfg || !out || cfg->max_inflight == 0 || cfg->queue_cap < cfg->max_inflight ||
      cfg->max_chan == 0 || cfg->max_request_samples == 0)
    return rd::set_error(RD_EINVAL, "rd_server_create: bad configuration");
  *out = nullptr;
  if (!rd_device_ok()) return rd::set_error(RD_EDEVICE, "rd_server_create: no usable CUDA device");
  rd_server* s = new rd_server();
  s->cfg = *cfg;
  s->slot_words = (size_t)cfg->max_chan * cfg->max_request_samples;
  const uint64_t slot_bytes = (uint64_t)s->slot_words * 4;
  if ((uint64_t)cfg->max_inflight * slot_bytes > cfg->hbm_budget) {
    delete s;
    return rd::set_error(RD_ENOMEM, "rd_server_create: %u request slots of %llu bytes exceed the "
                         "budget", cfg->max_inflight, (unsigned long long)slot_bytes);
  }
  s->slots.resize(cfg->max_inflight);
  for (Slot& sl : s->slots) {
    if (cudaMalloc(&sl.dev, slot_bytes) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
      rd_server_destroy(s);
      return rd::set_error(RD_ENOMEM, "rd_server_create: slot allocation failed");
    }
  }
  s->used = (uint64_t)cfg->max_inflight * slot_bytes;
  s->host.resize(cfg->queue_cap, nullptr);
  for (uint32_t k = 0; k < cfg->queue_cap; ++k) {
    if (cudaMallocHost(&s->host[k], slot_bytes) != cudaSuccess) {
      rd_server_destroy(s);
      return rd::set_error(RD_ENOMEM, "rd_server_create: pinned staging allocation failed");
    }
    s->free_host.push_back((int)k);
  }
  *out = s;
  return RD_OK;
}

void rd_server_destroy(rd_server* s) {
  if (!s) return;
  for (StreamState& st : s->streams)
    if (st.open) {
      cudaStreamSynchronize(st.cs);
      rd_chain_destroy(st.ch);  // and with it the stream
    }
  for (Slot& sl : s->slots) {
    if (sl.dev) cudaFree(sl.dev);
    if (sl.done) cudaEventDestroy(sl.done);
  }
  for (rd_cplx16* h : s->host)
    if (h) cudaFreeHost(h);
  for (PinnedBuf& b : s->cov_pool) cudaFreeHost(b.p);
  for (ExportBlock* b : s->xpool) {
    cudaFreeHost(b->host);
    delete b;
  }
  for (auto& kv : s->reqs) {
    if (kv.second.cov.p) cudaFreeHost(kv.second.cov.p);
    if (kv.second.xb) {
      cudaFreeHost(kv.second.xb->host);
      delete kv.second.xb;
    }
  }
  delete s;
}

rd_status rd_stream_open(rd_server* s, const rd_config* cfg, const rd_cplx16* coeff,
                         const rd_cplx16* weights, uint32_t* stream_id) {
  if (!s || !cfg || !coeff || !weights || !stream_id)
    return rd::set_error(RD_EINVAL, "rd_stream_open: null argument");
  rd_status st = rd_config_validate(cfg);
  if (st != RD_OK) return st;
  if (cfg->n_chan > s->cfg.max_chan)
    return rd::set_error(RD_EINVAL, "rd_stream_open: %u channels, the server's slots hold %u",
                         cfg->n_chan, s->cfg.max_chan);
  const uint64_t frames = s->cfg.max_request_samples / cfg->n_fft;
  const uint64_t fp = rd_chain_footprint(cfg, frames);
  if (s->used + fp > s->cfg.hbm_budget)
    return rd::set_error(RD_ENOMEM, "rd_stream_open: admission refused, the stream needs %llu "
                         "bytes and %llu of the %llu-byte budget are free",
                         (unsigned long long)fp, (unsigned long long)(s->cfg.hbm_budget - s->used),
                         (unsigned long long)s->cfg.hbm_budget);
  StreamState ss;
  ss.cfg = *cfg;
  ss.footprint = fp;
  ss.n_pairs = rd_cov_pairs(cfg);
  st = rd_chain_create(cfg, &ss.ch);
  if (st == RD_OK) st = rd_chain_set_coeff(ss.ch, coeff);
  if (st == RD_OK) st = rd_chain_set_weights(ss.ch, weights);
  // the stream's copies, launches and export all go on the chain's own
  // stream: no cross-stream events per request
  if (st == RD_OK) ss.cs = rd::chain_stream(ss.ch);
  if (st == RD_OK && frames) {
    // size the chain's per-call buffers with one request of the largest
    // size, so that requests never allocate (cudaMalloc would stall the
    // device), then return the chain to its initial state
    const uint64_t n = frames * cfg->n_fft;
    rd_cplx16* z = s->slots[0].used ? nullptr : s->slots[0].dev;
    rd_cplx16* tmp = nullptr;
    if (!z && cudaMalloc(&tmp, (size_t)cfg->n_chan * n * 4) == cudaSuccess) z = tmp;
    if (z && cudaMemsetAsync(z, 0, (size_t)cfg->n_chan * n * 4, ss.cs) == cudaSuccess) {
      st = rd_chain_process_device(ss.ch, z, n, n, ss.cs);
      if (st == RD_OK) st = rd_chain_reset(ss.ch, ss.cs);
      if (cudaStreamSynchronize(ss.cs) != cudaSuccess)
        st = rd::set_error(RD_EDEVICE, "rd_stream_open: warm-up failed");
    }
    if (tmp) cudaFree(tmp);
  }
  if (st != RD_OK) {
    if (ss.ch) rd_chain_destroy(ss.ch);
    return st;
  }
  ss.open = true;
  s->used += fp;
  // one page-locked block for the most window sums a request of this stream
  // can close, so that requests take them without allocating. The pool keeps
  // at most as many blocks as requests can be outstanding (retire() keeps the
  // same cap): when it is full, its smallest block makes room for this one if
  // it is too small for this stream, else nothing is added, so repeated
  // open / close cycles do not grow page-locked memory.
  if (ss.n_pairs && cfg->cov_source != RD_COV_OFF && frames) {
    const uint64_t wl = cfg->cov_window ? cfg->cov_window : 1u;
    const size_t words = (size_t)(frames / wl + 1u) * cfg->n_fft * ss.n_pairs * 2u;
    const size_t keep = (size_t)s->cfg.queue_cap + s->cfg.max_inflight;
    bool add = true;
    if (s->cov_pool.size() >= keep && !s->cov_pool.empty()) {
      size_t sm = 0;
      for (size_t k = 1; k < s->cov_pool.size(); ++k)
        if (s->cov_pool[k].cap < s->cov_pool[sm].cap) sm = k;
      if (s->cov_pool[sm].cap >= words) {
        add = false;
      } else {
        cudaFreeHost(s->cov_pool[sm].p);
        s->cov_pool.erase(s->cov_pool.begin() + (ptrdiff_t)sm);
      }
    }
    PinnedBuf b{};
    if (add && cudaMallocHost(&b.p, words * sizeof(int64_t)) == cudaSuccess) {
      b.cap = words;
      s->cov_pool.push_back(b);
    }
  }
  uint32_t id = 0;
  while (id < s->streams.size() && s->streams[id].open) ++id;
  if (id == s->streams.size()) s->streams.push_back(ss);
  else s->streams[id] = ss;
  *stream_id = id;
  return RD_OK;
}

rd_status rd_stream_close(rd_server* s, uint32_t id) {
  if (!s || id >= s->streams.size() || !s->streams[id].open)
    return rd::set_error(RD_EINVAL, "rd_stream_close: no such stream");
  StreamState& st = s->streams[id];
  if (st.outstanding) return rd::set_error(RD_EAGAIN, "rd_stream_close: requests outstanding");
  cudaStreamSynchronize(st.cs);
  rd_chain_destroy(st.ch);  // and with it the stream
  s->used -= st.footprint;
  st = StreamState{};
  return RD_OK;
}

rd_status rd_stream_set_pairs(rd_server* s, uint32_t id, const uint32_t* x, const uint32_t* y,
                              uint32_t n_pairs) {
  if (!s || id >= s->streams.size() || !s->streams[id].open)
    return rd::set_error(RD_EINVAL, "rd_stream_set_pairs: no such stream");
  StreamState& st = s->streams[id];
  if (st.outstanding || st.busy)
    return rd::set_error(RD_EINVAL, "rd_stream_set_pairs: the stream has requests");
  if (n_pairs != st.n_pairs)
    return rd::set_error(RD_EINVAL, "rd_stream_set_pairs: %u pairs, the stream was admitted with "
                         "cov_n_pairs %u", n_pairs, st.n_pairs);
  // the open's warm-up left the chain reset on its stream; the table goes in
  // before the stream's first request
  if (cudaStreamSynchronize(st.cs) != cudaSuccess)
    return rd::set_error(RD_EDEVICE, "rd_stream_set_pairs: stream sync failed");
  return rd_chain_set_pairs(st.ch, x, y, n_pairs);
}

rd_status rd_server_submit(rd_server* s, uint32_t id, const rd_cplx16* adc, uint64_t n,
                           uint64_t ld, uint64_t* req_id) {
  if (!s || !adc || !req_id || id >= s->streams.size() || !s->streams[id].open)
    return rd::set_error(RD_EINVAL, "rd_server_submit: bad argument");
  StreamState& st = s->streams[id];
  if (n == 0 || n % st.cfg.n_fft || n > s->cfg.max_request_samples || ld < n)
    return rd::set_error(RD_EINVAL, "rd_server_submit: %llu samples per channel (a multiple of "
                         "%u, at most %llu)", (unsigned long long)n, st.cfg.n_fft,
                         (unsigned long long)s->cfg.max_request_samples);
  if (s->free_host.empty()) return rd::set_error(RD_EAGAIN, "rd_server_submit: queue full");
  Request r;
  r.id = s->next_id++;
  r.stream = id;
  r.n = n;
  r.host_buf = s->free_host.back();
  s->free_host.pop_back();
  rd_cplx16* h = s->host[r.host_buf];
  for (uint32_t c = 0; c < st.cfg.n_chan; ++c) std::memcpy(h + (size_t)c * n, adc + (size_t)c * ld, n * 4);
  if (!s->pool.empty()) {  // buffers of an earlier request
    OutBufs& b = s->pool.back();
    r.events = std::move(b.events);
    r.flits = std::move(b.flits);
    r.windows = std::move(b.windows);
    s->pool.pop_back();
  }
  r.t_submit = s->now();
  *req_id = r.id;
  st.outstanding++;
  s->waiting.push_back(r.id);
  s->reqs.emplace(r.id, std::move(r));
  return start_ready(s);
}

rd_status rd_server_poll(rd_server* s, rd_completion* out, uint32_t cap, uint32_t* n_out) {
  if (!s) return rd::set_error(RD_EINVAL, "rd_server_poll: null server");
  for (Slot& sl : s->slots) {
    if (!sl.used) continue;
    const cudaError_t q = cudaEventQuery(sl.done);
    if (q == cudaErrorNotReady) continue;
    Request& r = s->reqs[sl.req];
    StreamState& st = s->streams[r.stream];
    r.status = q == cudaSuccess ? (r.xb ? finish_export(s, r) : collect(s, r))
                                : rd::set_error(RD_EDEVICE, "request failed: %s", cudaGetErrorString(q));
    r.t_done = s->now();
    r.done = true;
    sl.used = false;
    s->free_host.push_back(r.host_buf);
    r.host_buf = -1;
    st.busy = false;
    st.outstanding--;
    rd_completion c{};
    c.req_id = r.id;
    c.stream_id = r.stream;
    c.status = r.status;
    c.n_events = r.n_events;
    c.n_cov_windows = r.n_windows;
    c.t_submit_us = r.t_submit;
    c.t_start_us = r.t_start;
    c.t_done_us = r.t_done;
    s->finished.push_back(c);
  }
  rd_status st = start_ready(s);
  uint32_t k = 0;
  if (out) {
    k = (uint32_t)std::min<size_t>(cap, s->finished.size());
    std::memcpy(out, s->finished.data(), k * sizeof(rd_completion));
    s->finished.erase(s->finished.begin(), s->finished.begin() + k);
  }
  if (n_out) *n_out = k;
  return st;
}

rd_status rd_server_take(rd_server* s, uint64_t req_id, rd_output* out) {
  if (!s || !out) return rd::set_error(RD_EINVAL, "rd_server_take: null argument");
  auto it = s->reqs.find(req_id);
  if (it == s->reqs.end() || !it->second.done)
    return rd::set_error(RD_EINVAL, "rd_server_take: request %llu is not complete",
                         (unsigned long long)req_id);
  Request& r = it->second;
  bool trunc = false;
  out->n_events = r.n_events;
  out->n_flits = r.n_flits;
  out->flit_words = r.flit_words;
  out->n_cov_windows = r.n_windows;
  out->n_frames = r.n / s->streams[r.stream].cfg.n_fft;
  // exported outputs sit in the request's block (n_kept of them), else in
  // its vectors
  const rd_event* ev = r.xb ? r.xb->ev : r.events.data();
  const uint32_t* fl = r.xb ? r.xb->fl : r.flits.data();
  const uint64_t n_ev = r.xb ? r.n_kept : r.events.size();
  const uint64_t n_fl = r.xb ? r.n_kept * (r.n_events ? r.n_flits / r.n_events : 0) : r.n_flits;
  if (out->events) {
    const uint64_t k = std::min<uint64_t>(n_ev, out->cap_events);
    trunc |= k < r.n_events;
    std::memcpy(out->events, ev, k * sizeof(rd_event));
  }
  if (out->flits && r.flit_words) {
    const uint64_t k = std::min<uint64_t>(n_fl, out->cap_flits);
    trunc |= k < r.n_flits;
    std::memcpy(out->flits, fl, k * r.flit_words * 4);
  }
  if (r.n_windows) {
    const uint32_t k = std::min<uint32_t>(r.n_windows, out->cap_cov_windows);
    trunc |= k < r.n_windows;
    if (out->cov_windows) std::memcpy(out->cov_windows, r.windows.data(), k * sizeof(rd_cov_window));
    const size_t per = r.n_windows ? r.cov.len / r.n_windows : 0;
    if (out->cov_acc) std::memcpy(out->cov_acc, r.cov.p, k * per * 8);
  }
  const rd_status st = r.status;
  retire(s, it);
  if (st != RD_OK) return st;
  return trunc ? rd::set_error(RD_ETRUNC, "rd_server_take: output capacity exceeded") : RD_OK;
}

rd_status rd_server_info_get(rd_server* s, rd_server_info* info) {
  if (!s || !info) return rd::set_error(RD_EINVAL, "rd_server_info_get: null argument");
  info->hbm_budget = s->cfg.hbm_budget;
  info->hbm_used = s->used;
  info->streams = 0;
  for (const StreamState& st : s->streams) info->streams += st.open ? 1u : 0u;
  info->inflight = 0;
  for (const Slot& sl : s->slots) info->inflight += sl.used ? 1u : 0u;
  info->queued = (uint32_t)s->waiting.size();
  return RD_OK;
}

static constexpr double kTraceStallUs = 30e6;

rd_status rd_server_run_trace(rd_server* s, uint64_t n_req, const uint32_t* stream_ids,
                              const double* arrival_us, const rd_cplx16* const* adc,
                              const uint64_t* n, double* latency_us, double* makespan_us) {
  if (!s || !stream_ids || !arrival_us || !adc || !n || !latency_us)
    return rd::set_error(RD_EINVAL, "rd_server_run_trace: null argument");
  std::unordered_map<uint64_t, uint64_t> idx;  // request id -> trace index
  std::vector<rd_completion> comp(64);
  const double t0 = s->now();
  uint64_t next = 0, done = 0;
  rd_status first_err = RD_OK;
  // the loop gives up when requests are outstanding and none has completed
  // for kTraceStallUs of wall-clock time (a device that stopped answering)
  double t_progress = t0;
  uint64_t done_seen = 0;
  while (done < n_req) {
    const double t = s->now() - t0;
    if (done != done_seen) {
      done_seen = done;
      t_progress = t + t0;
    } else if (next > done && t + t0 - t_progress > kTraceStallUs) {
      if (makespan_us) *makespan_us = s->now() - t0;
      return rd::set_error(RD_ETIMEOUT, "rd_server_run_trace: no request completed for %.0f s "
                           "with %llu outstanding", kTraceStallUs * 1e-6,
                           (unsigned long long)(next - done));
    }
    while (next < n_req && arrival_us[next] <= t) {
      uint64_t id = 0;
      const rd_status st = rd_server_submit(s, stream_ids[next], adc[next], n[next], n[next], &id);
      if (st == RD_EAGAIN) break;  // queue full: the request waits on the host
      if (st != RD_OK) return st;
      idx[id] = next++;
    }
    uint32_t k = 0;
    const rd_status ps = rd_server_poll(s, comp.data(), (uint32_t)comp.size(), &k);
    if (ps != RD_OK) return ps;
    for (uint32_t i = 0; i < k; ++i) {
      const uint64_t j = idx[comp[i].req_id];
      latency_us[j] = (comp[i].t_done_us - t0) - arrival_us[j];
      if (comp[i].status != RD_OK && first_err == RD_OK) first_err = (rd_status)comp[i].status;
      retire(s, s->reqs.find(comp[i].req_id));  // the outputs are not kept
      ++done;
    }
  }
  if (makespan_us) *makespan_us = s->now() - t0;
  return first_err;
}
