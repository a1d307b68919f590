// api.cu - the C ABI of include/rd_chain.h: chain state, the launch sequence
// per chunk of frames, the history / align bookkeeping that needs no device
// work, and the per-block entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "fxp.cuh"
#include "rd_internal.h"

using namespace rd;

namespace {

thread_local std::string g_err;

rd_status fail(rd_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return st;
}

#define CK(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(RD_EDEVICE, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                              \
  } while (0)

bool is_pow2(uint32_t v) { return v && !(v & (v - 1)); }

}  // namespace

rd_status rd::set_error(rd_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return st;
}

namespace {

void sat_bump(uint32_t* c, uint64_t by) {
  const uint64_t v = (uint64_t)*c + by;
  *c = v > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)v;
}

// Whether chains of this configuration run the PFB as its own pass before the
// FFT kernel (then they hold its outputs: F x C x N words): taps the pass is
// specialised for and an FFT geometry with a specialised kernel.
bool pfb_pass(const rd_config& c) {
  return (c.taps == 4u || c.taps == 8u || c.taps == 16u) && front_fast_ok(c.n_fft, c.spc);
}

unsigned clog2(unsigned v) {
  unsigned w = 0;
  while ((1u << w) < v) ++w;
  return w;
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
    if (e == cudaSuccess) n = std::max<size_t>(want, 1);
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Host mirror of the history model's state machine (history_model.hpp:191-467)
// for the chain's write pattern: every antenna writes one whole frame, in
// order, then the align stage reads every bin at frame_off 0. Only the
// counters and pointers live here; the samples live in the device ring.
// ---------------------------------------------------------------------------
struct HistMirror {
  unsigned n_ant = 0, n = 0, lanes = 1, frames_max = 4, depth = 4;
  uint32_t frames_done = 0;
  unsigned done_slot = 0;
  unsigned epoch = 0;       // depth changes so far
  uint64_t base = 0;        // the stream frame of this epoch's frame 0 (ring slots)
  // the stream frame last written to the model's slot 0, which a read returns
  // when no frame is done in the epoch (the model never clears its store)
  uint64_t slot0_frame = 0;
  bool slot0_valid = false;
  uint32_t c_overwrite = 0, c_skew = 0, c_wbeat = 0, c_read = 0, c_collision = 0, c_error = 0;

  unsigned readable() const {
    const unsigned dm2 = depth <= 2 ? 0u : depth - 2u;
    return frames_done >= dm2 ? dm2 : (unsigned)frames_done;
  }
  // every antenna finished the next frame (write_beat x M each, then settle_)
  void write_frame() {
    sat_bump(&c_wbeat, (uint64_t)n_ant * (n / lanes));
    // the antennas finish a frame one after another: at depth 1 the first to
    // finish is a whole depth ahead of the frame count until the last one
    // does, a skew episode per frame (history_model.hpp:425-431)
    if (depth <= 1u && n_ant > 1u) sat_bump(&c_skew, 1);
    if (frames_done >= depth) sat_bump(&c_overwrite, 1);
    frames_done += 1;
    if (frames_done != 1) done_slot = (done_slot + 1 == depth) ? 0u : done_slot + 1u;
    if ((frames_done - 1u) % depth == 0u) {  // frame j of the epoch went to slot j % depth
      slot0_frame = base + frames_done - 1u;
      slot0_valid = true;
    }
  }
  struct Read {
    unsigned slot;
    uint32_t frame_id;
    unsigned flags;
    bool valid_data;
  };
  // read() (history_model.hpp:283-337) without touching the counters
  Read locate(unsigned bin, unsigned frame_off) const {
    const unsigned depth_mask = (1u << clog2(frames_max + 1)) - 1u;
    unsigned slot_w = clog2(frames_max);
    if (slot_w == 0) slot_w = 1;
    const unsigned slot_mask = (1u << slot_w) - 1u;
    const unsigned ext_mask = (1u << (slot_w + 1)) - 1u;
    const unsigned bin_p = bin & 0xFFFFu, off_p = frame_off & 0xFFFFu;
    const unsigned rd = readable();
    const bool oor = (bin_p >= n) || (rd == 0) || (off_p >= rd);
    const unsigned off_clamped = rd == 0 ? 0u : rd - 1u;
    const unsigned off_safe = oor ? off_clamped : (off_p & depth_mask);
    const unsigned off_ext = off_safe & ext_mask, done_ext = done_slot & ext_mask;
    const unsigned slot = (done_ext >= off_ext) ? ((done_ext - off_ext) & slot_mask)
                                                : (((done_ext - off_ext + depth) & ext_mask) & slot_mask);
    const unsigned write_slot = (done_slot + 1 == depth) ? 0u : (done_slot + 1) & slot_mask;
    const bool collision = (frames_done != 0) && (slot == write_slot);
    const uint32_t fid = (uint32_t)(frames_done - 1u - off_safe);
    const bool stale = (uint32_t)(frames_done - fid) > depth;
    Read r;
    r.slot = slot;
    r.frame_id = fid;
    r.flags = (oor ? 1u : 0u) | (collision ? 2u : 0u) | (stale ? 4u : 0u);
    r.valid_data = frames_done != 0;
    return r;
  }
  void count_reads(unsigned flags, uint64_t k) {
    sat_bump(&c_read, k);
    if (flags & 2u) sat_bump(&c_collision, k);
    if (flags & 1u) sat_bump(&c_error, k);
  }
};

namespace {
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};
}  // namespace

struct rd_chain {
  rd_config cfg;
  uint32_t R = 0;            // ring frames
  uint32_t launch_frames = 0;  // frames per launch (<= max_frames)
  uint32_t safe_in = 0;        // FFT inputs within this bound cannot saturate
  uint32_t S = 0, P = 0;     // covariance source length, pairs
  bool pairs_custom = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;  // ordering with the caller's stream

  DevBuf<uint32_t> coeff_t, weights, tail[2], ring, power, beams_bn, stage, tw_pos;
  DevBuf<int2> tw2;
  DevBuf<uint32_t> pfb_buf;  // the PFB pass's outputs, [max_frames][C][N]
  uint32_t coeff_real = 0;   // 1: the bank's imaginary parts are all 0
  // host-input staging: three buffers (stage, stage2, stage3), so a chunk's
  // copy may run up to two chunks ahead of the compute
  DevBuf<uint32_t> stage2, stage3;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_ready[3] = {nullptr, nullptr, nullptr}, ev_free[3] = {nullptr, nullptr, nullptr};
  // results drained into page-locked host buffers chunk by chunk
  cudaStream_t out_stream = nullptr;
  unsigned long long* h_snaps = nullptr;   // page-locked: events of the call after each chunk
  size_t h_snaps_n = 0;
  std::vector<cudaEvent_t> ev_snap;        // one per chunk of a call: its snapshot landed
  bool drained_events = false, drained_flits = false;
  uint32_t drained_windows = 0;
  DevBuf<int4> w_limbs;
  DevBuf<int2> coeff2;      // [T][N] unpacked coefficients
  DevBuf<uint2> coeff_dp;   // [T][N] byte limbs for the two-way dot products
  uint32_t pfb_dp = 0;
  uint32_t x_safe = 0;      // beamformer: |x| bound for exact int32 sums
  uint32_t pfb32 = 0;       // 1: int32 PFB accumulation is exact for this bank
  DevBuf<uint32_t> w_frag;  // warp-level tensor form: mma fragments of the limb-split weights
  DevBuf<uint32_t> w_t5;    // tcgen05 form: the canonical-layout weight operand
  bool t5 = false;          // the beamformer runs on tcgen05
  // tensor form of the exact covariance: plan, unit lists and pair map
  CovTcHost cov_tc{};
  bool cov_tc_ok = false;
  DevBuf<uint32_t> ct_units;
  DevBuf<int32_t> ct_pq;
  int tail_cur = 0;
  DevBuf<uint32_t> px, py;
  // integrator state [2][N][P]: each launch reads one copy and writes the
  // other, so the CTA that carries a window in never races the CTA that
  // carries the next one out
  DevBuf<long long> acc_re, acc_im, cov_out;
  uint32_t acc_cur = 0;
  // the beat-stream covariance engine: pairs, and [2][pairs][re, im] open
  // window accumulators (ping-pong)
  uint32_t eng_pairs = 0;
  DevBuf<long long> eng_acc;
  uint32_t eng_cur = 0;
  DevBuf<unsigned> sticky, satcnt, win_flags;
  DevBuf<uint32_t> counts, detsup, mask;   // CFAR per-frame decisions
  DevBuf<unsigned long long> totals;       // CFAR events per 8-frame group and per 64 groups
  DevBuf<uint4> slots;                     // CFAR detections per frame
  DevBuf<rd_event> events;
  DevBuf<uint32_t> flits;
  DevBuf<uint32_t> tap_pfb;
  DevBuf<DevStats> stats;

  // host-side state
  uint64_t frame = 0;        // frames processed so far
  uint32_t cov_count = 0;    // samples in the open covariance window
  uint32_t cov_window_id = 0;
  HistMirror hist;
  rd_stats host_st{};        // host-owned counters (history, align, packets)
  uint32_t align_seq = 0;
  // results of the last call
  uint64_t call_frames = 0;
  std::vector<rd_cov_window> call_windows;
  uint64_t call_cap_events = 0;
  uint64_t launches = 0;
  // stage timing (rd_chain_set_profiling)
  bool profiling = false;
  struct Pending {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  double ktime[8] = {0};
  uint64_t klaunch[8] = {0};
  cudaEvent_t ev_get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
};

static const char* kKernelNames[8] = {"k_front", "k_beam", "k_cov", "k_cfar",
                                      "",        "",       "",      "k_call"};
enum { KT_FRONT = 0, KT_BEAM, KT_COV, KT_CFAR, KT_CALL = 7 };

// Brackets one kernel launch with events on the chain's stream when stage
// timing is on.
// A stage's launches: an NVTX range always, CUDA events around them when
// the chain is profiling.
const char* const kStageNames[] = {"rd front (PFB + FFT)", "rd beamform + power",
                                   "rd covariance", "rd CFAR + events + packets"};

struct KTimer {
  rd_chain* ch;
  int id;
  cudaEvent_t a = nullptr;
  rd::NvtxRange range;
  KTimer(rd_chain* c, int i) : ch(c), id(i), range(i >= 0 && i < 4 ? kStageNames[i] : "rd call") {
    if (ch->profiling) {
      a = ch->ev_get();
      cudaEventRecord(a, ch->stream);
    }
  }
  ~KTimer() {
    if (a) {
      cudaEvent_t b = ch->ev_get();
      cudaEventRecord(b, ch->stream);
      ch->pending.push_back({id, a, b});
    }
  }
};

extern "C" {

const char* rd_last_error(void) { return g_err.c_str(); }
const char* rd_version(void) { return "rdgb 0.1 sm_103a"; }

int rd_device_ok(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0, major = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  return major >= 10 ? 1 : 0;
}

void rd_config_default(rd_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->n_chan = 4;
  c->n_fft = 64;
  c->taps = 4;
  c->spc = 2;
  c->scale_sched = 0xFFFFFFFFu;
  c->hist_frames = 8;
  c->n_beams = 2;
  c->cfar_enable = 1;  // cfar_model.hpp:112-128 defaults
  c->cfar_mode = RD_CFAR_CA;
  c->cfar_out_mode = RD_CFAR_EVENTS;
  c->guard_lead = c->guard_lag = 2;
  c->ref_lead = c->ref_lag = 8;
  c->alpha = 1u << 8;
  c->max_guard = 2;
  c->max_ref = 8;
  c->cov_source = RD_COV_CHANNEL;
  c->cov_mode = RD_COV_BLOCK;
  c->cov_window = 256;
  c->cov_acc_w = 64;
  c->packet_w = 64;
  c->max_frames = 1024;
  c->form = RD_FORM_CUDA_CORE;
}

uint32_t rd_flit_words(uint32_t packet_w) { return (packet_w + 5u + 31u) / 32u; }
uint32_t rd_detection_flits(uint32_t packet_w) {
  return packet_w ? 1u + (176u + packet_w - 1u) / packet_w : 0u;
}

uint32_t rd_cov_pairs(const rd_config* c) {
  if (c->cov_source == RD_COV_OFF) return 0;
  if (c->cov_n_pairs) return c->cov_n_pairs;
  const uint32_t s = c->cov_source == RD_COV_CHANNEL ? c->n_chan : c->n_beams;
  return s * (s + 1) / 2;
}

rd_status rd_config_validate(const rd_config* c) {
  if (!c) return fail(RD_EINVAL, "null config");
  if (c->n_chan < 1 || c->n_chan > 128) return fail(RD_EINVAL, "n_chan %u not in 1..128", c->n_chan);
  if (c->n_beams < 1 || c->n_beams > 128) return fail(RD_EINVAL, "n_beams %u not in 1..128", c->n_beams);
  if (!is_pow2(c->n_fft) || c->n_fft < 8 || c->n_fft > 1024)
    return fail(RD_EINVAL, "n_fft %u must be a power of two in 8..1024", c->n_fft);
  if (c->spc != 1 && c->spc != 2) return fail(RD_EINVAL, "spc %u must be 1 or 2", c->spc);
  if (c->n_fft / c->spc < 4) return fail(RD_EINVAL, "n_fft/spc must be >= 4");
  if (c->taps < 1 || c->taps > 64) return fail(RD_EINVAL, "taps %u not in 1..64", c->taps);
  if (!is_pow2(c->hist_frames) || c->hist_frames < 4 || c->hist_frames > 65536)
    return fail(RD_EINVAL, "hist_frames %u must be a power of two >= 4", c->hist_frames);
  if (c->packet_w < 64 || c->packet_w > 512 || (c->packet_w % 32) != 0)
    return fail(RD_EINVAL, "packet_w %u must be a multiple of 32 in 64..512", c->packet_w);
  if (c->max_guard > 31 || c->max_ref > 63) return fail(RD_EINVAL, "CFAR maxima out of range");
  if (c->cov_source > RD_COV_BEAM || c->cov_mode > RD_COV_EXP)
    return fail(RD_EINVAL, "bad covariance source/mode");
  if (c->cov_source != RD_COV_OFF) {
    if (c->cov_acc_w < 33 || c->cov_acc_w > 64) return fail(RD_EINVAL, "cov_acc_w must be 33..64");
    if (c->cov_exp_k > 15) return fail(RD_EINVAL, "cov_exp_k must be 0..15");
    if (c->cov_window > 65535) return fail(RD_EINVAL, "cov_window must fit 16 bits");
  }
  if (c->max_frames < 1 || c->max_frames > 65536) return fail(RD_EINVAL, "max_frames 1..65536");
  if (c->form > RD_FORM_TENSOR_WARP) return fail(RD_EINVAL, "bad form");
  if (c->form != RD_FORM_CUDA_CORE && c->n_chan > RD_TC_MAX_CHAN)
    return fail(RD_EINVAL, "the tensor form takes at most %u channels", RD_TC_MAX_CHAN);
  if (c->vc > 3 || c->src_id > 31 || c->dest > 15) return fail(RD_EINVAL, "packet header field out of range");
  return RD_OK;
}

static rd_status upload_pairs(rd_chain* ch, const uint32_t* x, const uint32_t* y, uint32_t n) {
  CK(ch->px.ensure(n));
  CK(ch->py.ensure(n));
  CK(cudaMemcpy(ch->px.p, x, n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ch->py.p, y, n * 4, cudaMemcpyHostToDevice));
  const size_t k = (size_t)ch->cfg.n_fft * n;
  CK(ch->acc_re.ensure(2 * k));
  CK(ch->acc_im.ensure(2 * k));
  CK(ch->sticky.ensure(k));
  CK(ch->satcnt.ensure(2 * k));
  CK(cudaMemset(ch->acc_re.p, 0, 2 * k * 8));
  CK(cudaMemset(ch->acc_im.p, 0, 2 * k * 8));
  ch->acc_cur = 0;
  CK(cudaMemset(ch->sticky.p, 0, k * 4));
  CK(cudaMemset(ch->satcnt.p, 0, k * 8));
  ch->P = n;
  ch->cov_tc_ok = false;
  if (ch->cfg.form != RD_FORM_CUDA_CORE && cov_tc_plan(ch->S, x, y, n, &ch->cov_tc)) {
    CK(ch->ct_units.ensure(ch->cov_tc.units.size()));
    CK(ch->ct_pq.ensure(ch->cov_tc.pq.size()));
    CK(cudaMemcpy(ch->ct_units.p, ch->cov_tc.units.data(), ch->cov_tc.units.size() * 4,
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ch->ct_pq.p, ch->cov_tc.pq.data(), ch->cov_tc.pq.size() * 4,
                  cudaMemcpyHostToDevice));
    ch->cov_tc.plan.units = ch->ct_units.p;
    ch->cov_tc.plan.pq = ch->ct_pq.p;
    ch->cov_tc_ok = true;
  }
  return RD_OK;
}

rd_status rd_chain_create(const rd_config* cfg, rd_chain** out) {
  if (!out) return fail(RD_EINVAL, "null out");
  *out = nullptr;
  rd_status st = rd_config_validate(cfg);
  if (st != RD_OK) return st;
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no CUDA device of compute capability 10.x or newer");
  rd_chain* ch = new rd_chain();
  ch->cfg = *cfg;
  const rd_config& c = ch->cfg;
  const uint32_t N = c.n_fft, C = c.n_chan, B = c.n_beams, T = c.taps, F = c.max_frames;
  ch->R = F + c.hist_frames;
  ch->launch_frames = F;
  ch->safe_in = front_safe_input(N, c.spc, c.scale_sched);
  ch->t5 = c.form == RD_FORM_TENSOR && beam_t5_ok(C, B);
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    fail(e == cudaErrorMemoryAllocation ? RD_ENOMEM : RD_EDEVICE, "allocation failed: %s",
         cudaGetErrorString(e));
    return true;
  };
  const uint32_t D = T > 1 ? T - 1 : 1;
  if (bad(cudaStreamCreateWithFlags(&ch->stream, cudaStreamNonBlocking)) ||
      bad(cudaEventCreateWithFlags(&ch->ev_in, cudaEventDisableTiming)) ||
      bad(cudaEventCreateWithFlags(&ch->ev_out, cudaEventDisableTiming)) ||
      bad(ch->coeff_t.ensure((size_t)T * N)) || bad(ch->coeff2.ensure((size_t)T * N)) ||
      bad(ch->coeff_dp.ensure((size_t)T * N)) ||
      bad(ch->weights.ensure((size_t)B * C)) ||
      bad(ch->w_limbs.ensure((size_t)B * C)) ||
      (c.form != RD_FORM_CUDA_CORE && !ch->t5 &&
       bad(ch->w_frag.ensure(beam_tc_fragment_words(C, B)))) ||
      (ch->t5 && bad(ch->w_t5.ensure(beam_t5_operand_words(C, B)))) ||
      bad(ch->tail[0].ensure((size_t)C * D * N)) || bad(ch->tail[1].ensure((size_t)C * D * N)) ||
      bad(ch->ring.ensure((size_t)ch->R * N * C)) || bad(ch->power.ensure((size_t)F * B * N)) ||
      bad(ch->counts.ensure((size_t)F * B)) || bad(ch->detsup.ensure((size_t)F * B)) ||
      bad(ch->mask.ensure((size_t)F * B * ((N + 31) / 32))) ||
      bad(ch->totals.ensure(cfar_tiles(F * B))) ||
      bad(ch->slots.ensure((size_t)F * B * kCfarSlots)) || bad(ch->stats.ensure(1)) ||
      (pfb_pass(c) && bad(ch->pfb_buf.ensure((size_t)F * C * N)))) {
    rd_chain_destroy(ch);
    return RD_ENOMEM;
  }
  ch->own_stream = true;
  cudaMemset(ch->coeff_t.p, 0, (size_t)T * N * 4);
  cudaMemset(ch->coeff2.p, 0, (size_t)T * N * sizeof(int2));
  cudaMemset(ch->coeff_dp.p, 0, (size_t)T * N * sizeof(uint2));
  cudaMemset(ch->weights.p, 0, (size_t)B * C * 4);
  cudaMemset(ch->w_limbs.p, 0, (size_t)B * C * sizeof(int4));
  if (c.form != RD_FORM_CUDA_CORE && !ch->t5)
    cudaMemset(ch->w_frag.p, 0, (size_t)beam_tc_fragment_words(C, B) * 4);
  if (ch->t5) cudaMemset(ch->w_t5.p, 0, (size_t)beam_t5_operand_words(C, B) * 4);
  cudaMemset(ch->tail[0].p, 0, (size_t)C * D * N * 4);
  cudaMemset(ch->tail[1].p, 0, (size_t)C * D * N * 4);
  cudaMemset(ch->ring.p, 0, (size_t)ch->R * N * C * 4);
  cudaMemset(ch->stats.p, 0, sizeof(DevStats));
  if (c.cov_source != RD_COV_OFF) {
    ch->S = c.cov_source == RD_COV_CHANNEL ? C : B;
    const uint32_t np = rd_cov_pairs(&c);
    std::vector<uint32_t> x, y;
    for (uint32_t i = 0; i < ch->S; ++i)
      for (uint32_t j = i; j < ch->S; ++j) {
        x.push_back(i);
        y.push_back(j);
      }
    x.resize(np);
    y.resize(np);
    st = upload_pairs(ch, x.data(), y.data(), np);
    if (st != RD_OK) {
      rd_chain_destroy(ch);
      return st;
    }
    if (c.cov_source == RD_COV_BEAM && bad(ch->beams_bn.ensure((size_t)F * N * B))) {
      rd_chain_destroy(ch);
      return RD_ENOMEM;
    }
  }
  // the beat-stream covariance engine reads the beamformer's outputs
  ch->eng_pairs = std::min<uint32_t>(c.engine_pairs, B >= 2u ? B / 2u : 1u);
  if (ch->eng_pairs) {
    if (bad(ch->beams_bn.ensure((size_t)F * N * B)) ||
        bad(ch->eng_acc.ensure(4u * ch->eng_pairs))) {
      rd_chain_destroy(ch);
      return RD_ENOMEM;
    }
    cudaMemset(ch->eng_acc.p, 0, 4u * ch->eng_pairs * sizeof(long long));
  }
  {
    std::vector<uint32_t> tp(5u * N);
    uint32_t words = 0;
    twiddle_positions(N, c.spc, tp.data(), &words);
    if (bad(ch->tw_pos.ensure(words ? words : 1))) {
      rd_chain_destroy(ch);
      return RD_ENOMEM;
    }
    if (words) cudaMemcpy(ch->tw_pos.p, tp.data(), words * 4, cudaMemcpyHostToDevice);
    std::vector<int2> t2(words ? words : 1u, int2{0, 0});
    for (uint32_t k = 0; k < words; ++k)
      t2[k] = int2{(int)(int16_t)(uint16_t)(tp[k] & 0xFFFFu), (int)tp[k] >> 16};
    if (bad(ch->tw2.ensure(t2.size()))) {
      rd_chain_destroy(ch);
      return RD_ENOMEM;
    }
    cudaMemcpy(ch->tw2.p, t2.data(), t2.size() * sizeof(int2), cudaMemcpyHostToDevice);
  }
  ch->hist.n_ant = C;
  ch->hist.n = N;
  ch->hist.lanes = c.spc;
  ch->hist.frames_max = c.hist_frames;
  ch->hist.depth = c.hist_frames;
  // the set-up copies ran on the legacy stream; wait for them without
  // synchronising the device (other chains may be running)
  if (cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess ||
      cudaStreamSynchronize(ch->stream) != cudaSuccess) {
    rd_chain_destroy(ch);
    return fail(RD_EDEVICE, "device sync failed at create");
  }
  *out = ch;
  return RD_OK;
}

void rd_chain_destroy(rd_chain* ch) {
  if (!ch) return;
  if (ch->stream) cudaStreamSynchronize(ch->stream);
  ch->coeff_t.release(); ch->coeff2.release(); ch->coeff_dp.release(); ch->weights.release(); ch->w_limbs.release(); ch->w_frag.release(); ch->w_t5.release(); ch->tail[0].release(); ch->tail[1].release();
  ch->ring.release(); ch->power.release(); ch->beams_bn.release(); ch->stage.release();
  ch->eng_acc.release();
  ch->stage2.release();
  ch->stage3.release();
  if (ch->copy_stream) cudaStreamSynchronize(ch->copy_stream);
  for (int b = 0; b < 3; ++b) {
    if (ch->ev_ready[b]) cudaEventDestroy(ch->ev_ready[b]);
    if (ch->ev_free[b]) cudaEventDestroy(ch->ev_free[b]);
  }
  if (ch->copy_stream) cudaStreamDestroy(ch->copy_stream);
  if (ch->out_stream) {
    cudaStreamSynchronize(ch->out_stream);
    cudaStreamDestroy(ch->out_stream);
  }
  if (ch->h_snaps) cudaFreeHost(ch->h_snaps);
  for (cudaEvent_t e : ch->ev_snap) cudaEventDestroy(e);
  ch->tw_pos.release(); ch->tw2.release(); ch->pfb_buf.release(); ch->ct_units.release(); ch->ct_pq.release();
  ch->px.release(); ch->py.release(); ch->acc_re.release(); ch->acc_im.release();
  ch->cov_out.release(); ch->sticky.release(); ch->satcnt.release(); ch->win_flags.release();
  ch->counts.release(); ch->detsup.release(); ch->mask.release(); ch->totals.release();
  ch->slots.release();
  ch->events.release(); ch->flits.release(); ch->tap_pfb.release(); ch->stats.release();
  for (const rd_chain::Pending& p : ch->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (cudaEvent_t e : ch->pool) cudaEventDestroy(e);
  if (ch->ev_in) cudaEventDestroy(ch->ev_in);
  if (ch->ev_out) cudaEventDestroy(ch->ev_out);
  if (ch->own_stream && ch->stream) cudaStreamDestroy(ch->stream);
  delete ch;
}

rd_status rd_chain_set_coeff(rd_chain* ch, const rd_cplx16* coeff) {
  if (!ch || !coeff) return fail(RD_EINVAL, "null argument");
  const uint32_t N = ch->cfg.n_fft, T = ch->cfg.taps;
  std::vector<uint32_t> t((size_t)T * N);
  for (uint32_t p = 0; p < N; ++p)
    for (uint32_t k = 0; k < T; ++k) t[(size_t)k * N + p] = coeff[(size_t)p * T + k];
  CK(cudaMemcpyAsync(ch->coeff_t.p, t.data(), t.size() * 4, cudaMemcpyHostToDevice, ch->stream));
  // unpacked copy, and whether every phase's L1 norm sum_k |hr| + |hi| keeps
  // the PFB sums of any int16 input inside int32 (|sum| <= 2^15 x norm)
  std::vector<int2> t2(t.size());
  // byte limbs for dp2a: h = 256 hh + hl, hl in [0, 255]; the real part uses
  // -hi, so a bank holding hi = -32768 (whose negation has no int8 high
  // limb) keeps the plain multiplies
  std::vector<uint2> tdp(t.size());
  bool neg_ok = true;
  auto lim = [](int v, int sh) { return (uint32_t)((sh ? (v >> 8) : (v & 0xFF)) & 0xFF); };
  uint64_t worst = 0;
  for (uint32_t p = 0; p < N; ++p) {
    uint64_t l1 = 0;
    for (uint32_t k = 0; k < T; ++k) {
      const uint32_t v = t[(size_t)k * N + p];
      const int re = (int16_t)(uint16_t)(v & 0xFFFFu), im = (int16_t)(uint16_t)(v >> 16);
      t2[(size_t)k * N + p] = make_int2(re, im);
      l1 += (uint64_t)(re < 0 ? -re : re) + (uint64_t)(im < 0 ? -im : im);
      if (im == -32768) neg_ok = false;
      const int ni = -im;
      // high limbs {re, -im, im, re}, low limbs likewise (bytes 0..3)
      tdp[(size_t)k * N + p] = make_uint2(
          lim(re, 1) | lim(ni, 1) << 8 | lim(im, 1) << 16 | lim(re, 1) << 24,
          lim(re, 0) | lim(ni, 0) << 8 | lim(im, 0) << 16 | lim(re, 0) << 24);
    }
    worst = std::max(worst, l1);
  }
  ch->pfb32 = worst <= 65535u ? 1u : 0u;
  ch->pfb_dp = ch->pfb32 && neg_ok ? 1u : 0u;
  ch->coeff_real = std::all_of(t2.begin(), t2.end(), [](const int2& h) { return h.y == 0; }) ? 1u : 0u;
  CK(cudaMemcpyAsync(ch->coeff2.p, t2.data(), t2.size() * sizeof(int2), cudaMemcpyHostToDevice,
                     ch->stream));
  CK(cudaMemcpyAsync(ch->coeff_dp.p, tdp.data(), tdp.size() * sizeof(uint2),
                     cudaMemcpyHostToDevice, ch->stream));
  CK(cudaStreamSynchronize(ch->stream));
  return RD_OK;
}

rd_status rd_chain_set_weights(rd_chain* ch, const rd_cplx16* w) {
  if (!ch || !w) return fail(RD_EINVAL, "null argument");
  const size_t n = (size_t)ch->cfg.n_beams * ch->cfg.n_chan;
  std::vector<int4> limbs(n);
  uint64_t l1max = 0;
  for (size_t i = 0; i < n; ++i) {  // w = 256 * wh + wl, wl in [0, 255]
    const int re = (int16_t)(uint16_t)(w[i] & 0xFFFFu), im = (int16_t)(uint16_t)(w[i] >> 16);
    limbs[i] = make_int4(re >> 8, im >> 8, re & 255, im & 255);
  }
  // |sum_a x_a w_ba| <= max|x| x sum_a (|wr| + |wi|): below 2^31 the plain
  // int32 sum is exact
  for (uint32_t b = 0; b < ch->cfg.n_beams; ++b) {
    uint64_t l1 = 0;
    for (uint32_t a = 0; a < ch->cfg.n_chan; ++a) {
      const uint32_t v = w[(size_t)b * ch->cfg.n_chan + a];
      const int re = (int16_t)(uint16_t)(v & 0xFFFFu), im = (int16_t)(uint16_t)(v >> 16);
      l1 += (uint64_t)(re < 0 ? -re : re) + (uint64_t)(im < 0 ? -im : im);
    }
    l1max = std::max(l1max, l1);
  }
  // sums within 2^31 - 2^15 also round in int32 without wrapping
  ch->x_safe = l1max ? (uint32_t)std::min<uint64_t>(0x7FFF7FFFull / l1max, 32768u) : 32768u;
  CK(cudaMemcpyAsync(ch->weights.p, w, n * 4, cudaMemcpyHostToDevice, ch->stream));
  CK(cudaMemcpyAsync(ch->w_limbs.p, limbs.data(), n * sizeof(int4), cudaMemcpyHostToDevice,
                     ch->stream));
  std::vector<uint32_t> frag;
  if (ch->t5) {
    frag.resize(beam_t5_operand_words(ch->cfg.n_chan, ch->cfg.n_beams));
    beam_t5_operand(w, ch->cfg.n_chan, ch->cfg.n_beams, frag.data());
    CK(cudaMemcpyAsync(ch->w_t5.p, frag.data(), frag.size() * 4, cudaMemcpyHostToDevice,
                       ch->stream));
  } else if (ch->cfg.form != RD_FORM_CUDA_CORE) {
    frag.resize(beam_tc_fragment_words(ch->cfg.n_chan, ch->cfg.n_beams));
    beam_tc_fragments(w, ch->cfg.n_chan, ch->cfg.n_beams, frag.data());
    CK(cudaMemcpyAsync(ch->w_frag.p, frag.data(), frag.size() * 4, cudaMemcpyHostToDevice,
                       ch->stream));
  }
  CK(cudaStreamSynchronize(ch->stream));
  return RD_OK;
}

rd_status rd_chain_set_pairs(rd_chain* ch, const uint32_t* x, const uint32_t* y, uint32_t n) {
  if (!ch || !x || !y || n == 0) return fail(RD_EINVAL, "null argument");
  if (ch->cfg.cov_source == RD_COV_OFF) return fail(RD_EINVAL, "covariance is off");
  if (ch->frame != 0) return fail(RD_EINVAL, "pairs can only be set before the first frame");
  for (uint32_t i = 0; i < n; ++i)
    if (x[i] >= ch->S || y[i] >= ch->S) return fail(RD_EINVAL, "pair %u out of range", i);
  ch->pairs_custom = true;
  return upload_pairs(ch, x, y, n);
}

__global__ void k_call_begin(DevStats* s) { s->events_call = 0; }

__global__ void k_call_end(DevStats* s) {
  s->scan_scratch[0] = s->events_call;  // events of the call just finished
  s->events_total += s->events_call;
}

// Launch sequence for one chunk of F frames whose channel-c samples start at
// adc + c*ld. tap_pfb (device) is optional.
static rd_status run_chunk(rd_chain* ch, const uint32_t* adc, uint64_t ld, uint32_t F,
                           uint32_t* d_tap_pfb) {
  const rd_config& c = ch->cfg;
  const uint32_t N = c.n_fft, C = c.n_chan, B = c.n_beams;
  cudaStream_t s = ch->stream;
  DevStats* st = ch->stats.p;
  const uint32_t ring_base = (uint32_t)(ch->frame % ch->R);

  FrontParams fp{};
  fp.adc = adc;
  fp.ld = ld;
  fp.tail = ch->tail[ch->tail_cur].p;
  fp.tail_out = c.taps > 1 ? ch->tail[ch->tail_cur ^ 1].p : nullptr;
  fp.coeff_t = ch->coeff_t.p;
  fp.coeff2 = ch->coeff2.p;
  fp.coeff_dp = ch->coeff_dp.p;
  fp.pfb_dp = ch->pfb_dp;
  fp.pfb32 = ch->pfb32;
  fp.coeff_real = ch->coeff_real;
  fp.pfb_buf = ch->pfb_buf.p;
  fp.pfb_in = nullptr;
  fp.ring = ch->ring.p;
  fp.ring_frames = ch->R;
  fp.ring_base = ring_base;
  fp.g0 = ch->frame;
  fp.tw_pos = ch->tw_pos.p;
  fp.tw2 = ch->tw2.p;
  fp.tap_pfb = d_tap_pfb;
  fp.F = F;
  fp.C = C;
  fp.N = N;
  fp.T = c.taps;
  fp.spc = c.spc;
  fp.sched = c.scale_sched;
  fp.safe_in = ch->safe_in;
  fp.stats = st;
  {
    KTimer t(ch, KT_FRONT);
    ch->launches += launch_front(fp, s);
  }
  ch->tail_cur ^= (c.taps > 1) ? 1 : 0;

  BeamParams bp{};
  bp.ring = ch->ring.p;
  bp.ring_frames = ch->R;
  bp.ring_base = ring_base;
  bp.g0 = ch->frame;
  bp.weights = ch->weights.p;
  bp.w_limbs = ch->w_limbs.p;
  bp.x_safe = ch->x_safe;
  bp.cshift = (C & (C - 1u)) == 0u ? __builtin_ctz(C) : -1;
  bp.w_frag = ch->w_frag.p;
  bp.w_t5 = ch->w_t5.p;
  bp.power = ch->power.p;
  bp.beams_bn = ch->beams_bn.p;
  bp.F = F;
  bp.C = C;
  bp.N = N;
  bp.B = B;
  bp.stats = st;
  {
    KTimer t(ch, KT_BEAM);
    if (ch->t5)
      launch_beam_t5(bp, s);
    else if (c.form != RD_FORM_CUDA_CORE)
      launch_beam_tc(bp, s);
    else
      launch_beam(bp, s);
  }
  ch->launches++;

  if (ch->eng_pairs) {  // the beat-stream covariance engine over this launch's beats
    EngineParams ep{};
    ep.beams = ch->beams_bn.p;
    ep.N = N;
    ep.B = B;
    ep.pairs = ch->eng_pairs;
    ep.beats = (uint64_t)F * (N / 2u);
    const uint64_t done = ch->frame * (N / 2u);  // beats before this launch
    ep.count0 = (uint32_t)(done % N);
    ep.n_seg = (uint32_t)((ep.count0 + ep.beats + N - 1u) / N);
    ep.acc_in = ch->eng_acc.p + (size_t)ch->eng_cur * 2u * ch->eng_pairs;
    ep.acc_out = ch->eng_acc.p + (size_t)(ch->eng_cur ^ 1u) * 2u * ch->eng_pairs;
    ep.stats = st;
    launch_engine(ep, s);
    ch->eng_cur ^= 1u;
    ch->launches++;
  }

  if (c.cov_source != RD_COV_OFF && ch->P) {
    const uint32_t wl = c.cov_window ? c.cov_window : 1u;
    const uint32_t n_win = (ch->cov_count + F) / wl;
    const uint32_t w0 = (uint32_t)ch->call_windows.size();
    CovParams cp{};
    cp.ring = ch->ring.p;
    cp.ring_frames = ch->R;
    cp.ring_base = ring_base;
    cp.g0 = ch->frame;
    // no step can saturate: exponential mode, or a block window whose worst
    // sum (wl terms of magnitude <= 2^31) fits acc_w (covar_model.hpp:82-90)
    cp.exact = (c.cov_mode == RD_COV_EXP) || c.cov_acc_w >= 64 ||
               (uint64_t)wl <= ((1ull << (c.cov_acc_w - 32)) - 1ull);
    cp.beams_bn = ch->beams_bn.p;
    cp.S = ch->S;
    cp.src_beam = c.cov_source == RD_COV_BEAM;
    cp.px = ch->px.p;
    cp.py = ch->py.p;
    cp.P = ch->P;
    cp.F = F;
    cp.N = N;
    const size_t nk = (size_t)N * ch->P;
    cp.acc_re = ch->acc_re.p + ch->acc_cur * nk;
    cp.acc_im = ch->acc_im.p + ch->acc_cur * nk;
    cp.acc_re_out = ch->acc_re.p + (ch->acc_cur ^ 1u) * nk;
    cp.acc_im_out = ch->acc_im.p + (ch->acc_cur ^ 1u) * nk;
    cp.sticky = ch->sticky.p;
    cp.satcnt = ch->satcnt.p;
    cp.count0 = ch->cov_count;
    cp.wl = wl;
    cp.exp_mode = c.cov_mode == RD_COV_EXP;
    cp.exp_k = c.cov_exp_k;
    cp.acc_w = c.cov_acc_w;
    const size_t per = (size_t)N * ch->P * 2;
    cp.out = ch->cov_out.p ? ch->cov_out.p + (size_t)w0 * per : nullptr;
    cp.win_flags = ch->win_flags.p ? ch->win_flags.p + w0 : nullptr;
    cp.n_windows = n_win;
    cp.stats = st;
    {
      KTimer t(ch, KT_COV);
      if (ch->cov_tc_ok && cp.exact && !cp.exp_mode) {
        if (c.form == RD_FORM_TENSOR && cov_t5_ok(ch->S, wl))
          launch_cov_t5(cp, ch->cov_tc.plan.pq, s);
        else
          launch_cov_tc(cp, ch->cov_tc.plan, s);
      } else {
        launch_cov(cp, s);
      }
    }
    CK(cudaGetLastError());  // a rejected launch (resources, configuration)
    ch->acc_cur ^= 1u;
    ch->launches++;
    // window headers, known on the host (covar_model.hpp:229-235)
    uint32_t cnt = ch->cov_count;
    for (uint32_t f = 0; f < F; ++f) {
      if (++cnt >= wl) {
        rd_cov_window h{};
        h.window_id = ch->cov_window_id;
        h.sample_count = cnt;
        h.end_frame = (uint32_t)(ch->frame + f);
        h.flushed = 0;
        h.truncated = cnt != wl;
        ch->call_windows.push_back(h);
        ch->cov_window_id = (ch->cov_window_id + 1u) & 0xFFFFu;
        cnt = 0;
      }
    }
    ch->cov_count = cnt;
  }

  CfarParams fp2{};
  fp2.power_u32 = ch->power.p;
  fp2.frames = F * B;
  fp2.n = N;
  fp2.beams = B;
  fp2.g0 = ch->frame;
  fp2.enable = c.cfar_enable != 0;
  fp2.go = c.cfar_mode == RD_CFAR_GO;
  fp2.dense = c.cfar_out_mode == RD_CFAR_DENSE;
  fp2.gl = std::min(c.guard_lead, c.max_guard);  // clamp_config, cfar_model.hpp:134-141
  fp2.gg = std::min(c.guard_lag, c.max_guard);
  fp2.rl = std::min(c.ref_lead, c.max_ref);
  fp2.rg = std::min(c.ref_lag, c.max_ref);
  fp2.alpha = c.alpha;
  fp2.counts = ch->counts.p;
  fp2.detsup = ch->detsup.p;
  fp2.mask = ch->mask.p;
  fp2.totals = ch->totals.p;
  fp2.slots = ch->slots.p;
  fp2.vec = (N % 4u) == 0;  // cudaMalloc'd power cells: 256-byte aligned
  fp2.ev16 = 1;
  fp2.events = ch->events.p;
  fp2.cap = ch->call_cap_events;
  fp2.flits = ch->flits.p;
  fp2.packet_w = c.packet_w;
  fp2.src_id = c.src_id;
  fp2.dest = c.dest;
  fp2.vc = c.vc;
  fp2.flit_words = rd_flit_words(c.packet_w);
  fp2.nfl = rd_detection_flits(c.packet_w);
  fp2.stats = st;
  {
    KTimer t(ch, KT_CFAR);
    launch_cfar(fp2, s);
  }
  ch->launches += 1;

  // host bookkeeping of the history and align counters, frame by frame
  for (uint32_t f = 0; f < F; ++f) {
    ch->hist.write_frame();
    const HistMirror::Read r = ch->hist.locate(0, 0);
    ch->hist.count_reads(r.flags, N);
    sat_bump(&ch->host_st.align_beats, N / 2);
    ch->align_seq = (ch->align_seq + N / 2) & 0xFFFFu;
    if (r.flags) ch->host_st.align_fault |= 8u;  // kUserHist (align_model.hpp:343-355)
  }
  ch->frame += F;
  return RD_OK;
}

static rd_status begin_call(rd_chain* ch, uint64_t frames, uint64_t cap_events) {
  const rd_config& c = ch->cfg;
  ch->call_frames = frames;
  ch->drained_events = ch->drained_flits = false;
  ch->drained_windows = 0;
  ch->call_windows.clear();
  ch->launches = 0;
  const uint64_t worst = frames * c.n_beams * (c.n_fft + 1ull);
  ch->call_cap_events = std::min<uint64_t>(cap_events, worst);
  const uint32_t nfl = rd_detection_flits(c.packet_w), words = rd_flit_words(c.packet_w);
  CK(ch->events.ensure(ch->call_cap_events));
  CK(ch->flits.ensure(ch->call_cap_events * nfl * words));
  if (c.cov_source != RD_COV_OFF && ch->P) {
    const uint32_t wl = c.cov_window ? c.cov_window : 1u;
    const uint64_t n_win = (ch->cov_count + frames) / wl;
    const size_t per = (size_t)c.n_fft * ch->P * 2;
    // one window of headroom: a call may close one more window than a
    // same-sized call that started on an empty window
    CK(ch->cov_out.ensure((n_win + 1) * per));
    CK(ch->win_flags.ensure(n_win + 1));
    if (n_win)  // flags of the windows this call closes (none: nothing reads them)
      CK(cudaMemsetAsync(ch->win_flags.p, 0, n_win * 4, ch->stream));
  }
  k_call_begin<<<1, 1, 0, ch->stream>>>(ch->stats.p);
  ch->launches++;
  return RD_OK;
}

static rd_status end_call(rd_chain* ch) {
  k_call_end<<<1, 1, 0, ch->stream>>>(ch->stats.p);
  ch->launches++;
  CK(cudaGetLastError());
  return RD_OK;
}

// Events of a call: every cell of every (frame, beam) in dense output,
// else room for one detection in 16 cells plus the summaries.
static uint64_t default_cap(const rd_config& c, uint64_t frames) {
  if (c.cfar_out_mode == RD_CFAR_DENSE) return frames * c.n_beams * (c.n_fft + 1ull);
  return frames * c.n_beams * (2ull + c.n_fft / 16u);
}

rd_status rd_chain_process_device(rd_chain* ch, const rd_cplx16* adc_dev, uint64_t n,
                                  uint64_t ld, void* stream) {
  if (!ch || !adc_dev) return fail(RD_EINVAL, "null argument");
  rd::NvtxRange range("rd_chain_process_device");
  const rd_config& c = ch->cfg;
  if (n % c.n_fft) return fail(RD_EINVAL, "n=%llu is not a multiple of n_fft", (unsigned long long)n);
  if (ld < n) return fail(RD_EINVAL, "ld < n");
  // NULL means the legacy default stream; the chain's own stream does not
  // synchronise with it implicitly, so the order is made explicit both ways.
  cudaStream_t user = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  // order the chain after the caller's stream (a wait uses the event's state
  // at the call, so one event per direction serves every call); nothing to
  // order when the caller enqueues on the chain's own stream
  const bool same = user == ch->stream;
  if (!same) {
    CK(cudaEventRecord(ch->ev_in, user));
    CK(cudaStreamWaitEvent(ch->stream, ch->ev_in, 0));
  }
  const uint64_t frames = n / c.n_fft;
  rd_status st = begin_call(ch, frames, std::max<uint64_t>(ch->events.n, default_cap(c, frames)));
  if (st != RD_OK) return st;
  for (uint64_t f = 0; f < frames; f += ch->launch_frames) {
    const uint32_t F = (uint32_t)std::min<uint64_t>(ch->launch_frames, frames - f);
    st = run_chunk(ch, adc_dev + f * c.n_fft, ld, F, nullptr);
    if (st != RD_OK) return st;
  }
  st = end_call(ch);
  if (st != RD_OK) return st;
  // and the caller's stream after the chain
  if (!same) {
    CK(cudaEventRecord(ch->ev_out, ch->stream));
    CK(cudaStreamWaitEvent(user, ch->ev_out, 0));
  }
  return RD_OK;
}

uint64_t rd_chain_last_launches(const rd_chain* ch) { return ch ? ch->launches : 0; }

rd_status rd_chain_fetch(rd_chain* ch, rd_output* out) {
  if (!ch || !out) return fail(RD_EINVAL, "null argument");
  const rd_config& c = ch->cfg;
  CK(cudaStreamSynchronize(ch->stream));
  if (ch->out_stream) CK(cudaStreamSynchronize(ch->out_stream));
  DevStats ds;
  CK(cudaMemcpy(&ds, ch->stats.p, sizeof(ds), cudaMemcpyDeviceToHost));
  if (ds.dev_timeout)
    return fail(RD_ETIMEOUT, "a bounded wait inside a tensor-core kernel gave up; results invalid");
  const uint64_t n_ev = ds.scan_scratch[0];
  const uint32_t nfl = rd_detection_flits(c.packet_w), words = rd_flit_words(c.packet_w);
  bool trunc = n_ev > ch->call_cap_events;
  const uint64_t avail = std::min<uint64_t>(n_ev, ch->call_cap_events);
  out->n_events = n_ev;
  out->n_flits = n_ev * nfl;
  out->flit_words = words;
  out->n_frames = ch->call_frames;
  if (out->events) {
    const uint64_t k = std::min<uint64_t>(avail, out->cap_events);
    if (k < n_ev) trunc = true;
    if (k && !ch->drained_events)
      CK(cudaMemcpy(out->events, ch->events.p, k * sizeof(rd_event), cudaMemcpyDeviceToHost));
  }
  if (out->flits) {
    const uint64_t k = std::min<uint64_t>(avail, out->cap_flits / nfl);
    if (k < n_ev) trunc = true;
    if (k && !ch->drained_flits)
      CK(cudaMemcpy(out->flits, ch->flits.p, k * nfl * words * 4, cudaMemcpyDeviceToHost));
  }
  const uint32_t nw = (uint32_t)ch->call_windows.size();
  out->n_cov_windows = nw;
  if (nw) {
    const uint32_t k = std::min<uint32_t>(nw, out->cap_cov_windows);
    if (k < nw) trunc = true;
    std::vector<unsigned> wf(nw);
    CK(cudaMemcpy(wf.data(), ch->win_flags.p, nw * 4, cudaMemcpyDeviceToHost));
    if (out->cov_windows)
      for (uint32_t w = 0; w < k; ++w) {
        out->cov_windows[w] = ch->call_windows[w];
        out->cov_windows[w].sat_flags = (uint8_t)wf[w];
      }
    const uint32_t d = std::min(ch->drained_windows, k);  // already there
    if (out->cov_acc && k > d) {
      const size_t per = (size_t)c.n_fft * ch->P * 2;
      CK(cudaMemcpy(out->cov_acc + d * per, ch->cov_out.p + d * per, (size_t)(k - d) * per * 8,
                    cudaMemcpyDeviceToHost));
    }
  }
  return trunc ? fail(RD_ETRUNC, "output capacity exceeded") : RD_OK;
}

rd_status rd_chain_process(rd_chain* ch, const rd_cplx16* adc, uint64_t n, uint64_t ld,
                           rd_output* out) {
  if (!ch || !adc || !out) return fail(RD_EINVAL, "null argument");
  rd::NvtxRange range("rd_chain_process");
  const rd_config& c = ch->cfg;
  if (n % c.n_fft) return fail(RD_EINVAL, "n=%llu is not a multiple of n_fft", (unsigned long long)n);
  if (ld < n) return fail(RD_EINVAL, "ld < n");
  const uint32_t N = c.n_fft, C = c.n_chan, B = c.n_beams;
  const uint64_t frames = n / N;
  const uint64_t sld = (uint64_t)c.max_frames * N;
  CK(ch->stage.ensure((size_t)C * sld));
  CK(ch->stage2.ensure((size_t)C * sld));
  CK(ch->stage3.ensure((size_t)C * sld));
  if (!ch->copy_stream) {
    CK(cudaStreamCreateWithFlags(&ch->copy_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 3; ++b) {
      CK(cudaEventCreateWithFlags(&ch->ev_ready[b], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ch->ev_free[b], cudaEventDisableTiming));
    }
  }
  const bool taps = out->tap_pfb || out->tap_spectrum || out->tap_beams || out->tap_power;
  if (taps) {
    CK(ch->tap_pfb.ensure((size_t)c.max_frames * C * N));
    if (out->tap_beams && !ch->beams_bn.p) CK(ch->beams_bn.ensure((size_t)c.max_frames * N * B));
  }
  const uint64_t cap = out->events ? out->cap_events : default_cap(c, frames);
  rd_status st = begin_call(ch, frames, std::max<uint64_t>(cap, 1));
  if (st != RD_OK) return st;
  // chunk i is copied into staging buffer i % 3 on the copy stream once the
  // chain has finished with that buffer's previous chunk, so the copies of
  // chunks i + 1 and i + 2 may run while chunk i computes
  for (int b = 0; b < 3; ++b) CK(cudaEventRecord(ch->ev_free[b], ch->stream));
  std::vector<uint32_t> hb;
  // results into page-locked host buffers are copied chunk by chunk on a third
  // stream while later chunks compute: once chunk i - 1 has finished, the
  // host reads its event count (a page-locked snapshot) and queues the copy of
  // exactly its events, packets and closed windows. Other host buffers are
  // filled at the end.
  auto pinned = [](const void* p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.type == cudaMemoryTypeHost;
  };
  const bool dev_ev = !taps && pinned(out->events), dev_fl = !taps && pinned(out->flits);
  const bool dev_cov = !taps && pinned(out->cov_acc);
  const bool drain = dev_ev || dev_fl || dev_cov;
  // chunk sizes: a quarter-size first chunk, so that compute starts after a
  // quarter of a full copy, then chunks growing by half each time (a chunk's
  // copy, at ~1.5x the chain's sample rate, then ends while its predecessor
  // computes), full chunks, and a quarter-size last one, so that less compute
  // and fewer results follow the last copy (the results do not depend on the
  // chunking)
  std::vector<uint32_t> sizes;
  {
    const uint64_t L = ch->launch_frames, q = std::max<uint64_t>(L / 4u, 1u);
    uint64_t left = frames;
    if (frames >= 2u * L) {
      for (uint64_t s0 = q; s0 < L && left > s0 + L + q; s0 = std::min<uint64_t>(L, s0 * 3u / 2u)) {
        sizes.push_back((uint32_t)s0);
        left -= s0;
      }
      while (left > L + q) {
        sizes.push_back((uint32_t)L);
        left -= L;
      }
      if (left > q) {
        sizes.push_back((uint32_t)(left - q));
        left = q;
      }
      sizes.push_back((uint32_t)left);
    } else {
      while (left) {
        const uint64_t F = std::min(L, left);
        sizes.push_back((uint32_t)F);
        left -= F;
      }
    }
  }
  const uint64_t n_chunks = sizes.size();
  const uint32_t nfl = rd_detection_flits(c.packet_w);
  const size_t pk = (size_t)nfl * rd_flit_words(c.packet_w);
  if (drain) {
    if (!ch->out_stream) CK(cudaStreamCreateWithFlags(&ch->out_stream, cudaStreamNonBlocking));
    while (ch->ev_snap.size() < n_chunks) {
      cudaEvent_t e = nullptr;
      CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ch->ev_snap.push_back(e);
    }
    if (ch->h_snaps_n < n_chunks) {
      if (ch->h_snaps) CK(cudaFreeHost(ch->h_snaps));
      ch->h_snaps = nullptr;
      ch->h_snaps_n = 0;
      CK(cudaHostAlloc((void**)&ch->h_snaps, n_chunks * sizeof(unsigned long long),
                       cudaHostAllocDefault));
      ch->h_snaps_n = n_chunks;
    }
  }
  const uint64_t cap_ev = std::min<uint64_t>(ch->call_cap_events, out->cap_events);
  const uint64_t cap_fl = std::min<uint64_t>(ch->call_cap_events, out->cap_flits / nfl);
  const size_t cov_per = (size_t)N * ch->P * 2;
  std::vector<uint32_t> win_end(n_chunks, 0);  // windows closed by the end of each chunk
  // queue the copies of chunk k's results (its snapshot has landed)
  auto drain_chunk = [&](uint64_t k) -> rd_status {
    CK(cudaEventSynchronize(ch->ev_snap[k]));  // chunk k is done: its results are final
    const uint64_t lo = k ? ch->h_snaps[k - 1] : 0, hi = ch->h_snaps[k];
    const uint64_t e1 = std::min(hi, cap_ev), f1 = std::min(hi, cap_fl);
    if (dev_ev && e1 > lo)
      CK(cudaMemcpyAsync(out->events + lo, ch->events.p + lo, (e1 - lo) * sizeof(rd_event),
                         cudaMemcpyDeviceToHost, ch->out_stream));
    if (dev_fl && f1 > lo)
      CK(cudaMemcpyAsync(out->flits + lo * pk, ch->flits.p + lo * pk, (f1 - lo) * pk * 4,
                         cudaMemcpyDeviceToHost, ch->out_stream));
    const uint32_t w0 = k ? win_end[k - 1] : 0u;
    const uint32_t w1 = std::min<uint32_t>(win_end[k], out->cap_cov_windows);
    if (dev_cov && w1 > w0)
      CK(cudaMemcpyAsync(out->cov_acc + w0 * cov_per, ch->cov_out.p + w0 * cov_per,
                         (size_t)(w1 - w0) * cov_per * 8, cudaMemcpyDeviceToHost, ch->out_stream));
    if (dev_cov) ch->drained_windows = std::max(ch->drained_windows, w1);
    return RD_OK;
  };
  unsigned bi = 0, chunk = 0;
  for (uint64_t f = 0; chunk < n_chunks; f += sizes[chunk], bi = bi == 2u ? 0u : bi + 1u, ++chunk) {
    const uint32_t F = sizes[chunk];
    uint32_t* stg = bi == 0u ? ch->stage.p : (bi == 1u ? ch->stage2.p : ch->stage3.p);
    CK(cudaStreamWaitEvent(ch->copy_stream, ch->ev_free[bi], 0));
    CK(cudaMemcpy2DAsync(stg, sld * 4, adc + f * N, ld * 4, (size_t)F * N * 4, C,
                         cudaMemcpyHostToDevice, ch->copy_stream));
    CK(cudaEventRecord(ch->ev_ready[bi], ch->copy_stream));
    CK(cudaStreamWaitEvent(ch->stream, ch->ev_ready[bi], 0));
    const uint64_t g0 = ch->frame;
    st = run_chunk(ch, stg, sld, F, taps ? ch->tap_pfb.p : nullptr);
    if (st != RD_OK) return st;
    CK(cudaEventRecord(ch->ev_free[bi], ch->stream));
    if (drain) {
      // the chunk's event count (its CFAR's events_call) into the snapshot
      win_end[chunk] = (uint32_t)ch->call_windows.size();
      CK(cudaMemcpyAsync(ch->h_snaps + chunk, &ch->stats.p->events_call,
                         sizeof(unsigned long long), cudaMemcpyDeviceToHost, ch->stream));
      CK(cudaEventRecord(ch->ev_snap[chunk], ch->stream));
    }
    if (taps) {  // debug taps: copied out chunk by chunk
      CK(cudaStreamSynchronize(ch->stream));
      const size_t fcn = (size_t)F * C * N, fbn = (size_t)F * B * N;
      if (out->tap_pfb)
        CK(cudaMemcpy(out->tap_pfb + f * C * N, ch->tap_pfb.p, fcn * 4, cudaMemcpyDeviceToHost));
      if (out->tap_spectrum) {
        for (uint32_t k = 0; k < F; ++k) {
          const uint64_t slot = (g0 + k) % ch->R;
          CK(cudaMemcpy(out->tap_spectrum + (f + k) * N * C, ch->ring.p + slot * N * C,
                        (size_t)N * C * 4, cudaMemcpyDeviceToHost));
        }
      }
      if (out->tap_power)
        CK(cudaMemcpy(out->tap_power + f * B * N, ch->power.p, fbn * 4, cudaMemcpyDeviceToHost));
      if (out->tap_beams && ch->beams_bn.p) {
        hb.resize(fbn);
        CK(cudaMemcpy(hb.data(), ch->beams_bn.p, fbn * 4, cudaMemcpyDeviceToHost));
        for (uint32_t k = 0; k < F; ++k)
          for (uint32_t b = 0; b < B; ++b)
            for (uint32_t i = 0; i < N; ++i)
              out->tap_beams[((f + k) * B + b) * N + i] = hb[((size_t)k * N + i) * B + b];
      }
    }
  }
  // every chunk's copies and launches are queued before the first host wait
  // (the input copies wait for their staging buffer on the device), so a
  // stalled host thread stalls neither the copies in nor the compute; the
  // results then leave chunk by chunk as each one ends
  if (drain)
    for (uint64_t k = 0; k < n_chunks; ++k) {
      st = drain_chunk(k);
      if (st != RD_OK) return st;
    }
  st = end_call(ch);
  if (st != RD_OK) return st;
  ch->drained_events = dev_ev;
  ch->drained_flits = dev_fl;
  st = rd_chain_fetch(ch, out);
  // what was copied chunk by chunk went to this call's buffers only: a later
  // rd_chain_fetch into other buffers copies everything again
  ch->drained_events = ch->drained_flits = false;
  ch->drained_windows = 0;
  return st;
}

__global__ void k_cov_flush(long long* acc_re, long long* acc_im, unsigned* sticky,
                            unsigned* satcnt, uint64_t n, long long* out, int emit) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (emit) {
    out[2 * i] = acc_re[i];
    out[2 * i + 1] = acc_im[i];
  }
  acc_re[i] = 0;
  acc_im[i] = 0;
  sticky[i] = 0;
  satcnt[2 * i] = 0;
  satcnt[2 * i + 1] = 0;
}
__global__ void k_cov_flush_stats(DevStats* s) {
  s->cov_flags = 0;
  s->cov_sat_steps = 0;
}

rd_status rd_chain_flush_cov(rd_chain* ch, rd_output* out) {
  if (!ch || !out) return fail(RD_EINVAL, "null argument");
  out->n_cov_windows = 0;
  const rd_config& c = ch->cfg;
  if (c.cov_source == RD_COV_OFF || !ch->P) return RD_OK;
  const uint64_t n = (uint64_t)c.n_fft * ch->P;
  const bool emit = ch->cov_count != 0;
  if (emit && out->cap_cov_windows < 1) return fail(RD_ETRUNC, "no room for the flushed window");
  CK(ch->cov_out.ensure(n * 2));
  k_cov_flush<<<(unsigned)((n + 255) / 256), 256, 0, ch->stream>>>(
      ch->acc_re.p + ch->acc_cur * (size_t)n, ch->acc_im.p + ch->acc_cur * (size_t)n, ch->sticky.p, ch->satcnt.p, n, ch->cov_out.p, emit ? 1 : 0);
  k_cov_flush_stats<<<1, 1, 0, ch->stream>>>(ch->stats.p);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ch->stream));
  if (emit) {
    rd_cov_window h{};
    const uint32_t wl = c.cov_window ? c.cov_window : 1u;
    h.window_id = ch->cov_window_id;
    h.sample_count = ch->cov_count;
    h.end_frame = (uint32_t)ch->frame;
    h.flushed = 1;
    h.truncated = ch->cov_count != wl;
    if (out->cov_windows) out->cov_windows[0] = h;
    if (out->cov_acc) CK(cudaMemcpy(out->cov_acc, ch->cov_out.p, n * 16, cudaMemcpyDeviceToHost));
    out->n_cov_windows = 1;
  }
  ch->cov_count = 0;
  ch->cov_window_id = 0;
  return RD_OK;
}

rd_status rd_chain_set_profiling(rd_chain* ch, int on) {
  if (!ch) return fail(RD_EINVAL, "null chain");
  ch->profiling = on != 0;
  return RD_OK;
}

rd_status rd_chain_kernel_times(rd_chain* ch, rd_kernel_time* out, uint32_t cap, uint32_t* n) {
  if (!ch || !n) return fail(RD_EINVAL, "null argument");
  CK(cudaStreamSynchronize(ch->stream));
  for (const rd_chain::Pending& p : ch->pending) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, p.a, p.b));
    ch->ktime[p.id] += ms;
    ch->klaunch[p.id] += 1;
    ch->pool.push_back(p.a);
    ch->pool.push_back(p.b);
  }
  ch->pending.clear();
  uint32_t k = 0;
  for (int i = 0; i < 8; ++i) {
    if (!ch->klaunch[i]) continue;
    if (out && k < cap) {
      std::memset(&out[k], 0, sizeof(out[k]));
      std::strncpy(out[k].name, kKernelNames[i], sizeof(out[k].name) - 1);
      out[k].launches = ch->klaunch[i];
      out[k].total_ms = ch->ktime[i];
    }
    ++k;
    ch->klaunch[i] = 0;
    ch->ktime[i] = 0;
  }
  *n = k;
  return RD_OK;
}

rd_status rd_chain_set_launch_frames(rd_chain* ch, uint32_t frames) {
  if (!ch) return fail(RD_EINVAL, "null argument");
  if (frames == 0 || frames > ch->cfg.max_frames)
    return fail(RD_EINVAL, "launch frames %u outside 1..%u", frames, ch->cfg.max_frames);
  ch->launch_frames = frames;
  return RD_OK;
}

rd_status rd_chain_reset(rd_chain* ch, void* stream) {
  if (!ch) return fail(RD_EINVAL, "null argument");
  const rd_config& c = ch->cfg;
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  const uint32_t D = c.taps > 1 ? c.taps - 1 : 1;
  const size_t tail = (size_t)c.n_chan * D * c.n_fft * 4;
  // the chain's own stream may still be running the previous call (under
  // stream capture the graph's own dependencies order the replays instead)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(s, &cap));
  if (cap == cudaStreamCaptureStatusNone) {
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, ch->stream));
    CK(cudaStreamWaitEvent(s, ev, 0));
    cudaEventDestroy(ev);
  }
  CK(cudaMemsetAsync(ch->tail[0].p, 0, tail, s));
  CK(cudaMemsetAsync(ch->tail[1].p, 0, tail, s));
  CK(cudaMemsetAsync(ch->stats.p, 0, sizeof(DevStats), s));
  if (ch->P) {
    const size_t k = (size_t)c.n_fft * ch->P;
    CK(cudaMemsetAsync(ch->acc_re.p, 0, 2 * k * 8, s));
    CK(cudaMemsetAsync(ch->acc_im.p, 0, 2 * k * 8, s));
    CK(cudaMemsetAsync(ch->sticky.p, 0, k * 4, s));
    CK(cudaMemsetAsync(ch->satcnt.p, 0, 2 * k * 4, s));
  }
  if (ch->eng_pairs) CK(cudaMemsetAsync(ch->eng_acc.p, 0, 4u * ch->eng_pairs * sizeof(long long), s));
  ch->eng_cur = 0;
  ch->tail_cur = 0;
  ch->acc_cur = 0;
  ch->frame = 0;
  ch->cov_count = 0;
  ch->cov_window_id = 0;
  const HistMirror h0 = ch->hist;
  ch->hist = HistMirror{};
  ch->hist.n_ant = h0.n_ant;
  ch->hist.n = h0.n;
  ch->hist.lanes = h0.lanes;
  ch->hist.frames_max = h0.frames_max;
  ch->hist.depth = h0.frames_max;  // a new model's depth
  ch->host_st = rd_stats{};
  ch->align_seq = 0;
  ch->call_frames = 0;
  ch->call_windows.clear();
  return RD_OK;
}

rd_status rd_chain_set_history_depth(rd_chain* ch, uint32_t frames) {
  if (!ch) return fail(RD_EINVAL, "rd_chain_set_history_depth: null chain");
  HistMirror& h = ch->hist;
  h.depth = std::min<unsigned>(std::max<unsigned>(frames, 1u), h.frames_max);
  h.epoch += 1;
  h.frames_done = 0;
  h.done_slot = 0;
  h.base = ch->frame;  // the stored frames mean nothing now; new ones count from here
  return RD_OK;
}

// ---- checkpoint / resume --------------------------------------------------
}  // extern "C"

namespace {

constexpr char kStateMagic[8] = {'r', 'd', 's', 't', 'a', 't', 'e', '1'};

// The blob: this header, then DevStats, the current delay line, the current
// covariance accumulators (re, im), sticky flags, saturation counts, the
// beat-stream engine's open-window accumulators, and the last `ring_frames`
// frames of the history ring, oldest first.
struct StateHeader {
  char magic[8];
  uint32_t version, cfg_bytes;
  rd_config cfg;
  uint32_t P, ring_frames;
  uint64_t frame;
  uint32_t cov_count, cov_window_id, align_seq, pad;
  HistMirror hist;
  rd_stats host_st;
  uint64_t tail_words, acc_words, eng_words, total_bytes;
};
// the header travels as raw bytes: no member may own memory
static_assert(std::is_trivially_copyable<StateHeader>::value, "the state header must be plain data");

struct StateSizes {
  uint64_t tail_words, acc_words, eng_words, ring_frames, frame_words, total;
};

StateSizes state_sizes(const rd_chain* ch) {
  const rd_config& c = ch->cfg;
  StateSizes z{};
  const uint64_t D = c.taps > 1 ? c.taps - 1u : 1u;
  z.tail_words = (uint64_t)c.n_chan * D * c.n_fft;
  z.acc_words = ch->P ? (uint64_t)c.n_fft * ch->P : 0u;
  z.ring_frames = std::min<uint64_t>(std::min<uint64_t>(c.hist_frames, ch->R), ch->frame);
  z.frame_words = (uint64_t)c.n_fft * c.n_chan;
  z.eng_words = 2u * (uint64_t)ch->eng_pairs;
  z.total = sizeof(StateHeader) + sizeof(DevStats) + z.tail_words * 4 + z.acc_words * 16 +
            z.acc_words * 4 * 3 + z.eng_words * 8 + z.ring_frames * z.frame_words * 4;
  return z;
}

// copies of the ring frames [frame - n, frame) between the ring and a
// contiguous buffer, at most two runs of slots
template <class Copy>
rd_status ring_runs(const rd_chain* ch, uint64_t n, Copy&& copy) {
  uint64_t f = ch->frame - n, done = 0;
  while (done < n) {
    const uint64_t slot = f % ch->R;
    const uint64_t run = std::min<uint64_t>(n - done, ch->R - slot);
    const rd_status st = copy(slot, done, run);
    if (st != RD_OK) return st;
    done += run;
    f += run;
  }
  return RD_OK;
}

}  // namespace

extern "C" {

uint64_t rd_chain_state_size(const rd_chain* ch) { return ch ? state_sizes(ch).total : 0u; }

rd_status rd_chain_save_state(rd_chain* ch, void* buf, uint64_t cap) {
  if (!ch || !buf) return fail(RD_EINVAL, "rd_chain_save_state: null argument");
  const StateSizes z = state_sizes(ch);
  if (cap < z.total)
    return fail(RD_EINVAL, "rd_chain_save_state: %llu bytes, the state takes %llu",
                (unsigned long long)cap, (unsigned long long)z.total);
  CK(cudaStreamSynchronize(ch->stream));
  if (ch->out_stream) CK(cudaStreamSynchronize(ch->out_stream));
  unsigned char* p = static_cast<unsigned char*>(buf);
  StateHeader h;
  std::memset(static_cast<void*>(&h), 0, sizeof(h));  // padding too: equal states, equal blobs
  std::memcpy(h.magic, kStateMagic, 8);
  h.version = 1;
  h.cfg_bytes = sizeof(rd_config);
  h.cfg = ch->cfg;
  h.P = ch->P;
  h.ring_frames = (uint32_t)z.ring_frames;
  h.frame = ch->frame;
  h.cov_count = ch->cov_count;
  h.cov_window_id = ch->cov_window_id;
  h.align_seq = ch->align_seq;
  h.hist = ch->hist;
  h.host_st = ch->host_st;
  h.tail_words = z.tail_words;
  h.acc_words = z.acc_words;
  h.eng_words = z.eng_words;
  h.total_bytes = z.total;
  std::memcpy(p, &h, sizeof(h));
  p += sizeof(h);
  CK(cudaMemcpy(p, ch->stats.p, sizeof(DevStats), cudaMemcpyDeviceToHost));
  p += sizeof(DevStats);
  CK(cudaMemcpy(p, ch->tail[ch->tail_cur].p, z.tail_words * 4, cudaMemcpyDeviceToHost));
  p += z.tail_words * 4;
  if (z.acc_words) {
    const size_t k = z.acc_words;
    CK(cudaMemcpy(p, ch->acc_re.p + ch->acc_cur * k, k * 8, cudaMemcpyDeviceToHost));
    p += k * 8;
    CK(cudaMemcpy(p, ch->acc_im.p + ch->acc_cur * k, k * 8, cudaMemcpyDeviceToHost));
    p += k * 8;
    CK(cudaMemcpy(p, ch->sticky.p, k * 4, cudaMemcpyDeviceToHost));
    p += k * 4;
    CK(cudaMemcpy(p, ch->satcnt.p, 2 * k * 4, cudaMemcpyDeviceToHost));
    p += 2 * k * 4;
  }
  if (z.eng_words) {  // the engine's open window
    CK(cudaMemcpy(p, ch->eng_acc.p + (size_t)ch->eng_cur * z.eng_words, z.eng_words * 8,
                  cudaMemcpyDeviceToHost));
    p += z.eng_words * 8;
  }
  const size_t fb = z.frame_words * 4;
  return ring_runs(ch, z.ring_frames, [&](uint64_t slot, uint64_t at, uint64_t run) -> rd_status {
    CK(cudaMemcpy(p + at * fb, ch->ring.p + slot * z.frame_words, run * fb,
                  cudaMemcpyDeviceToHost));
    return RD_OK;
  });
}

rd_status rd_chain_load_state(rd_chain* ch, const void* buf, uint64_t len) {
  if (!ch || !buf) return fail(RD_EINVAL, "rd_chain_load_state: null argument");
  StateHeader h;
  if (len < sizeof(h)) return fail(RD_EINVAL, "rd_chain_load_state: %llu bytes is no state",
                                   (unsigned long long)len);
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1 ||
      h.cfg_bytes != sizeof(rd_config))
    return fail(RD_EINVAL, "rd_chain_load_state: not a chain state of this library");
  if (std::memcmp(&h.cfg, &ch->cfg, sizeof(rd_config)) != 0 || h.P != ch->P)
    return fail(RD_EINVAL, "rd_chain_load_state: the state is of another configuration");
  const rd_config& c = ch->cfg;
  const uint64_t D = c.taps > 1 ? c.taps - 1u : 1u;
  const uint64_t frame_words = (uint64_t)c.n_fft * c.n_chan;
  const uint64_t ring_frames =
      std::min<uint64_t>(std::min<uint64_t>(c.hist_frames, ch->R), h.frame);
  const uint64_t acc_words = ch->P ? (uint64_t)c.n_fft * ch->P : 0u;
  const uint64_t eng_words = 2u * (uint64_t)ch->eng_pairs;
  const uint64_t total = sizeof(StateHeader) + sizeof(DevStats) +
                         (uint64_t)c.n_chan * D * c.n_fft * 4 + acc_words * 28 + eng_words * 8 +
                         ring_frames * frame_words * 4;
  if (h.tail_words != (uint64_t)c.n_chan * D * c.n_fft || h.acc_words != acc_words ||
      h.eng_words != eng_words ||
      h.ring_frames != ring_frames || h.total_bytes != total || len < total)
    return fail(RD_EINVAL, "rd_chain_load_state: damaged or truncated state (%llu of %llu bytes)",
                (unsigned long long)len, (unsigned long long)total);
  CK(cudaStreamSynchronize(ch->stream));
  if (ch->out_stream) CK(cudaStreamSynchronize(ch->out_stream));
  const unsigned char* p = static_cast<const unsigned char*>(buf) + sizeof(h);
  CK(cudaMemcpy(ch->stats.p, p, sizeof(DevStats), cudaMemcpyHostToDevice));
  p += sizeof(DevStats);
  CK(cudaMemcpy(ch->tail[0].p, p, h.tail_words * 4, cudaMemcpyHostToDevice));
  p += h.tail_words * 4;
  if (acc_words) {
    const size_t k = acc_words;
    CK(cudaMemcpy(ch->acc_re.p, p, k * 8, cudaMemcpyHostToDevice));
    p += k * 8;
    CK(cudaMemcpy(ch->acc_im.p, p, k * 8, cudaMemcpyHostToDevice));
    p += k * 8;
    CK(cudaMemcpy(ch->sticky.p, p, k * 4, cudaMemcpyHostToDevice));
    p += k * 4;
    CK(cudaMemcpy(ch->satcnt.p, p, 2 * k * 4, cudaMemcpyHostToDevice));
    p += 2 * k * 4;
  }
  if (eng_words) {
    CK(cudaMemcpy(ch->eng_acc.p, p, eng_words * 8, cudaMemcpyHostToDevice));
    p += eng_words * 8;
  }
  ch->eng_cur = 0;
  ch->tail_cur = 0;
  ch->acc_cur = 0;
  ch->frame = h.frame;
  ch->cov_count = h.cov_count;
  ch->cov_window_id = h.cov_window_id;
  ch->align_seq = h.align_seq;
  ch->hist = h.hist;
  ch->host_st = h.host_st;
  ch->call_frames = 0;
  ch->call_windows.clear();
  const size_t fb = frame_words * 4;
  return ring_runs(ch, ring_frames, [&](uint64_t slot, uint64_t at, uint64_t run) -> rd_status {
    CK(cudaMemcpy(ch->ring.p + slot * frame_words, p + at * fb, run * fb,
                  cudaMemcpyHostToDevice));
    return RD_OK;
  });
}

uint64_t rd_chain_footprint(const rd_config* cfg, uint64_t frames_per_call) {
  if (!cfg || rd_config_validate(cfg) != RD_OK) return 0;
  const rd_config& c = *cfg;
  const uint64_t N = c.n_fft, C = c.n_chan, B = c.n_beams, T = c.taps, F = c.max_frames;
  const uint64_t R = F + c.hist_frames, D = T > 1 ? T - 1 : 1;
  uint64_t b = 0;
  b += T * N * 4 + B * C * (4 + 16);                         // coefficients, weights
  if (c.form != RD_FORM_CUDA_CORE)
    b += (uint64_t)std::max(beam_tc_fragment_words(c.n_chan, c.n_beams),
                            beam_t5_operand_words(c.n_chan, c.n_beams)) * 4;
  b += 2 * C * D * N * 4 + R * N * C * 4;                    // delay lines, spectrum ring
  b += F * B * N * 4 + F * B * (4 + 8 + 8) + F * B * ((N + 31) / 32) * 4;  // power, CFAR
  b += sizeof(DevStats) + 5 * N * 4;
  if (pfb_pass(c)) b += F * C * N * 4;                          // PFB pass outputs
  if (c.cov_source != RD_COV_OFF) {
    const uint64_t S = c.cov_source == RD_COV_CHANNEL ? C : B;
    const uint64_t P = rd_cov_pairs(cfg);
    b += P * 8 + N * P * (2 * 2 * 8 + 4 + 8);                // pairs, state
    if (c.form != RD_FORM_CUDA_CORE) b += S * S * 4 + 4096;   // pair map, unit lists
    if (c.cov_source == RD_COV_BEAM) b += F * N * B * 4;
    const uint64_t wl = c.cov_window ? c.cov_window : 1;
    b += (frames_per_call / wl + 1) * (N * P * 16 + 4);       // closed windows of a call
  }
  if (c.engine_pairs) {  // the beat-stream engine: beam outputs, open windows
    if (c.cov_source != RD_COV_BEAM) b += F * N * B * 4;
    b += 4 * std::min<uint64_t>(c.engine_pairs, B >= 2 ? B / 2 : 1) * 8;
  }
  const uint64_t cap = frames_per_call * B * (2 + N / 16);    // default event capacity
  b += cap * (sizeof(rd_event) + (uint64_t)rd_detection_flits(c.packet_w) *
                                     rd_flit_words(c.packet_w) * 4);
  return b;
}

rd_status rd_chain_stats(const rd_chain* ch, rd_stats* st) {
  if (!ch || !st) return fail(RD_EINVAL, "null argument");
  CK(cudaStreamSynchronize(ch->stream));
  DevStats ds;
  CK(cudaMemcpy(&ds, ch->stats.p, sizeof(ds), cudaMemcpyDeviceToHost));
  if (ds.dev_timeout)
    return fail(RD_ETIMEOUT, "a bounded wait inside a tensor-core kernel gave up");
  *st = ch->host_st;
  st->frames = ch->frame;
  st->pfb_flags = ds.pfb_flags;
  st->pfb_sat_samples = ds.pfb_sat;
  for (int g = 0; g < 11; ++g) st->fft_stage_flags[g] = (ds.fft_flags >> (2 * g)) & 3u;
  st->bf_flags = ds.bf_flags;
  st->bf_sat_samples = ds.bf_sat;
  st->cov_flags = ds.cov_flags;
  st->cov_sat_steps = ds.cov_sat_steps;
  st->hist_frames_done = ch->hist.frames_done;
  st->hist_write_beats = ch->hist.c_wbeat;
  st->hist_reads = ch->hist.c_read;
  st->hist_collisions = ch->hist.c_collision;
  st->hist_errors = ch->hist.c_error;
  st->hist_overwrites = ch->hist.c_overwrite;
  st->hist_skew = ch->hist.c_skew;
  st->hist_depth = ch->hist.depth;
  st->hist_epoch = ch->hist.epoch;
  if (ch->eng_pairs) {  // windows of n_fft beats, n_fft / 2 beats a frame, no flush
    const uint64_t N = ch->cfg.n_fft, beats = ch->frame * (N / 2u);
    st->engine_window = beats >= N ? (uint32_t)((beats / N - 1u) & 0xFFFFu) : 0u;
    st->engine_samples = beats >= N ? (uint32_t)N : 0u;
    st->engine_sat = ds.eng_sat ? 1u : 0u;
  }
  st->cfar_det = ds.cfar_det;
  st->cfar_sup = ds.cfar_sup;
  st->cfar_frames = ch->frame * ch->cfg.n_beams;
  st->packets = ds.events_total;
  st->flits = ds.events_total * rd_detection_flits(ch->cfg.packet_w);
  st->next_seq = (uint32_t)(ds.events_total & 0xFFFFu);
  return RD_OK;
}

rd_status rd_chain_doppler(rd_chain* ch, uint32_t n_frames, uint32_t scale_sched,
                           rd_cplx16* out, uint8_t* stage_flags) {
  if (!ch || !out) return fail(RD_EINVAL, "null argument");
  const rd_config& c = ch->cfg;
  if (!is_pow2(n_frames) || n_frames < 8 || n_frames > 1024)
    return fail(RD_EINVAL, "n_frames %u must be a power of two in 8..1024", n_frames);
  if (n_frames > ch->frame || n_frames > ch->R)
    return fail(RD_EINVAL, "%u frames requested, %llu processed, %u held in the ring", n_frames,
                (unsigned long long)ch->frame, ch->R);
  const uint32_t N = c.n_fft, C = c.n_chan;
  const size_t n = (size_t)C * N * n_frames;
  const unsigned stages = clog2(n_frames);
  Scratch sc;
  uint32_t *dv, *dbins, *dtw;
  uint8_t* dsf = nullptr;
  CK(sc.alloc(&dv, n));
  CK(sc.alloc(&dbins, n));
  if (stage_flags) CK(sc.alloc(&dsf, (size_t)C * N * stages));
  std::vector<uint32_t> tp(5u * n_frames);
  uint32_t words = 0;
  twiddle_positions(n_frames, 1, tp.data(), &words);
  CK(sc.alloc(&dtw, words ? words : 1));
  if (words) CK(cudaMemcpy(dtw, tp.data(), words * 4, cudaMemcpyHostToDevice));
  CK(cudaStreamSynchronize(ch->stream));
  launch_doppler_gather(ch->ring.p, ch->R, ch->frame - n_frames, N, C, n_frames, dv, ch->stream);
  launch_fft_block(n_frames, 1, scale_sched, 1, dtw, dv, C * N, nullptr, dbins, dsf, ch->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(ch->stream));
  CK(cudaMemcpy(out, dbins, n * 4, cudaMemcpyDeviceToHost));
  if (stage_flags) CK(cudaMemcpy(stage_flags, dsf, (size_t)C * N * stages, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_chain_read_history(rd_chain* ch, uint32_t bin, uint32_t frame_off, rd_cplx16* vec,
                                uint32_t* frame_id, uint32_t* flags) {
  if (!ch || !vec || !frame_id || !flags) return fail(RD_EINVAL, "null argument");
  const HistMirror::Read r = ch->hist.locate(bin, frame_off);
  const uint32_t C = ch->cfg.n_chan, N = ch->cfg.n_fft;
  if (r.valid_data || ch->hist.slot0_valid) {
    // the slot holds the newest frame written to it, which is frame_id
    // whenever frame_off is in range or clamped (history_model.hpp:294-305);
    // with no frame done in this epoch the read lands on slot 0, which still
    // holds what an earlier epoch wrote there
    const uint64_t slot =
        (r.valid_data ? ch->hist.base + r.frame_id : ch->hist.slot0_frame) % ch->R;
    CK(cudaStreamSynchronize(ch->stream));
    CK(cudaMemcpy(vec, ch->ring.p + (slot * N + ((bin & 0xFFFFu) % N)) * C, (size_t)C * 4,
                  cudaMemcpyDeviceToHost));
  } else {
    std::memset(vec, 0, (size_t)C * 4);
  }
  *frame_id = r.frame_id;
  *flags = r.flags;
  ch->hist.count_reads(r.flags, 1);
  return RD_OK;
}

// ---------------------------------------------------------------------------
// Per-block entry points: copy in, one kernel, copy out.
// ---------------------------------------------------------------------------

rd_status rd_pfb_run(uint32_t phases, uint32_t taps, const rd_cplx16* coeff, rd_cplx16* state,
                     const rd_cplx16* in, uint32_t beats, rd_cplx16* out, uint8_t* flags_out) {
  if (!coeff || !state || !in || !out || phases == 0 || taps == 0 || taps > 64)
    return fail(RD_EINVAL, "bad argument");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t *dc, *ds, *dn, *di, *dout;
  uint8_t* df = nullptr;
  const size_t D = taps > 1 ? taps - 1 : 1;
  CK(sc.alloc(&dc, (size_t)phases * taps));
  CK(sc.alloc(&ds, D * phases));
  CK(sc.alloc(&dn, D * phases));
  CK(sc.alloc(&di, (size_t)beats * phases));
  CK(sc.alloc(&dout, (size_t)beats * phases));
  if (flags_out) CK(sc.alloc(&df, (size_t)beats * phases));
  CK(cudaMemcpy(dc, coeff, (size_t)phases * taps * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ds, state, D * phases * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(di, in, (size_t)beats * phases * 4, cudaMemcpyHostToDevice));
  launch_pfb_block(phases, taps, dc, ds, di, beats, dout, df, 0);
  launch_tail_update(di, 0, ds, dn, beats, 1, phases, taps, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, dout, (size_t)beats * phases * 4, cudaMemcpyDeviceToHost));
  if (flags_out) CK(cudaMemcpy(flags_out, df, (size_t)beats * phases, cudaMemcpyDeviceToHost));
  if (taps > 1) CK(cudaMemcpy(state, dn, D * phases * 4, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_fft_run(uint32_t n_fft, uint32_t spc, uint32_t sched, int reorder,
                     const rd_cplx16* in, uint32_t frames, rd_cplx16* out, rd_cplx16* bins,
                     uint8_t* stage_flags) {
  if (!in || !is_pow2(n_fft) || n_fft < 8 || n_fft > 1024 || (spc != 1 && spc != 2) ||
      n_fft / spc < 4)
    return fail(RD_EINVAL, "invalid FFT geometry (fft_ref.hpp:216-219)");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t *di, *dout = nullptr, *dbins = nullptr;
  uint8_t* dsf = nullptr;
  const size_t n = (size_t)frames * n_fft;
  const unsigned stages = clog2(n_fft);
  CK(sc.alloc(&di, n));
  if (out) CK(sc.alloc(&dout, n));
  if (bins) CK(sc.alloc(&dbins, n));
  if (stage_flags) CK(sc.alloc(&dsf, (size_t)frames * stages));
  CK(cudaMemcpy(di, in, n * 4, cudaMemcpyHostToDevice));
  std::vector<uint32_t> tp(5u * n_fft);
  uint32_t words = 0;
  twiddle_positions(n_fft, spc, tp.data(), &words);
  uint32_t* dtw;
  CK(sc.alloc(&dtw, words ? words : 1));
  if (words) CK(cudaMemcpy(dtw, tp.data(), words * 4, cudaMemcpyHostToDevice));
  launch_fft_block(n_fft, spc, sched, reorder, dtw, di, frames, dout, dbins, dsf, 0);
  CK(cudaGetLastError());
  if (out) CK(cudaMemcpy(out, dout, n * 4, cudaMemcpyDeviceToHost));
  if (bins) CK(cudaMemcpy(bins, dbins, n * 4, cudaMemcpyDeviceToHost));
  if (stage_flags) CK(cudaMemcpy(stage_flags, dsf, (size_t)frames * stages, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_bf_run(uint32_t n_ant, uint32_t n_beams, const rd_cplx16* w, const rd_cplx16* x,
                    uint64_t n_vec, rd_cplx16* y, int64_t* acc, uint8_t* flags, uint32_t form) {
  if (!w || !x || !y || n_ant == 0 || n_beams == 0 || form > RD_FORM_TENSOR_WARP)
    return fail(RD_EINVAL, "bad argument");
  if (form != RD_FORM_CUDA_CORE && n_ant > RD_TC_MAX_CHAN)
    return fail(RD_EINVAL, "the tensor form takes at most %u antennas", RD_TC_MAX_CHAN);
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t *dw, *dx, *dy;
  long long* dacc = nullptr;
  uint8_t* df = nullptr;
  DevStats* dst;
  CK(sc.alloc(&dw, (size_t)n_ant * n_beams));
  CK(sc.alloc(&dx, n_vec * n_ant));
  CK(sc.alloc(&dy, n_vec * n_beams));
  CK(sc.alloc(&dst, 1));
  if (acc) CK(sc.alloc(&dacc, n_vec * n_beams * 2));
  if (flags) CK(sc.alloc(&df, n_vec * n_beams));
  CK(cudaMemcpy(dw, w, (size_t)n_ant * n_beams * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dx, x, n_vec * n_ant * 4, cudaMemcpyHostToDevice));
  CK(cudaMemset(dst, 0, sizeof(DevStats)));
  if (form != RD_FORM_CUDA_CORE) {
    // the vectors as a one-bin "ring" of n_vec frames, in launches of < 2^31 rows
    const bool t5 = form == RD_FORM_TENSOR && beam_t5_ok(n_ant, n_beams);
    std::vector<uint32_t> frag(t5 ? beam_t5_operand_words(n_ant, n_beams)
                                  : beam_tc_fragment_words(n_ant, n_beams));
    if (t5)
      beam_t5_operand(w, n_ant, n_beams, frag.data());
    else
      beam_tc_fragments(w, n_ant, n_beams, frag.data());
    uint32_t* dfrag;
    CK(sc.alloc(&dfrag, frag.size()));
    CK(cudaMemcpy(dfrag, frag.data(), frag.size() * 4, cudaMemcpyHostToDevice));
    const uint64_t step = 1ull << 30;
    for (uint64_t v0 = 0; v0 < n_vec; v0 += step) {
      const uint32_t F = (uint32_t)(n_vec - v0 < step ? n_vec - v0 : step);
      BeamParams bp{};
      bp.ring = dx + v0 * n_ant;
      bp.ring_frames = F;
      bp.w_frag = dfrag;
      bp.w_t5 = dfrag;
      bp.y_rows = dy + v0 * n_beams;
      bp.acc_rows = dacc ? dacc + v0 * n_beams * 2 : nullptr;
      bp.flag_rows = df ? df + v0 * n_beams : nullptr;
      bp.F = F;
      bp.C = n_ant;
      bp.N = 1;
      bp.B = n_beams;
      bp.stats = dst;
      if (t5)
        launch_beam_t5(bp, 0);
      else
        launch_beam_tc(bp, 0);
    }
  } else {
    launch_bf_block(n_ant, n_beams, dw, dx, n_vec, dy, dacc, df, 0);
  }
  CK(cudaGetLastError());
  DevStats hs;
  CK(cudaMemcpy(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost));
  if (hs.dev_timeout) return fail(RD_ETIMEOUT, "a bounded wait inside the tensor-core kernel gave up");
  CK(cudaMemcpy(y, dy, n_vec * n_beams * 4, cudaMemcpyDeviceToHost));
  if (acc) CK(cudaMemcpy(acc, dacc, n_vec * n_beams * 16, cudaMemcpyDeviceToHost));
  if (flags) CK(cudaMemcpy(flags, df, n_vec * n_beams, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_power_run(const rd_cplx16* x, uint64_t n, int64_t* power) {
  if (!x || !power) return fail(RD_EINVAL, "null argument");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t* dx;
  long long* dp;
  CK(sc.alloc(&dx, n));
  CK(sc.alloc(&dp, n));
  CK(cudaMemcpy(dx, x, n * 4, cudaMemcpyHostToDevice));
  launch_power_block(dx, n, dp, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpy(power, dp, n * 8, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_cross_power_run(const rd_cplx16* x, const rd_cplx16* y, uint64_t n, int64_t* cross) {
  if (!x || !y || !cross) return fail(RD_EINVAL, "null argument");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t *dx, *dy;
  long long* dc;
  CK(sc.alloc(&dx, n));
  CK(sc.alloc(&dy, n));
  CK(sc.alloc(&dc, 2 * n));
  CK(cudaMemcpy(dx, x, n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dy, y, n * 4, cudaMemcpyHostToDevice));
  launch_cross_block(dx, dy, n, dc, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpy(cross, dc, n * 16, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_cfar_run(const int64_t* cells, uint32_t n, uint32_t frames, const rd_config* cfg,
                      const uint32_t* frame_ids, rd_event* events, uint64_t cap,
                      uint64_t* n_events) {
  if (!cells || !cfg || !frame_ids || !n_events || n == 0 || n > 1024)
    return fail(RD_EINVAL, "bad argument (frames of 1..1024 cells)");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  long long* dc;
  uint32_t *dfid, *dcnt, *dds, *dmask;
  unsigned long long* dtot;
  uint4* dslot;
  rd_event* dev = nullptr;
  DevStats* dst;
  CK(sc.alloc(&dc, (size_t)frames * n));
  CK(sc.alloc(&dfid, frames));
  CK(sc.alloc(&dcnt, frames));
  CK(sc.alloc(&dds, frames));
  CK(sc.alloc(&dmask, (size_t)frames * ((n + 31) / 32)));
  CK(sc.alloc(&dtot, cfar_tiles(frames)));
  CK(sc.alloc(&dslot, (size_t)frames * kCfarSlots));
  CK(sc.alloc(&dst, 1));
  CK(sc.alloc(&dev, std::max<uint64_t>(cap, 1)));
  CK(cudaMemcpy(dc, cells, (size_t)frames * n * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dfid, frame_ids, (size_t)frames * 4, cudaMemcpyHostToDevice));
  CK(cudaMemset(dst, 0, sizeof(DevStats)));
  CfarParams p{};
  p.cells_i64 = (const int64_t*)dc;
  p.frames = frames;
  p.n = n;
  p.beams = 1;
  p.frame_ids = dfid;
  p.enable = cfg->cfar_enable != 0;
  p.go = cfg->cfar_mode == RD_CFAR_GO;
  p.dense = cfg->cfar_out_mode == RD_CFAR_DENSE;
  p.gl = std::min(cfg->guard_lead, cfg->max_guard);
  p.gg = std::min(cfg->guard_lag, cfg->max_guard);
  p.rl = std::min(cfg->ref_lead, cfg->max_ref);
  p.rg = std::min(cfg->ref_lag, cfg->max_ref);
  p.alpha = cfg->alpha;
  p.counts = dcnt;
  p.detsup = dds;
  p.mask = dmask;
  p.totals = dtot;
  p.slots = dslot;
  p.vec = (n % 4u) == 0;  // cudaMalloc'd cells: 256-byte aligned
  p.ev16 = 1;
  p.events = dev;
  p.cap = cap;
  p.stats = dst;
  launch_cfar(p, 0);
  CK(cudaGetLastError());
  DevStats hs;
  CK(cudaMemcpy(&hs, dst, sizeof(hs), cudaMemcpyDeviceToHost));
  *n_events = hs.events_call;
  const uint64_t k = std::min<uint64_t>(hs.events_call, cap);
  if (k && events) CK(cudaMemcpy(events, dev, k * sizeof(rd_event), cudaMemcpyDeviceToHost));
  return hs.events_call > cap ? fail(RD_ETRUNC, "event capacity exceeded") : RD_OK;
}

rd_status rd_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w, uint32_t src_id,
                       uint32_t dest, uint32_t vc, uint32_t seq0, uint32_t* flits) {
  if (!ev || !flits || packet_w < 64 || packet_w > 512 || (packet_w % 32) != 0)
    return fail(RD_EINVAL, "bad argument");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  rd_event* de;
  uint32_t* df;
  const size_t nw = (size_t)n * rd_detection_flits(packet_w) * rd_flit_words(packet_w);
  CK(sc.alloc(&de, n));
  CK(sc.alloc(&df, nw));
  CK(cudaMemcpy(de, ev, n * sizeof(rd_event), cudaMemcpyHostToDevice));
  launch_packetize(de, n, packet_w, src_id, dest, vc, seq0, df, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpy(flits, df, nw * 4, cudaMemcpyDeviceToHost));
  return RD_OK;
}

rd_status rd_fxp_apply(const uint32_t* op, const int64_t* a, const int64_t* b, const uint32_t* sh,
                       const uint32_t* w, uint64_t n, int64_t* y, uint8_t* flags) {
  if (!op || !a || !b || !sh || !w || !y || !flags) return fail(RD_EINVAL, "null argument");
  if (!rd_device_ok()) return fail(RD_EDEVICE, "no usable CUDA device");
  Scratch sc;
  uint32_t *dop, *dsh, *dw;
  long long *da, *db, *dy;
  uint8_t* df;
  CK(sc.alloc(&dop, n));
  CK(sc.alloc(&dsh, n));
  CK(sc.alloc(&dw, n));
  CK(sc.alloc(&da, n));
  CK(sc.alloc(&db, n));
  CK(sc.alloc(&dy, n));
  CK(sc.alloc(&df, n));
  CK(cudaMemcpy(dop, op, n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dsh, sh, n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dw, w, n * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(da, a, n * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(db, b, n * 8, cudaMemcpyHostToDevice));
  launch_fxp(dop, (const int64_t*)da, (const int64_t*)db, dsh, dw, n, (int64_t*)dy, df, 0);
  CK(cudaGetLastError());
  CK(cudaMemcpy(y, dy, n * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(flags, df, n, cudaMemcpyDeviceToHost));
  return RD_OK;
}

}  // extern "C"

rd_egress_source rd::chain_egress_source(const rd_chain* ch) {
  rd_egress_source e{};
  e.flits = ch->flits.p;
  e.count_dev = (const uint64_t*)&ch->stats.p->scan_scratch[0];  // set by k_call_end
  e.n_packets = ch->flits.p ? ch->call_cap_events : 0;
  e.dest = ch->cfg.dest;
  return e;
}

uint32_t rd::chain_packet_w(const rd_chain* ch) { return ch->cfg.packet_w; }

namespace {

static_assert(sizeof(rd_event) == 32, "an event is two 16-byte words");

// The call's count and flag, and its first min(count, call_cap, cap) events
// and packets, into mapped host memory (grid-stride, 16-byte words for the
// events)
__global__ void k_export(const DevStats* st, const rd_event* ev, const uint32_t* fl,
                         uint64_t call_cap, uint64_t cap, uint32_t pk_words, rd::ExportHdr* hdr,
                         rd_event* ev_out, uint32_t* fl_out) {
  const uint64_t n = st->scan_scratch[0];
  const uint64_t k = n < call_cap ? (n < cap ? n : cap) : (call_cap < cap ? call_cap : cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    hdr->n_events = n;
    hdr->dev_timeout = st->dev_timeout;
  }
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
  const uint4* es = reinterpret_cast<const uint4*>(ev);
  uint4* ed = reinterpret_cast<uint4*>(ev_out);
  for (uint64_t i = t; i < 2u * k; i += nth) ed[i] = es[i];
  if (fl) {  // 16 bytes a store where both ends allow it, the tail by words
    const uint64_t nw = k * pk_words;
    const bool v16 = ((reinterpret_cast<uintptr_t>(fl) | reinterpret_cast<uintptr_t>(fl_out)) & 15u) == 0;
    const uint64_t nv = v16 ? nw / 4u : 0u;
    const uint4* fs = reinterpret_cast<const uint4*>(fl);
    uint4* fd = reinterpret_cast<uint4*>(fl_out);
    for (uint64_t i = t; i < nv; i += nth) fd[i] = fs[i];
    for (uint64_t i = 4u * nv + t; i < nw; i += nth) fl_out[i] = fl[i];
  }
}

}  // namespace

rd_status rd::chain_export(rd_chain* ch, const ExportDst& d, cudaStream_t s) {
  const rd_config& c = ch->cfg;
  const uint32_t pk_words = rd_detection_flits(c.packet_w) * rd_flit_words(c.packet_w);
  const uint32_t nw = (uint32_t)ch->call_windows.size();
  const size_t per = (size_t)c.n_fft * ch->P * 2;
  if (nw > d.cap_windows || (d.cov && (size_t)nw * per > d.cov_words))
    return fail(RD_EINVAL, "chain_export: %u windows do not fit", nw);
  // a CTA per 64 KB of the most the call can export (8 to 256 CTAs)
  const uint64_t most = std::min<uint64_t>(ch->call_cap_events, d.cap_events) *
                        (sizeof(rd_event) + (d.flits ? pk_words * 4ull : 0ull));
  const unsigned grid = (unsigned)std::min<uint64_t>(std::max<uint64_t>(most >> 16, 8u), 256u);
  k_export<<<grid, 256, 0, s>>>(ch->stats.p, ch->events.p, d.flits ? ch->flits.p : nullptr,
                                ch->call_cap_events, d.cap_events, pk_words, d.hdr, d.events,
                                d.flits);
  CK(cudaGetLastError());
  if (nw) {
    CK(cudaMemcpyAsync(d.win_flags, ch->win_flags.p, nw * sizeof(unsigned), cudaMemcpyDeviceToHost,
                       s));
    if (per && d.cov)
      CK(cudaMemcpyAsync(d.cov, ch->cov_out.p, (size_t)nw * per * 8, cudaMemcpyDeviceToHost, s));
  }
  return RD_OK;
}

const std::vector<rd_cov_window>& rd::chain_call_windows(const rd_chain* ch) {
  return ch->call_windows;
}

uint64_t rd::chain_call_cap(const rd_chain* ch) { return ch->call_cap_events; }

uint64_t rd::chain_call_frames(const rd_chain* ch) { return ch->call_frames; }

cudaStream_t rd::chain_stream(const rd_chain* ch) { return ch->stream; }

size_t rd::chain_window_words(const rd_chain* ch) { return (size_t)ch->cfg.n_fft * ch->P * 2; }

