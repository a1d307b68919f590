// rd_internal.h - launch interfaces between the host ABI (api.cu) and the
// kernel translation units (k_frontend.cu, k_backend.cu).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <atomic>
#include <vector>

#include "../../include/rd_chain.h"

namespace rd {

// Set-up that belongs to one device's context (a kernel's dynamic
// shared-memory opt-in): once() runs f the first time it is reached with a
// given device current, so every device the process uses gets its own call.
// Devices past the 64 the mask tracks run f every time (it is cheap).
struct PerDevice {
  std::atomic<unsigned long long> done{0};
  template <class F>
  void once(F&& f) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
      cudaGetLastError();
      dev = -1;
    }
    const unsigned long long bit = (dev >= 0 && dev < 64) ? 1ull << dev : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return;
    f();
    if (bit) done.fetch_or(bit, std::memory_order_acq_rel);
  }
};

// A named NVTX range for its scope: the chain's stages, calls, batch runs
// and served requests show on a profiler's timeline (nsys, ncu's range
// filters). With no tool attached an NVTX call returns at once.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Device-side cumulative statistics of one stream (zeroed at create).
struct DevStats {
  unsigned pfb_flags;
  unsigned fft_flags;       // 2 bits per sub-stage g at bits [2g+1:2g]
  unsigned bf_flags;
  unsigned cov_flags;
  unsigned long long pfb_sat;
  unsigned long long bf_sat;
  unsigned long long cov_sat_steps;
  unsigned long long cfar_det;
  unsigned long long cfar_sup;
  unsigned long long events_total;   // events emitted so far (packet seq base)
  unsigned long long events_call;    // events of the current call
  unsigned long long scan_scratch[4];
  unsigned dev_timeout;              // a bounded device wait gave up (tcgen05 kernels)
  unsigned eng_sat;                  // beat-stream engine: some pair's integrator saturated
};

// ---- the beat-stream covariance engine (k_engine.cu) ------------------------
struct EngineParams {
  const uint32_t* beams;      // [F][N][B] packed beamformer outputs of the launch
  uint32_t N, B, pairs;       // FFT size (window length in beats), beams, engine pairs
  uint64_t beats;             // beats of the launch: F x N / 2
  uint32_t count0;            // beats already in the open window
  uint32_t n_seg;             // window segments the launch touches
  const long long* acc_in;    // [pairs][re, im] the open window's accumulators
  long long* acc_out;         // [pairs][re, im] after the launch (the other buffer)
  DevStats* stats;
};
void launch_engine(const EngineParams& p, cudaStream_t s);

// ---- front end: PFB + FFT + corner turn into the spectrum ring ------------
struct FrontParams {
  const uint32_t* adc;      // chunk frame 0 of channel 0; channel c at +c*ld
  uint64_t ld;
  const uint32_t* tail;     // [C][T-1][N]: tail[c][k][p] = frame -1-k
  uint32_t* tail_out;       // the delay line after this chunk (the other buffer), or null
  const uint32_t* coeff_t;  // [T][N] (tap-major copy of the phase-major bank)
  const int2* coeff2;       // [T][N] the same, unpacked {re, im}
  uint32_t pfb32;           // 1: the bank's phase L1 norms keep every sum in int32
  const uint2* coeff_dp;    // [T][N] byte limbs {hh: re, -im, im, re}, {hl: ...} for dp2a
  uint32_t pfb_dp;          // 1: pfb32 and the limbs hold (no im = -32768): dp2a path
  uint32_t coeff_real;      // 1: every coefficient's imaginary part is 0
  uint32_t* pfb_buf;        // [max_frames][C][N] for the PFB pass's outputs (or null)
  const uint32_t* pfb_in;   // the PFB pass's outputs, [F][C][N], when it ran
  uint32_t* ring;           // [R][N][C]
  uint32_t ring_frames;     // R
  uint32_t ring_base;       // ring slot of chunk frame 0 (g0 mod R)
  uint64_t g0;              // stream frame index of chunk frame 0
  const uint32_t* tw_pos;   // per-position twiddles, twiddle_positions()
  const int2* tw2;          // the same unpacked {re, im}
  uint32_t* tap_pfb;        // [F][C][N] chunk-relative, or null
  uint32_t F, C, N, T, spc, sched;
  uint32_t safe_in;         // PFB outputs within this bound cannot saturate the FFT
  DevStats* stats;
};
// Returns the launches made: the front end writes tail_out itself where it can,
// else a second launch does (pfb_model.hpp:170-175).
unsigned launch_front(const FrontParams& p, cudaStream_t s);
// The largest per-component magnitude of the FFT input for which no
// sub-stage of an (n, spc) transform with this scaling schedule can
// saturate (k_frontend.cu).
uint32_t front_safe_input(uint32_t n, uint32_t spc, uint32_t sched);
// The geometry-specialised kernel (k_front_fast.cu); false when the geometry
// has no specialisation.
bool launch_front_fast(const FrontParams& p, cudaStream_t s);
bool front_fast_ok(uint32_t n, uint32_t spc);
// The PFB as its own frame-blocked pass (k_pfb_rows.cu), for banks whose sums
// stay in int32 and 4, 8 or 16 taps; writes [F][C][N] to out and the next
// delay line.
bool pfb_rows_ok(const FrontParams& p);
void launch_pfb_rows(const FrontParams& p, uint32_t* out, cudaStream_t s);
void launch_tail_update(const uint32_t* adc, uint64_t ld, const uint32_t* old_tail,
                        uint32_t* new_tail, uint32_t F, uint32_t C, uint32_t N,
                        uint32_t T, cudaStream_t s);

// ---- per-block front-end kernels ------------------------------------------
void launch_pfb_block(uint32_t phases, uint32_t taps, const uint32_t* coeff,
                      const uint32_t* state, const uint32_t* in, uint32_t beats,
                      uint32_t* out, uint8_t* flags, cudaStream_t s);
void launch_fft_block(uint32_t n, uint32_t spc, uint32_t sched, int reorder,
                      const uint32_t* tw_pos, const uint32_t* in, uint32_t frames,
                      uint32_t* out, uint32_t* bins, uint8_t* stage_flags, cudaStream_t s);

// Per-position twiddle tables of an (n_fft, spc) transform: for the k-th
// twiddle sub-stage s (odd s with s + 1 < log2(n/spc)), entry [k][i] is the
// twiddle lane position i multiplies by, kTw[r22_tw_exp(l2l, i) << (10-l2l)]
// with l2l = log2(n/spc) - s + 1 (fft_ref.hpp:123-133, 368-377); then, for
// spc = 2, the merge twiddle of position i, kTw[bitrev(i) << (10-l2l-1)]
// (fft_ref.hpp:139-147, 380-406). Indexing by position keeps shared-memory
// reads bank-conflict free.
void twiddle_positions(uint32_t n, uint32_t spc, uint32_t* out /* 5 * n words */,
                       uint32_t* words);

// ---- back end ----------------------------------------------------------------
struct BeamParams {
  const uint32_t* ring;     // [R][N][C]
  uint32_t ring_frames;
  uint32_t ring_base;       // ring slot of chunk frame 0
  uint64_t g0;
  const uint32_t* weights;  // [B][C]
  const int4* w_limbs;      // [B][C] {wh.re, wh.im, wl.re, wl.im}, w = 256 wh + wl
  const uint32_t* w_frag;   // warp-level tensor form: beam_tc_fragments() of the weights
  const uint32_t* w_t5;     // tcgen05 form: beam_t5_operand() of the weights
  uint32_t* power;          // [F][B][N] (or null)
  uint32_t* beams_bn;       // [F][N][B] beam samples (null unless needed)
  uint32_t* y_rows;         // per-block entry: [rows][B] y, acc, flags (or null)
  long long* acc_rows;
  uint8_t* flag_rows;
  uint32_t F, C, N, B;
  uint32_t x_safe;          // spectrum tiles within this magnitude sum exactly in int32
  int cshift;               // log2 C when C is a power of two, else -1
  DevStats* stats;          // may be null
};
void launch_beam(const BeamParams& p, cudaStream_t s);
// Tensor-core form (k_beam_tc.cu): mma fragments of the limb-split weights.
void launch_beam_tc(const BeamParams& p, cudaStream_t s);
uint32_t beam_tc_fragment_words(uint32_t C, uint32_t B);
size_t beam_tc_smem(uint32_t C);
void beam_tc_fragments(const uint32_t* w, uint32_t C, uint32_t B, uint32_t* out);
// tcgen05 form (k_beam_t5.cu): whether the geometry fits it (C <= 64 and the
// shared-memory plan), the weight operand image and the launch.
bool beam_t5_ok(uint32_t C, uint32_t B);
uint32_t beam_t5_operand_words(uint32_t C, uint32_t B);
void beam_t5_operand(const uint32_t* w, uint32_t C, uint32_t B, uint32_t* out);
void launch_beam_t5(const BeamParams& p, cudaStream_t s);

struct CovParams {
  const uint32_t* ring;     // channel source: [R][N][C]
  uint32_t ring_frames;
  uint32_t ring_base;       // ring slot of chunk frame 0
  uint64_t g0;
  uint32_t exact;           // 1: no step can saturate (see launch_cov)
  const uint32_t* beams_bn; // beam source: [F][N][B]
  uint32_t S;               // source vector length
  uint32_t src_beam;        // 1: beams_bn, 0: ring
  const uint32_t* px;
  const uint32_t* py;
  uint32_t P, F, N;
  long long* acc_re;        // [N][P] integrator state carried in
  long long* acc_im;
  long long* acc_re_out;    // [N][P] integrator state carried out (another copy)
  long long* acc_im_out;
  unsigned* sticky;         // [N][P] (re << 2 | im)
  unsigned* satcnt;         // [N][P][2]
  uint32_t count0;          // samples already in the open window
  uint32_t wl;              // effective window length
  uint32_t exp_mode, exp_k, acc_w;
  long long* out;           // [n_windows][N][P][2]
  unsigned* win_flags;      // [n_windows]
  uint32_t n_windows;       // windows that close in this chunk
  DevStats* stats;
};
void launch_cov(const CovParams& p, cudaStream_t s);

// Tensor-core form of the exact block covariance (k_cov_tc.cu). The plan is
// built once per pair table on the host: S <= 128 and no repeated pair.
struct CovTcPlan {
  uint32_t Sp, log2_sp;     // channels padded to a power of two >= 16
  uint32_t NB;              // bins per CTA
  uint32_t UPW, G;          // units per warp, CTA groups per bin block
  const uint32_t* units;    // [G][8 warps][UPW]: bin << 16 | m-tile << 8 | triple, or ~0
  const int32_t* pq;        // [S][S]: pair index of (x, y), or -1
};
struct CovTcHost {
  CovTcPlan plan;
  std::vector<uint32_t> units;
  std::vector<int32_t> pq;
};
bool cov_tc_plan(uint32_t S, const uint32_t* px, const uint32_t* py, uint32_t P,
                 CovTcHost* out);
size_t cov_tc_smem(const CovTcPlan& t);
void launch_cov_tc(const CovParams& p, const CovTcPlan& t, cudaStream_t s);
// tcgen05 form of the exact block covariance (k_cov_t5.cu): for up to 64
// source channels and windows of 64 to 256 frames; pq is the plan's pair map.
bool cov_t5_ok(uint32_t S, uint32_t wl);
void launch_cov_t5(const CovParams& p, const int32_t* pq, cudaStream_t s);

// Detections a CFAR frame keeps from its decision for the emit pass; a frame
// with more (DENSE output, clutter) re-decides its events there.
constexpr unsigned kCfarSlots = 16;

struct CfarParams {
  const uint32_t* power_u32;  // [frames][n] (chain) ...
  const int64_t* cells_i64;   // ... or raw signed cells (per-block entry)
  uint32_t frames, n;         // CFAR frames (frame*beam) and cells per frame
  uint32_t beams;             // frame index = u / beams, beam = u % beams
  uint64_t g0;                // stream frame of chunk frame 0
  const uint32_t* frame_ids;  // per CFAR frame (per-block entry) or null
  int enable, go, dense;
  uint32_t gl, gg, rl, rg, alpha;  // clamped geometry
  uint32_t* counts;           // [frames] events per CFAR frame (SUMMARY included)
  uint32_t* detsup;           // [frames] detected | suppressed << 16
  uint32_t* mask;             // [frames][ceil(n / 32)] emitted-cell bitmask
  unsigned long long* totals; // [cfar_tiles(frames)] events per 8-frame group, then per 64 groups
  uint4* slots;               // [frames][kCfarSlots] the frame's first detections
  int vec;                    // n % 4 == 0 and the cells 16-byte aligned: 16-byte loads
  int ev16;                   // events 16-byte aligned: 16-byte stores
  rd_event* events;           // output, capacity cap
  uint64_t cap;
  uint32_t* flits;            // output flits or null
  uint32_t packet_w, src_id, dest, vc, flit_words, nfl;
  DevStats* stats;
};
// Decide, then events and packets at their offsets: two launches (k_backend.cu)
void launch_cfar(const CfarParams& p, cudaStream_t s);
unsigned cfar_tiles(uint32_t frames);

void launch_bf_block(uint32_t n_ant, uint32_t n_beams, const uint32_t* w,
                     const uint32_t* x, uint64_t n_vec, uint32_t* y, long long* acc,
                     uint8_t* flags, cudaStream_t s);
void launch_power_block(const uint32_t* x, uint64_t n, long long* p, cudaStream_t s);
void launch_cross_block(const uint32_t* x, const uint32_t* y, uint64_t n, long long* c,
                        cudaStream_t s);
void launch_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w, uint32_t src,
                      uint32_t dest, uint32_t vc, uint32_t seq0, uint32_t* flits,
                      cudaStream_t s);
void launch_fxp(const uint32_t* op, const int64_t* a, const int64_t* b, const uint32_t* sh,
                const uint32_t* w, uint64_t n, int64_t* y, uint8_t* flags, cudaStream_t s);

// Records a formatted message for rd_last_error() and returns st (api.cu).
rd_status set_error(rd_status st, const char* fmt, ...);

// Slow-time vectors [C][N][H] of the last H ring frames from stream frame
// g_first on (k_frontend.cu)
void launch_doppler_gather(const uint32_t* ring, uint32_t R, uint64_t g_first, uint32_t N,
                           uint32_t C, uint32_t H, uint32_t* out, cudaStream_t s);

// The packets of the chain's last call as an egress source: its flit
// buffer, the device count of the call's events (capped at the buffer) and
// its configured destination port (api.cu)
rd_egress_source chain_egress_source(const rd_chain* ch);
uint32_t chain_packet_w(const rd_chain* ch);

// The outputs of a chain's last call exported into host memory on a stream,
// so that a host loop reads them without a synchronous copy (server.cu): a
// kernel writes the call's event count, its dev_timeout flag and at most
// cap_events events and their packets into mapped page-locked memory, and
// the closed windows' flags and sums follow by DMA into page-locked memory.
struct ExportHdr {
  unsigned long long n_events;  // the call's events (may exceed what was kept)
  unsigned dev_timeout;
  unsigned pad;
};
struct ExportDst {
  ExportHdr* hdr;        // device views of mapped page-locked memory
  rd_event* events;      // cap_events entries
  uint32_t* flits;       // cap_events packets
  uint64_t cap_events;
  unsigned* win_flags;   // page-locked host memory, cap_windows entries
  uint32_t cap_windows;
  int64_t* cov;          // page-locked host memory, cov_words
  size_t cov_words;
};
// Enqueued on s, which must be ordered after the call (the stream given to
// rd_chain_process_device). RD_EINVAL when the call's windows do not fit.
rd_status chain_export(rd_chain* ch, const ExportDst& d, cudaStream_t s);
// The window headers of the chain's last call (their sat_flags are on the
// device until exported) and its event capacity.
const std::vector<rd_cov_window>& chain_call_windows(const rd_chain* ch);
uint64_t chain_call_cap(const rd_chain* ch);
// Frames of the chain's last call.
uint64_t chain_call_frames(const rd_chain* ch);
// The chain's own stream: work enqueued on it is ordered with the chain's
// launches without events (rd_chain_process_device skips its two waits).
cudaStream_t chain_stream(const rd_chain* ch);
// Words of one closed window's sums: n_fft x pairs x (re, im).
size_t chain_window_words(const rd_chain* ch);

// rd_egress_merge on a stream (fabric.cu)
rd_status egress_merge(const rd_egress_source* src, uint32_t n_src, uint32_t packet_w,
                       uint32_t n_ports, uint32_t* ring_dev, uint64_t cap_per_port,
                       uint32_t* src_of_dev, uint64_t* port_count_dev, cudaStream_t st);

// Q1.15 twiddle table in device global memory (k_frontend.cu)
const uint32_t* twiddles_device();

}  // namespace rd
