/*
 * rd_chain.h - C ABI of the GB300 radar chain.
 *
 * The chain is the bit-exact fixed-point pipeline that the reference model
 * (fpga-professional-association/agilex-7-radar-detect, directory model/cpp)
 * computes block by block and that rtl/top/benchmark_sim_top.sv wires
 * together:
 *
 *   ADC -> polyphase FIR bank -> radix-2^2 FFT -> history / corner turn
 *       -> bin alignment -> beamforming -> power + covariance -> CA/GO-CFAR
 *       -> 176-bit detection events -> packet flits
 *
 * Every entry point computes on one GB300 (sm_103a) with hand-written CUDA
 * kernels. There is no CPU fallback: when no device is usable the call returns
 * RD_EDEVICE. Plain C types only; no exceptions cross this boundary.
 *
 * Conventions
 *   - Samples are complex Q1.15 packed in one 32-bit word, real part in the
 *     low half, imaginary in the high half (model/cpp/fxp/fxp.hpp:288-297,
 *     fxp::Complex::packed).
 *   - Flags are packed {sat_pos<<1 | sat_neg} (model/cpp/fxp/fxp.hpp:148-150).
 *   - One host thread per rd_chain handle; several handles may coexist.
 *   - rd_last_error() returns a thread-local description of the last failure.
 */
#ifndef RD_CHAIN_H_
#define RD_CHAIN_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint32_t rd_cplx16; /* packed {im, re}, re in bits 15:0 */

typedef enum rd_status {
  RD_OK = 0,
  RD_EINVAL = 1,    /* bad argument or geometry */
  RD_ENOMEM = 2,    /* device memory or admission budget refused */
  RD_ETIMEOUT = 3,  /* a bounded device wait gave up */
  RD_EDEVICE = 4,   /* no usable CUDA device, or a CUDA call failed */
  RD_ETRUNC = 5,    /* an output buffer was too small; counts say how much */
  RD_EAGAIN = 6     /* request not finished yet (rd_chain_poll) */
} rd_status;

/* CFAR (model/cpp/cfar/cfar_model.hpp:89-90) */
enum { RD_CFAR_CA = 0, RD_CFAR_GO = 1 };
enum { RD_CFAR_EVENTS = 0, RD_CFAR_DENSE = 1 };
/* CFAR event kinds (model/cpp/cfar/cfar_model.hpp:92-97) */
enum { RD_EV_DETECT = 0, RD_EV_BIN = 1, RD_EV_SUPPRESSED = 2, RD_EV_SUMMARY = 3 };

/* Covariance source vector and integrator mode
 * (model/cpp/covariance/covar_model.hpp:157). */
enum { RD_COV_OFF = 0, RD_COV_CHANNEL = 1, RD_COV_BEAM = 2 };
enum { RD_COV_BLOCK = 0, RD_COV_EXP = 1 };

/* Form of the beamforming and covariance contractions. All are bit-exact.
 * RD_FORM_CUDA_CORE: integer multiply-accumulate on the CUDA cores.
 * RD_FORM_TENSOR: the int16 operands split into 8-bit limbs held exactly in
 * fp16, multiplied on the tensor cores with fp32 accumulation whose every
 * partial sum is an integer below 2^24 (hence n_chan <= RD_TC_MAX_CHAN),
 * recombined in int64; the covariance in this form for its exact block mode.
 * The beamformer runs on the 5th-generation tensor cores (tcgen05, TMEM
 * accumulators) for up to 64 channels, else as RD_FORM_TENSOR_WARP.
 * RD_FORM_TENSOR_WARP: the same limb split on the warp-level mma
 * instruction. */
enum { RD_FORM_CUDA_CORE = 0, RD_FORM_TENSOR = 1, RD_FORM_TENSOR_WARP = 2 };
#define RD_TC_MAX_CHAN 128u

/* Stream geometry and block configuration. Zero-initialise, then fill;
 * rd_config_default() gives the values the reference's defaults imply. */
typedef struct rd_config {
  uint32_t n_chan;       /* C antennas (ADC channels), 1..128 */
  uint32_t n_fft;        /* N: FFT size = PFB phases, power of two, 8..1024 */
  uint32_t taps;         /* T: PFB taps per phase, 1..64 */
  uint32_t spc;          /* FFT samples per cycle = history lanes: 1 or 2 */
  uint32_t scale_sched;  /* FFT per-sub-stage shift mask (fft_ref.hpp:155) */
  uint32_t hist_frames;  /* H: history depth, power of two, >= 4 */
  uint32_t n_beams;      /* B: beams, 1..128 */
  /* CFAR (cfar_model.hpp:112-128) */
  uint32_t cfar_enable;
  uint32_t cfar_mode;     /* RD_CFAR_CA / RD_CFAR_GO */
  uint32_t cfar_out_mode; /* RD_CFAR_EVENTS / RD_CFAR_DENSE */
  uint32_t guard_lead, guard_lag, ref_lead, ref_lag;
  uint32_t alpha;         /* UQ8.8 threshold multiplier */
  uint32_t max_guard, max_ref; /* elaborated maxima (clamp_config) */
  /* covariance (covar_model.hpp:159-169) */
  uint32_t cov_source;    /* RD_COV_* */
  uint32_t cov_mode;      /* RD_COV_BLOCK / RD_COV_EXP */
  uint32_t cov_exp_k;     /* 0..15 */
  uint32_t cov_window;    /* window length in frames (0 behaves as 1) */
  uint32_t cov_acc_w;     /* integrator width in bits, 33..64 */
  uint32_t cov_n_pairs;   /* 0: every (i<=j) pair of the source vector */
  /* packets (packet_model.hpp:74-127) */
  uint32_t packet_w;      /* payload bits per flit, 64..512, multiple of 32 */
  uint32_t src_id, dest, vc;
  /* engine */
  uint32_t max_frames;    /* frames per internal launch (sizes device state) */
  uint32_t form;          /* RD_FORM_* of the beamformer */
  /* the RTL's telemetry-only beat-stream covariance engine (covar_model.hpp:
   * 318-416 as benchmark_sim_top.sv:1124-1200 wires it): pairs of beams
   * (2p, 2p+1) mod n_beams of every beamformer beat's even bin, 40-bit block
   * integrators over n_fft beats; 0 leaves it out, more than n_beams / 2
   * (1 for one beam) is clamped. Its telemetry is in rd_stats. */
  uint32_t engine_pairs;
} rd_config;

/* One CFAR event as the chain emits it. w[] holds the 176-bit event of
 * model/cpp/cfar/cfar_model.hpp:75-84, little endian, bits 176..191 zero:
 * kind[1:0] bin[17:2] frame_id[33:18] ref_cnt[40:34] alpha[56:41]
 * det[72:57] sup[88:73] cut_power[128:89] noise_sum[175:129]. */
typedef struct rd_event {
  uint64_t w[3];
  uint32_t frame;   /* stream frame index the event belongs to */
  uint16_t beam;    /* beam (CFAR instance) that produced it */
  uint8_t kind;     /* RD_EV_* (also bits 1:0 of w[0]) */
  uint8_t framing;  /* bit0 sof, bit1 eof (cfar_model.hpp:190-192) */
} rd_event;

/* Header of one closed covariance window (covar_model.hpp:171-184). The
 * accumulators of every (bin, pair) of the window are stored separately. */
typedef struct rd_cov_window {
  uint32_t window_id;     /* 16-bit window counter */
  uint32_t sample_count;  /* samples in the window */
  uint32_t end_frame;     /* stream frame that closed the window */
  uint8_t flushed;
  uint8_t truncated;
  uint8_t sat_flags;      /* OR of every integrator step's flags in it */
  uint8_t pad;
} rd_cov_window;

/* Results of one process call. Every pointer may be NULL (that output is
 * skipped); counts are always filled. When a capacity is too small the call
 * fills what fits and returns RD_ETRUNC. */
typedef struct rd_output {
  rd_event* events;       uint64_t cap_events;   uint64_t n_events;
  uint32_t* flits;        uint64_t cap_flits;    uint64_t n_flits;
  /* flit f occupies flit_words u32 words starting at flits[f*flit_words] */
  uint32_t flit_words;
  rd_cov_window* cov_windows; uint32_t cap_cov_windows; uint32_t n_cov_windows;
  /* [cap_cov_windows][n_fft][n_pairs][2] int64 (re, im) */
  int64_t* cov_acc;
  /* optional per-frame taps, [n_frames] outer: */
  rd_cplx16* tap_pfb;      /* [frames][C][N] PFB output, phase order */
  rd_cplx16* tap_spectrum; /* [frames][N][C] natural-bin spectra (history) */
  rd_cplx16* tap_beams;    /* [frames][B][N] beamformer output */
  uint32_t* tap_power;     /* [frames][B][N] power cells (<= 2^31) */
  uint64_t n_frames;       /* frames processed by this call */
} rd_output;

/* Cumulative per-stream statistics. */
typedef struct rd_stats {
  uint64_t frames;
  uint32_t pfb_flags;        /* OR over every PFB output */
  uint64_t pfb_sat_samples;  /* PFB outputs with any flag set */
  uint32_t fft_stage_flags[11]; /* OR per FFT sub-stage (fft_ref.hpp:230) */
  uint32_t bf_flags;
  uint64_t bf_sat_samples;
  uint32_t cov_flags;
  uint64_t cov_sat_steps;
  /* history (history_model.hpp:364-384) */
  uint32_t hist_frames_done, hist_write_beats, hist_reads, hist_collisions;
  uint32_t hist_errors, hist_overwrites, hist_skew;
  /* align (align_model.hpp:209-215) */
  uint32_t align_beats, align_missing, align_dup, align_orphan, align_timeout;
  uint32_t align_fault;
  /* CFAR */
  uint64_t cfar_det, cfar_sup, cfar_frames;
  /* packets */
  uint64_t packets, flits;
  uint32_t next_seq;         /* per-VC packet sequence number (16 bits) */
  /* history depth in frames and the depth changes so far (history_model.hpp:364-365) */
  uint32_t hist_depth, hist_epoch;
  /* the beat-stream covariance engine's telemetry (benchmark_sim_top.sv:1197-1199):
   * pair 0's last closed window id and sample count, any pair's sticky saturation */
  uint32_t engine_window, engine_samples, engine_sat;
} rd_stats;

typedef struct rd_chain rd_chain;

/* ---- configuration ------------------------------------------------------ */
void rd_config_default(rd_config* cfg);
rd_status rd_config_validate(const rd_config* cfg);
uint32_t rd_flit_words(uint32_t packet_w);           /* ceil((W+5)/32) */
uint32_t rd_detection_flits(uint32_t packet_w);       /* 1 + ceil(176/W) */
uint32_t rd_cov_pairs(const rd_config* cfg);          /* pairs in the table */

/* ---- chain lifecycle (replaces composing model/cpp block objects by hand:
 *      pfb::PfbModel pfb_model.hpp:207, fft::Engine fft_ref.hpp:246,
 *      hist::Model history_model.hpp:191, algn::Model align_model.hpp:207,
 *      bf::BeamformerModel beamformer_model.hpp:255, covar::Integrator
 *      covar_model.hpp:186, cfar::run_frame cfar_model.hpp:295) ---------- */
rd_status rd_chain_create(const rd_config* cfg, rd_chain** out);
void rd_chain_destroy(rd_chain* ch);

/* PFB coefficients, n_fft*taps, phase-major tap-minor (pfb_model.hpp:108).
 * Takes effect at the next frame; the delay lines are kept, as
 * pfb::PfbModel::swap_coeff does (pfb_model.hpp:229-233). */
rd_status rd_chain_set_coeff(rd_chain* ch, const rd_cplx16* coeff);
/* Beam weights, n_beams*n_chan, beam-major (beamformer_model.hpp:137-139).
 * Takes effect at the next frame (BeamformerModel::swap_weights :276). */
rd_status rd_chain_set_weights(rd_chain* ch, const rd_cplx16* w);
/* Covariance pair table (covar_model.hpp:306-309): x[i], y[i] index the
 * source vector. Only legal before the first frame. */
rd_status rd_chain_set_pairs(rd_chain* ch, const uint32_t* x, const uint32_t* y,
                             uint32_t n_pairs);

/* Process n samples per channel (a multiple of n_fft) from HOST memory laid
 * out [n_chan][ld]. Copies in, runs, copies the results out. Synchronous.
 * The copies overlap the kernels chunk by chunk: each chunk's input is copied
 * while the previous chunk computes, and results into page-locked host
 * buffers (cudaHostAlloc, cudaHostRegister) are copied as each chunk
 * finishes; into pageable buffers they are copied at the end. A call of at
 * least two launches' worth of frames starts with a quarter-size chunk,
 * grows the next chunks by half up to the launch size and ends with a
 * quarter-size chunk, so that little of the first copy and of the last
 * results stays uncovered. */
rd_status rd_chain_process(rd_chain* ch, const rd_cplx16* adc, uint64_t n,
                           uint64_t ld, rd_output* out);

/* The same on DEVICE memory, asynchronous on `stream` (a cudaStream_t, NULL
 * for the legacy default stream). Results stay on the device until
 * rd_chain_fetch(). */
rd_status rd_chain_process_device(rd_chain* ch, const rd_cplx16* adc_dev,
                                  uint64_t n, uint64_t ld, void* stream);
/* Copies the results of the last rd_chain_process_device to the host. */
rd_status rd_chain_fetch(rd_chain* ch, rd_output* out);
/* Number of kernels the last process call launched. */
uint64_t rd_chain_last_launches(const rd_chain* ch);

/* Stage timing: when enabled, every kernel the chain launches is bracketed by
 * CUDA events on the chain's stream. rd_chain_kernel_times() waits for the
 * stream and returns, per kernel, the launches and the summed device time
 * since the last call (then resets). */
typedef struct rd_kernel_time {
  char name[32];
  uint64_t launches;
  double total_ms;
} rd_kernel_time;
rd_status rd_chain_set_profiling(rd_chain* ch, int on);
rd_status rd_chain_kernel_times(rd_chain* ch, rd_kernel_time* out, uint32_t cap,
                                uint32_t* n);

/* Emits every open covariance window as a flushed, truncated result
 * (covar::Integrator::step with flush=1, covar_model.hpp:226-249). */
rd_status rd_chain_flush_cov(rd_chain* ch, rd_output* out);

rd_status rd_chain_stats(const rd_chain* ch, rd_stats* st);

/* Returns the chain to its just-created state - delay lines, history,
 * covariance windows, counters and packet sequence - keeping the
 * coefficients, weights and pair table (no reference counterpart: the
 * models are reset by constructing new ones). The device part is enqueued
 * on `stream` (NULL: the legacy stream), so it can be captured in a graph. */
rd_status rd_chain_reset(rd_chain* ch, void* stream);

/* hist::Model::request_depth (history_model.hpp:260-266, 435-451): the
 * history keeps `frames` frames from now on (clamped to 1..hist_frames). The
 * change lands at once - a call boundary is always a safe boundary, no
 * antenna being mid-frame - and discards the history: the depth epoch
 * advances, the frame count and slots restart, so reads report no data until
 * new frames arrive. Counters are kept. */
rd_status rd_chain_set_history_depth(rd_chain* ch, uint32_t frames);

/* Checkpoint and resume of a stream (no reference counterpart): the state a
 * call leaves for the next - PFB delay line, the last hist_frames frames of
 * the history ring, the covariance accumulators and window counters, the
 * device and host counters and the packet sequence - as one byte blob.
 * rd_chain_state_size gives its size (0 for NULL). rd_chain_save_state
 * waits for the chain's work, then writes it (RD_EINVAL when cap is short).
 * rd_chain_load_state restores it into a chain created with the same
 * rd_config and pair count, and given the same coefficients and weights; the
 * chain then continues the saved stream bit for bit. RD_EINVAL for a blob of
 * another configuration or a damaged one. Host memory, synchronous. */
uint64_t rd_chain_state_size(const rd_chain* ch);
rd_status rd_chain_save_state(rd_chain* ch, void* buf, uint64_t cap);
rd_status rd_chain_load_state(rd_chain* ch, const void* buf, uint64_t len);

/* Frames per kernel launch, 1..max_frames (default max_frames). Results do
 * not depend on it; the batch autotuner varies it. Longer launches fill more
 * waves of every kernel and pay fewer launch gaps, at the cost of device
 * memory (the spectrum ring and the CFAR buffers grow with it). */
rd_status rd_chain_set_launch_frames(rd_chain* ch, uint32_t frames);

/* Device bytes a chain of this configuration holds, with the output
 * buffers of calls of `frames_per_call` frames (admission by HBM budget). */
uint64_t rd_chain_footprint(const rd_config* cfg, uint64_t frames_per_call);

/* Range-Doppler map: for every (channel, bin), the slow-time transform of
 * that bin over the newest n_frames frames of the history ring (the map
 * model/python/range_doppler.py:254-266 computes in floating point; here the
 * chain's own fixed-point R2^2 transform, fft::transform of
 * fft_ref.hpp:409-412 with spc 1, natural output order and the given scaling
 * schedule). out: [n_chan][n_fft][n_frames], Doppler bin k of channel c, range
 * bin r at (c * n_fft + r) * n_frames + k (no fftshift); stage_flags:
 * [n_chan * n_fft][log2 n_frames] or NULL. n_frames: a power of two in 8..1024,
 * at most the frames processed and the frames the ring holds
 * (max_frames + hist_frames). No counterpart in the C++ model. */
rd_status rd_chain_doppler(rd_chain* ch, uint32_t n_frames, uint32_t scale_sched,
                           rd_cplx16* out, uint8_t* stage_flags);

/* hist::Model::read (history_model.hpp:283-337): the antenna vector of
 * natural bin `bin`, `frame_off` frames back from the newest complete one. */
rd_status rd_chain_read_history(rd_chain* ch, uint32_t bin, uint32_t frame_off,
                                rd_cplx16* vec, uint32_t* frame_id,
                                uint32_t* flags);

/* ---- batching: many independent scenarios in one CUDA graph ------------
 * No counterpart in the reference (its chain is one RTL instance). Each
 * scenario is a chain; a run resets every chain and processes one input per
 * scenario, the scenarios spread largest-first over `n_streams` concurrent
 * streams, all of it captured once into a CUDA graph and replayed. */
/* Concurrency across the batch's streams (and the server's) needs the
 * device's hardware work queues: set CUDA_DEVICE_MAX_CONNECTIONS=32 in the
 * environment before the process creates its CUDA context (the default 8
 * makes streams share queues and wait on one another's launches). */
typedef struct rd_batch rd_batch;
typedef struct {
  uint32_t n_streams;          /* concurrent streams (0: autotune) */
  uint32_t launch_frames;      /* frames per launch of a 1024-point FFT: an N-point
                                  scenario takes launch_frames x 1024 / N (the same
                                  samples per launch), capped by its max_frames
                                  (0: autotune) */
  int use_graph;               /* 1: capture once, replay; 0: launch eagerly */
} rd_batch_options;
rd_status rd_batch_create(uint32_t n, const rd_config* cfgs, const rd_cplx16* const* coeff,
                          const rd_cplx16* const* weights, const rd_batch_options* opt,
                          rd_batch** out);
void rd_batch_destroy(rd_batch* b);
/* adc_dev[i]: device samples of scenario i, [C][n_samples[i]]. Ordered after
 * the work already on `stream` and before the work enqueued on it later. */
rd_status rd_batch_run(rd_batch* b, const rd_cplx16* const* adc_dev, const uint64_t* n_samples,
                       void* stream);
/* The scenarios one after another on one stream, eagerly: the baseline the
 * batched run is compared with. */
rd_status rd_batch_run_sequential(rd_batch* b, const rd_cplx16* const* adc_dev,
                                  const uint64_t* n_samples, void* stream);
rd_status rd_batch_fetch(rd_batch* b, uint32_t i, rd_output* out);
/* Results written to host memory by every run itself, each scenario's as soon
 * as its launches end (overlapping the other scenarios' work): outs[i] names
 * scenario i's page-locked host buffers - events (required) and flits mapped
 * into the device's address space (cudaHostAlloc, or cudaHostRegister with
 * cudaHostRegisterMapped), cov_acc page-locked - and their capacities. The
 * pointers are kept; NULL stops the export. RD_EINVAL for memory the device
 * cannot reach. A run then needs no rd_batch_fetch: once its stream has
 * completed, rd_batch_results fills out's counts and window headers (and
 * returns RD_ETRUNC or RD_ETIMEOUT as rd_batch_fetch would) without reading
 * the device. */
rd_status rd_batch_set_outputs(rd_batch* b, const rd_output* outs);
rd_status rd_batch_results(rd_batch* b, uint32_t i, rd_output* out);
/* Autotuner: times every (n_streams, launch_frames) candidate on these
 * inputs (graph replays, median of `reps`), keeps the fastest and reports
 * it. */
rd_status rd_batch_tune(rd_batch* b, const rd_cplx16* const* adc_dev, const uint64_t* n_samples,
                        uint32_t reps, rd_batch_options* chosen, double* best_ms);
/* rd_batch_tune with an on-disk cache: when the text file `cache_path` holds
 * a choice for these scenarios (the device, this library, every scenario's
 * rd_config and sample count) it is applied without timing anything
 * (*hit = 1, *best_ms the time recorded with it); otherwise the batch is
 * tuned and the choice appended to the file (created if missing; a file that
 * cannot be written is not an error). */
rd_status rd_batch_tune_cached(rd_batch* b, const rd_cplx16* const* adc_dev,
                               const uint64_t* n_samples, uint32_t reps, const char* cache_path,
                               rd_batch_options* chosen, double* best_ms, int* hit);
/* The detection packets of the last run, every scenario a source (index i,
 * port cfgs[i].dest), merged by rd_egress_merge on `stream` - the stream the
 * run was given, or one ordered after it. Counts are read on the device, so
 * nothing waits for the run. */
rd_status rd_batch_egress(rd_batch* b, uint32_t n_ports, uint32_t* ring_dev, uint64_t cap_per_port,
                          uint32_t* src_of_dev, uint64_t* port_count_dev, void* stream);

/* ---- serving: a request loop over many resident streams -----------------
 * (the submit / poll / stream_open shape of a streaming front end; no
 * counterpart in the reference model). Each stream keeps its chain state -
 * PFB delay lines, history, covariance windows, CFAR/packet counters - on
 * the device between requests. A request is one block of samples of one
 * stream; requests of a stream run in submission order, requests of
 * different streams overlap on the device as request slots free up
 * (continuous batching). Streams are admitted against a device-memory
 * budget (RD_ENOMEM when a stream does not fit). */
typedef struct rd_server rd_server;
typedef struct {
  uint64_t hbm_budget;          /* device bytes for streams + request slots */
  uint32_t max_inflight;        /* requests on the device at once */
  uint32_t queue_cap;           /* requests submitted but not finished */
  uint32_t max_chan;            /* the largest n_chan a stream may have */
  uint64_t max_request_samples; /* per channel */
} rd_server_config;
typedef struct {
  uint64_t req_id;
  uint32_t stream_id;
  int32_t status;               /* rd_status of the request */
  uint64_t n_events;
  uint32_t n_cov_windows;
  double t_submit_us, t_start_us, t_done_us;  /* server clock */
} rd_completion;
typedef struct {
  uint64_t hbm_budget, hbm_used;
  uint32_t streams, inflight, queued;
} rd_server_info;
rd_status rd_server_create(const rd_server_config* cfg, rd_server** out);
void rd_server_destroy(rd_server* s);
/* Admits a stream (RD_ENOMEM when its chain does not fit the budget). Besides
 * the chain's device state it reserves one page-locked host block for the
 * most covariance window sums a request of the stream can close (34 MB for a
 * 64-channel, 1024-bin stream), so that requests read them by DMA without
 * allocating; blocks stay with the server for later requests and streams
 * until rd_server_destroy, at most queue_cap + max_inflight of them (a full
 * pool gives up its smallest block for a larger one). */
rd_status rd_stream_open(rd_server* s, const rd_config* cfg, const rd_cplx16* coeff,
                         const rd_cplx16* weights, uint32_t* stream_id);
rd_status rd_stream_close(rd_server* s, uint32_t stream_id);
/* The stream's covariance pair table, as rd_chain_set_pairs; only before the
 * stream's first request, with the cov_n_pairs it was admitted with. */
rd_status rd_stream_set_pairs(rd_server* s, uint32_t stream_id, const uint32_t* x,
                              const uint32_t* y, uint32_t n_pairs);
/* Copies the request's samples ([C][n], row stride ld) and queues it;
 * RD_EAGAIN when queue_cap requests are outstanding. */
rd_status rd_server_submit(rd_server* s, uint32_t stream_id, const rd_cplx16* adc, uint64_t n,
                           uint64_t ld, uint64_t* req_id);
/* Starts queued requests on free slots and collects finished ones (up to
 * cap completions). */
rd_status rd_server_poll(rd_server* s, rd_completion* out, uint32_t cap, uint32_t* n_out);
/* The outputs of a completed request (events, flits, covariance windows),
 * handed over once. */
rd_status rd_server_take(rd_server* s, uint64_t req_id, rd_output* out);
rd_status rd_server_info_get(rd_server* s, rd_server_info* info);
/* A native request loop for measurement: request k (stream stream_ids[k],
 * samples adc[k], n[k] per channel) arrives at arrival_us[k] after the
 * start; each is submitted when it arrives (or as soon as the queue has
 * room) and polled to completion. latency_us[k] = completion - arrival.
 * Returns RD_ETIMEOUT when requests are outstanding and none completes for
 * 30 s of wall-clock time. */
rd_status rd_server_run_trace(rd_server* s, uint64_t n_req, const uint32_t* stream_ids,
                              const double* arrival_us, const rd_cplx16* const* adc,
                              const uint64_t* n, double* latency_us, double* makespan_us);

/* ---- packet fabric egress --------------------------------------------------
 * Many streams' detection packets merged into per-port DMA rings. Each port
 * is fed by one round-robin arbiter over the sources that target it, the
 * fabric's arbiter (rtl/packet/pkt_rr_arb.sv: the lowest requesting index at
 * or after the pointer, the pointer one past the grant): with every source's
 * packets queued that is cyclic source order, skipping sources that have run
 * dry, and each source's packets keep their order - the per-(src, VC, dest)
 * ordering the fabric's scoreboard checks (packet_model.hpp:475-500). No
 * counterpart in the C++ model, which checks a fabric rather than being one. */
#define RD_EGRESS_MAX_SRC 512u
typedef struct rd_egress_source {
  const uint32_t* flits;      /* device: packets of rd_detection_flits(packet_w)
                                 flits of rd_flit_words(packet_w) words each */
  const uint64_t* count_dev;  /* device: packet count, read when the merge runs; or NULL */
  uint64_t n_packets;         /* the packet count (count_dev NULL), else its upper bound */
  uint32_t dest;              /* egress port, < n_ports */
  uint32_t reserved;
} rd_egress_source;

/* Asynchronous on `stream`: ring_dev [n_ports][cap_per_port] packets,
 * src_of_dev [n_ports][cap_per_port] source indices (or NULL), and
 * port_count_dev [n_ports] the packets each port was given - more than
 * cap_per_port means that port's ring dropped the rest. */
rd_status rd_egress_merge(const rd_egress_source* src, uint32_t n_src, uint32_t packet_w,
                          uint32_t n_ports, uint32_t* ring_dev, uint64_t cap_per_port,
                          uint32_t* src_of_dev, uint64_t* port_count_dev, void* stream);

/* packet_model::route_path (packet_model.hpp:283-309): the wires a packet
 * from src to dest occupies in a stages-stage radix-radix butterfly, path[0]
 * = src, stages + 1 entries; the last equals dest (route determinism). */
rd_status rd_route_path(uint32_t src, uint32_t dest, uint32_t radix, uint32_t stages,
                        uint32_t* path);

/* ---- per-block entry points (the model/cpp call surface, on the GPU) ---- */

/* pfb::PfbModel::step over `beats` beats (pfb_model.hpp:242-251).
 * state: [taps-1][phases] delay line, state[k] = x[n-1-k]; updated in place.
 * flags_out: [beats][phases] bytes, (f_re << 2) | f_im, may be NULL. */
rd_status rd_pfb_run(uint32_t phases, uint32_t taps, const rd_cplx16* coeff,
                     rd_cplx16* state, const rd_cplx16* in, uint32_t beats,
                     rd_cplx16* out, uint8_t* flags_out);

/* fft::transform (fft_ref.hpp:409-412) on `frames` independent frames.
 * out: beat order, bins: natural order (either may be NULL),
 * stage_flags: [frames][log2 n_fft] packed flags (may be NULL). */
rd_status rd_fft_run(uint32_t n_fft, uint32_t spc, uint32_t scale_sched,
                     int reorder, const rd_cplx16* in, uint32_t frames,
                     rd_cplx16* out, rd_cplx16* bins, uint8_t* stage_flags);

/* bf::dot / BeamformerModel::step (beamformer_model.hpp:162-179,283-303) for
 * n_vec antenna vectors x[n_vec][n_ant] -> y[n_vec][n_beams].
 * acc: [n_vec][n_beams][2] exact accumulators (may be NULL);
 * flags: [n_vec][n_beams] bytes (f_re << 2) | f_im (may be NULL).
 * form: RD_FORM_*; the tensor forms need n_ant <= RD_TC_MAX_CHAN. */
rd_status rd_bf_run(uint32_t n_ant, uint32_t n_beams, const rd_cplx16* w,
                    const rd_cplx16* x, uint64_t n_vec, rd_cplx16* y,
                    int64_t* acc, uint8_t* flags, uint32_t form);

/* covar::power and covar::cross_power (covar_model.hpp:99-151) elementwise:
 * power[i] = |x[i]|^2, cross[i] = x[i] * conj(y[i]) as (re, im) int64. */
rd_status rd_power_run(const rd_cplx16* x, uint64_t n, int64_t* power);
rd_status rd_cross_power_run(const rd_cplx16* x, const rd_cplx16* y, uint64_t n,
                             int64_t* cross);

/* cfar::run_frame (cfar_model.hpp:295-340) on `frames` frames of n cells
 * each, 1 <= n <= 1024 (raw signed power, clamped as clamp_cell does). Events of frame i
 * carry frame_ids[i]; beam field = frame index i. */
rd_status rd_cfar_run(const int64_t* cells, uint32_t n, uint32_t frames,
                      const rd_config* cfg, const uint32_t* frame_ids,
                      rd_event* events, uint64_t cap, uint64_t* n_events);

/* The CFAR detector of rd_cfar_run on caller-provided DEVICE buffers, without
 * allocating anything. It has no counterpart in the reference. It is for
 * callers that are handed device memory but may not call cudaMalloc (code
 * inside another framework's memory pool, real-time loops where an
 * allocation would synchronise the device, processes whose allocator is
 * locked after start-up). Its scratch is a static device array of about
 * 1.6 MB that every GPU loading the library holds until exit, shared by every
 * call on a device: at most RD_STATIC_CFAR_MAX_FRAMES frames of at most
 * RD_STATIC_CFAR_MAX_CELLS cells (larger sizes return RD_EINVAL); calls whose
 * work overlaps on the GPU race on it. The first call on each device looks up
 * the scratch address and should come before any stream capture. cells,
 * frame_ids, events and n_events (one uint64) are device pointers; the call
 * is asynchronous on `stream` (a cudaStream_t, NULL = legacy stream).
 * Because nothing waits for the device, an overflow is not reported as
 * RD_ETRUNC: *n_events receives the full event count, only the first `cap`
 * events are written, and the caller compares *n_events with cap. */
#define RD_STATIC_CFAR_MAX_FRAMES 4096u
#define RD_STATIC_CFAR_MAX_CELLS 1024u
rd_status rd_cfar_run_static(const int64_t* cells, uint32_t n, uint32_t frames,
                             const rd_config* cfg, const uint32_t* frame_ids,
                             rd_event* events, uint64_t cap, uint64_t* n_events,
                             void* stream);

/* Detection packet flits for n events (packet_model.hpp:122-260 and the DMA
 * tap of rtl/top/benchmark_sim_top.sv:1818-1936): header flit then payload
 * flits LS word first; seq = (seq0 + i) mod 2^16. */
rd_status rd_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w,
                       uint32_t src_id, uint32_t dest, uint32_t vc,
                       uint32_t seq0, uint32_t* flits);

/* fxp primitives (model/cpp/fxp/fxp_ops.hpp:109-177) evaluated on the GPU:
 * op codes RD_OP_*; a, b, y int64; sh, w unsigned; flags packed. */
enum {
  RD_OP_SAT = 0, RD_OP_TRUNC, RD_OP_ROUND_EVEN, RD_OP_ROUND_HALF_UP,
  RD_OP_ROUND, RD_OP_ROUND_SAT, RD_OP_ADD_SAT, RD_OP_SUB_SAT, RD_OP_NEG_SAT,
  RD_OP_MUL_Q15, RD_OP_MUL_Q15_RS, RD_OP_CMUL_RE, RD_OP_CMUL_IM,
  RD_OP_ACC_W, RD_OP_GROWTH_BITS
};
rd_status rd_fxp_apply(const uint32_t* op, const int64_t* a, const int64_t* b,
                       const uint32_t* sh, const uint32_t* w, uint64_t n,
                       int64_t* y, uint8_t* flags);

/* ---- diagnostics ---------------------------------------------------------- */
const char* rd_last_error(void);
/* 1 when a usable sm_100+ device is present. */
int rd_device_ok(void);
const char* rd_version(void);

#ifdef __cplusplus
}
#endif

#endif /* RD_CHAIN_H_ */
