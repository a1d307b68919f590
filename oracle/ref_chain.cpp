// ref_chain.cpp - composition driver over the reference's own model headers.
//
// TEST INFRASTRUCTURE ONLY: this file is the "real reference" leg of the
// oracle. It is compiled with -I<reference>/model/cpp and calls the
// reference's block models unchanged, composing them in the order
// rtl/top/benchmark_sim_top.sv wires them (the model has no chained entry
// point of its own; sim/verilator/harness/pipeline_tb.h:15-20 says the chain
// is never checked against a model). The result is the bit-exact expected
// output of the chain. It implements oracle/orc.h and builds into
// oracle/_ref/liborc_ref.so; nothing outside tests/ loads it.
//
// Orderings the RTL leaves to arbitration timing are fixed here, and the CUDA
// product follows the same choices:
//   * align reads frame_off 0 (the newest complete frame) after every frame,
//     the value every pipeline test programs (sim/verilator/harness/
//     pipeline_tb.cpp:182);
//   * CFAR frame_id is the stream frame index mod 2^16 (the RTL takes the
//     input seq at SOF, rtl/cfar/cfar_core.sv:477-481);
//   * events are emitted frame by frame, beam 0 first, each beam's events in
//     run_frame order (the RTL merges beams with pkt_rr_arb, :1600-1611);
//   * one packet per event on the DMA tap (:1716-1960): dest 0, type
//     DETECTION, vc 0, src 0, len = detection_flits, per-VC seq counter.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "align/align_model.hpp"
#include "beamformer/beamformer_model.hpp"
#include "cfar/cfar_model.hpp"
#include "covariance/covar_model.hpp"
#include "fft/fft_ref.hpp"
#include "fxp/fxp.hpp"
#include "fxp/fxp_ops.hpp"
#include "history/history_model.hpp"
#include "packet/packet_model.hpp"
#include "pfb/pfb_model.hpp"

#include "orc.h"

namespace {

using fxp::Complex;

Complex cx(rd_cplx16 p) { return Complex::from_packed(p); }

unsigned pack_flags(fxp::Flags f) { return f.packed(); }

// 176-bit event, cfar_model.hpp:75-84 field offsets, masked to field widths.
void set_bits(uint64_t* w, unsigned lsb, unsigned n, uint64_t v) {
  for (unsigned i = 0; i < n; ++i) {
    const unsigned b = lsb + i;
    if ((v >> i) & 1ULL) w[b / 64] |= (1ULL << (b % 64));
  }
}

rd_event pack_event(const cfar::Event& e, uint32_t frame, uint16_t beam) {
  rd_event r;
  std::memset(&r, 0, sizeof(r));
  set_bits(r.w, cfar::kEvKindLsb, cfar::kEvKindW, e.kind);
  set_bits(r.w, cfar::kEvBinLsb, cfar::kBinW, e.bin);
  set_bits(r.w, cfar::kEvFrameIdLsb, cfar::kFrameIdW, e.frame_id);
  set_bits(r.w, cfar::kEvRefCntLsb, cfar::kTotRefW, e.ref_count);
  set_bits(r.w, cfar::kEvAlphaLsb, cfar::kAlphaW, e.alpha);
  set_bits(r.w, cfar::kEvDetLsb, cfar::kCntW, e.det_count);
  set_bits(r.w, cfar::kEvSupLsb, cfar::kCntW, e.sup_count);
  set_bits(r.w, cfar::kEvCellLsb, cfar::kPowerW, e.cut_power);
  set_bits(r.w, cfar::kEvSumLsb, cfar::kSumW, e.noise_sum);
  r.frame = frame;
  r.beam = beam;
  r.kind = static_cast<uint8_t>(e.kind);
  r.framing = static_cast<uint8_t>((e.sof ? 1 : 0) | (e.eof ? 2 : 0));
  return r;
}

uint64_t event_bit_slice(const rd_event& e, unsigned lsb, unsigned n) {
  uint64_t v = 0;
  for (unsigned i = 0; i < n; ++i) {
    const unsigned b = lsb + i;
    if (b >= 192) break;
    if ((e.w[b / 64] >> (b % 64)) & 1ULL) v |= (1ULL << i);
  }
  return v;
}

// One detection packet through packet_model::hdr_pack / make_flit.
void packet_flits(const rd_event& e, unsigned pw, unsigned src, unsigned dest,
                  unsigned vc, unsigned seq, uint32_t* out) {
  namespace pm = packet_model;
  const unsigned nfl = pm::detection_flits(pw);
  const unsigned words = (pw + pm::kFlitCtrlW + 31) / 32;
  pm::Header h;
  h.dest = dest;
  h.src = src;
  h.vc = vc;
  h.ptype = pm::kTypeDetection;
  h.length = nfl;
  h.seq = seq & 0xFFFFu;
  const pm::Flit hf = pm::make_flit(pw, vc, true, nfl == 1, {pm::hdr_pack(h)});
  for (unsigned k = 0; k < words; ++k) out[k] = hf.w[k];
  for (unsigned f = 1; f < nfl; ++f) {
    std::vector<uint64_t> data;
    for (unsigned k = 0; k * 64 < pw; ++k) {
      const unsigned lo = (f - 1) * pw + k * 64;
      const unsigned n = (pw - k * 64 >= 64) ? 64 : (pw - k * 64);
      data.push_back(event_bit_slice(e, lo, n));
    }
    const pm::Flit pf = pm::make_flit(pw, vc, false, f + 1 == nfl, data);
    for (unsigned k = 0; k < words; ++k) out[f * words + k] = pf.w[k];
  }
}

}  // namespace

struct orc_chain {
  rd_config cfg;
  std::vector<pfb::PfbModel> pfb;
  fft::Config fcfg;
  hist::Model hist;
  algn::Model align;
  bf::BeamformerModel bfm;
  std::vector<Complex> weights;
  std::vector<uint32_t> px, py;
  std::vector<covar::Integrator> cov_re, cov_im;  // [bin][pair]
  covar::Config ccfg;
  uint64_t frame = 0;
  rd_stats st;
  // the RTL's beat-stream covariance engine as benchmark_sim_top.sv:1124-1200
  // instantiates it (N_SRC = BEAM_PAR = n_beams, pairs (2p, 2p+1) mod n_beams,
  // ACC_W = COVAR_POWER_W = 40, WINDOW_W = 16, CMULT_PIPE_STAGES = MULT_PIPE
  // = 4, window FFT_SIZE beats, block mode, enable all, no flush)
  std::vector<covar::Engine> eng;  // empty, or one engine
  covar::Config ecfg;
  unsigned eng_pairs = 0;

  orc_chain(const rd_config& c, const hist::Config& hc, const algn::Config& ac)
      : cfg(c), hist(hc), align(ac) {
    std::memset(&st, 0, sizeof(st));
  }

  // one clock of the engine; pair 0's registered result becomes the telemetry
  void engine_step(bool valid, const std::vector<Complex>& src) {
    const std::vector<bool> en(eng_pairs, true);
    const std::vector<covar::PairResult> r = eng[0].step(ecfg, en, valid, src, false, false);
    if (r[0].valid) {
      st.engine_window = r[0].re.window_id;
      st.engine_samples = r[0].re.sample_count;
    }
  }
};

extern "C" {

const char* orc_name(void) { return "reference model/cpp headers"; }

void orc_twiddles(uint32_t* out) {
  for (unsigned i = 0; i < fft::kTwN; ++i) out[i] = fft::kTw[i];
}

int orc_chain_create(const rd_config* c, const rd_cplx16* coeff,
                     const rd_cplx16* weights, const uint32_t* pair_x,
                     const uint32_t* pair_y, uint32_t n_pairs,
                     orc_chain** out) {
  hist::Config hc;
  hc.n_ant = c->n_chan;
  hc.fft_size = c->n_fft;
  hc.lanes = c->spc;
  hc.frames_max = c->hist_frames;
  hc.sample_w = 16;
  hc.bit_reversed = false;
  algn::Config ac;
  ac.n_ant = c->n_chan;
  ac.fft_size = c->n_fft;
  ac.lanes = c->spc;
  ac.frames_max = c->hist_frames;
  ac.sample_w = 16;
  ac.bin_par = 2;
  ac.groups = 4;
  if (!hc.valid() || !ac.valid()) return RD_EINVAL;
  orc_chain* ch = new orc_chain(*c, hc, ac);
  ch->st.hist_depth = ch->hist.depth();
  {
    const unsigned most = c->n_beams >= 2 ? c->n_beams / 2u : 1u;
    ch->eng_pairs = std::min(c->engine_pairs, most);
    if (ch->eng_pairs) {
      ch->eng.emplace_back(c->n_beams, ch->eng_pairs, 40u, 16u, 4u);
      for (unsigned p = 0; p < ch->eng_pairs; ++p)
        ch->eng[0].set_table(p, covar::PairEntry{(2u * p) % c->n_beams, (2u * p + 1u) % c->n_beams});
      ch->ecfg.window_len = c->n_fft;
      ch->ecfg.mode = covar::Mode::kBlock;
      ch->eng[0].reset(ch->ecfg);
    }
  }
  const unsigned N = c->n_fft, T = c->taps, C = c->n_chan, B = c->n_beams;
  std::vector<Complex> cf(N * T);
  for (unsigned i = 0; i < N * T; ++i) cf[i] = cx(coeff[i]);
  for (unsigned a = 0; a < C; ++a) ch->pfb.emplace_back(N, T, cf);
  ch->fcfg.n_fft = N;
  ch->fcfg.spc = c->spc;
  ch->fcfg.scale_sched = c->scale_sched;
  ch->fcfg.reorder = true;
  ch->weights.resize(B * C);
  for (unsigned i = 0; i < B * C; ++i) ch->weights[i] = cx(weights[i]);
  ch->bfm = bf::BeamformerModel(C, B, 2, ch->weights);
  if (c->cov_source != RD_COV_OFF) {
    ch->px.assign(pair_x, pair_x + n_pairs);
    ch->py.assign(pair_y, pair_y + n_pairs);
    ch->ccfg.window_len = c->cov_window;
    ch->ccfg.mode = c->cov_mode == RD_COV_EXP ? covar::Mode::kExp : covar::Mode::kBlock;
    ch->ccfg.exp_k = c->cov_exp_k;
    ch->ccfg.enable = true;
    const size_t n_int = static_cast<size_t>(N) * n_pairs;
    for (size_t i = 0; i < n_int; ++i) {
      ch->cov_re.emplace_back(c->cov_acc_w, 16);
      ch->cov_im.emplace_back(c->cov_acc_w, 16);
      ch->cov_re.back().reset(ch->ccfg);
      ch->cov_im.back().reset(ch->ccfg);
    }
  }
  *out = ch;
  return RD_OK;
}

void orc_chain_destroy(orc_chain* ch) { delete ch; }

int orc_chain_set_coeff(orc_chain* ch, const rd_cplx16* coeff) {
  const unsigned n = ch->cfg.n_fft * ch->cfg.taps;
  std::vector<Complex> cf(n);
  for (unsigned i = 0; i < n; ++i) cf[i] = cx(coeff[i]);
  for (auto& p : ch->pfb) p.swap_coeff(cf);
  return RD_OK;
}

int orc_chain_set_weights(orc_chain* ch, const rd_cplx16* w) {
  const unsigned n = ch->cfg.n_beams * ch->cfg.n_chan;
  for (unsigned i = 0; i < n; ++i) ch->weights[i] = cx(w[i]);
  ch->bfm.swap_weights(ch->weights);
  return RD_OK;
}

int orc_chain_process(orc_chain* ch, const rd_cplx16* adc, uint64_t n,
                      uint64_t ld, rd_output* out, int /*threads*/) {
  const rd_config& c = ch->cfg;
  const unsigned N = c.n_fft, C = c.n_chan, B = c.n_beams, spc = c.spc;
  const unsigned M = N / spc;
  if (n % N != 0) return RD_EINVAL;
  const uint64_t frames = n / N;
  const size_t P = ch->px.size();
  const unsigned pw = c.packet_w;
  const unsigned words = rd_flit_words(pw);
  const unsigned nfl = rd_detection_flits(pw);
  bool trunc = false;

  out->n_events = 0;
  out->n_flits = 0;
  out->flit_words = words;
  out->n_cov_windows = 0;
  out->n_frames = frames;

  cfar::Config cc;
  cc.enable = c.cfar_enable != 0;
  cc.mode = c.cfar_mode == RD_CFAR_GO ? cfar::Mode::kGO : cfar::Mode::kCA;
  cc.out_mode = c.cfar_out_mode == RD_CFAR_DENSE ? cfar::OutMode::kDense
                                                 : cfar::OutMode::kEvents;
  cc.guard_lead = c.guard_lead;
  cc.guard_lag = c.guard_lag;
  cc.ref_lead = c.ref_lead;
  cc.ref_lag = c.ref_lag;
  cc.alpha = c.alpha;

  std::vector<Complex> beat(N);
  std::vector<std::vector<uint64_t>> cells(B, std::vector<uint64_t>(N));
  std::vector<Complex> src;

  for (uint64_t fl = 0; fl < frames; ++fl) {
    const uint64_t f = ch->frame;
    // 1-3: PFB, FFT, history write, per antenna (benchmark_sim_top.sv:553-760)
    for (unsigned a = 0; a < C; ++a) {
      const rd_cplx16* x = adc + a * ld + fl * N;
      for (unsigned p = 0; p < N; ++p) beat[p] = cx(x[p]);
      const pfb::BeatResult pr = ch->pfb[a].step(beat);
      for (unsigned p = 0; p < N; ++p) {
        const unsigned fb = pack_flags(pr.flags_re[p]) | pack_flags(pr.flags_im[p]);
        ch->st.pfb_flags |= fb;
        if (fb) ch->st.pfb_sat_samples++;
        if (out->tap_pfb)
          out->tap_pfb[(fl * C + a) * N + p] = pr.y[p].packed();
      }
      const fft::Result fr = fft::transform(ch->fcfg, pr.y);
      for (size_t s = 0; s < fr.stage_flags.size(); ++s)
        ch->st.fft_stage_flags[s] |= pack_flags(fr.stage_flags[s]);
      for (unsigned j = 0; j < M; ++j) {
        std::vector<Complex> lanes(spc);
        for (unsigned q = 0; q < spc; ++q) lanes[q] = fr.out[j * spc + q];
        ch->hist.write_beat(a, lanes, j == 0, j == M - 1);
      }
    }
    // 4-7: align (frame_off 0), beamform, power, covariance
    for (unsigned g = 0; g < N / 2; ++g) {
      ch->align.open(g, 0, false);
      for (unsigned l = 0; l < 2; ++l) {
        const hist::Response r = ch->hist.read(2 * g + l, 0);
        algn::Word w;
        w.vec = r.vec;
        w.bin = r.bin;
        w.frame_off = r.frame_off;
        w.frame_id = r.frame_id;
        w.flags = r.flags;
        ch->align.deliver(w);
      }
      const algn::Beat ab = ch->align.retire(false);
      std::vector<std::vector<Complex>> bfin(2, std::vector<Complex>(C));
      for (unsigned l = 0; l < 2; ++l)
        for (unsigned a = 0; a < C; ++a) bfin[l][a] = ab.data[l * C + a];
      const bf::BeamBeat bb = ch->bfm.step(bfin);
      if (ch->eng_pairs) {  // the beat's bin_par 0 beams into the engine
        std::vector<Complex> esrc(B);
        for (unsigned b = 0; b < B; ++b) esrc[b] = bb.y[b][0];
        ch->engine_step(true, esrc);
      }
      for (unsigned l = 0; l < 2; ++l) {
        const unsigned bin = 2 * g + l;
        if (out->tap_spectrum)
          for (unsigned a = 0; a < C; ++a)
            out->tap_spectrum[(fl * N + bin) * C + a] = bfin[l][a].packed();
        for (unsigned b = 0; b < B; ++b) {
          const unsigned fb = pack_flags(bb.f_re[b][l]) | pack_flags(bb.f_im[b][l]);
          ch->st.bf_flags |= fb;
          if (fb) ch->st.bf_sat_samples++;
          const fxp::wide_t pwr = covar::power(bb.y[b][l]);
          cells[b][bin] = cfar::clamp_cell(pwr);
          if (out->tap_beams)
            out->tap_beams[(fl * B + b) * N + bin] = bb.y[b][l].packed();
          if (out->tap_power)
            out->tap_power[(fl * B + b) * N + bin] = static_cast<uint32_t>(pwr);
        }
        if (c.cov_source != RD_COV_OFF) {
          src.clear();
          if (c.cov_source == RD_COV_CHANNEL) {
            src = bfin[l];
          } else {
            for (unsigned b = 0; b < B; ++b) src.push_back(bb.y[b][l]);
          }
          for (size_t p = 0; p < P; ++p) {
            const covar::Cross xp = covar::cross_power(src[ch->px[p]], src[ch->py[p]]);
            covar::Result rr, ri;
            const size_t k = static_cast<size_t>(bin) * P + p;
            const bool er = ch->cov_re[k].step(ch->ccfg, true, xp.re, false, false, &rr);
            const bool ei = ch->cov_im[k].step(ch->ccfg, true, xp.im, false, false, &ri);
            if (er != ei) return RD_EDEVICE;  // the two halves must emit together
            if (er) {
              // Integrators run in lockstep: (bin 0, pair 0) opens the record.
              const uint32_t wi = out->n_cov_windows - ((bin == 0 && p == 0) ? 0 : 1);
              if (bin == 0 && p == 0) {
                if (out->n_cov_windows < out->cap_cov_windows && out->cov_windows) {
                  rd_cov_window& h = out->cov_windows[out->n_cov_windows];
                  std::memset(&h, 0, sizeof(h));
                  h.window_id = rr.window_id;
                  h.sample_count = rr.sample_count;
                  h.end_frame = static_cast<uint32_t>(f);
                  h.flushed = rr.flushed;
                  h.truncated = rr.truncated;
                } else {
                  trunc = true;
                }
                out->n_cov_windows++;
              }
              if (wi < out->cap_cov_windows) {
                if (out->cov_acc) {
                  int64_t* acc = out->cov_acc + ((static_cast<size_t>(wi) * N + bin) * P + p) * 2;
                  acc[0] = rr.acc;
                  acc[1] = ri.acc;
                }
                if (out->cov_windows) {
                  const unsigned sf = pack_flags(ch->cov_re[k].sat_flags()) |
                                      pack_flags(ch->cov_im[k].sat_flags());
                  out->cov_windows[wi].sat_flags |= static_cast<uint8_t>(sf);
                }
              }
            }
          }
        }
      }
    }
    // 8: CFAR per beam, in natural bin order (benchmark_sim_top.sv:1517-1560)
    // 9: packets in (frame, beam, event) order (benchmark_sim_top.sv:1716-1960)
    for (unsigned b = 0; b < B; ++b) {
      const std::vector<cfar::Event> ev = cfar::run_frame(
          cells[b], cc, c.max_guard, c.max_ref, static_cast<unsigned>(f & 0xFFFFu));
      ch->st.cfar_frames++;
      for (const cfar::Event& e : ev) {
        if (e.kind == cfar::kEvSummary) {
          ch->st.cfar_det += e.det_count;
          ch->st.cfar_sup += e.sup_count;
        }
        const rd_event re = pack_event(e, static_cast<uint32_t>(f), static_cast<uint16_t>(b));
        if (out->n_events < out->cap_events && out->events) {
          out->events[out->n_events] = re;
        } else if (out->events) {
          trunc = true;
        }
        if (out->flits) {
          if ((out->n_flits + nfl) <= out->cap_flits) {
            packet_flits(re, pw, c.src_id, c.dest, c.vc, ch->st.next_seq,
                         out->flits + out->n_flits * words);
          } else {
            trunc = true;
          }
        }
        out->n_events++;
        out->n_flits += nfl;
        ch->st.packets++;
        ch->st.flits += nfl;
        ch->st.next_seq = (ch->st.next_seq + 1) & 0xFFFFu;
      }
    }
    ch->frame++;
    ch->st.frames++;
  }
  if (ch->eng_pairs) {  // the clock runs on after the call: every product lands
    const std::vector<Complex> idle(B);
    for (int k = 0; k < 4; ++k) ch->engine_step(false, idle);
    bool sat = false;
    for (unsigned p = 0; p < ch->eng_pairs; ++p)
      sat = sat || ch->eng[0].re(p).sat_sticky() || ch->eng[0].im(p).sat_sticky();
    ch->st.engine_sat = sat ? 1u : 0u;
  }
  // counters mirrored from the block models
  ch->st.hist_frames_done = ch->hist.frames_done();
  ch->st.hist_write_beats = ch->hist.write_beat_count();
  ch->st.hist_reads = ch->hist.read_count();
  ch->st.hist_collisions = ch->hist.collision_count();
  ch->st.hist_errors = ch->hist.error_count();
  ch->st.hist_overwrites = ch->hist.overwrite_count();
  ch->st.hist_skew = ch->hist.skew_count();
  ch->st.hist_depth = ch->hist.depth();
  ch->st.hist_epoch = ch->hist.epoch();
  const algn::Model::Counters ac = ch->align.counters();
  ch->st.align_beats = ac.beats;
  ch->st.align_missing = ac.missing;
  ch->st.align_dup = ac.dup;
  ch->st.align_orphan = ac.orphan;
  ch->st.align_timeout = ac.timeout;
  ch->st.align_fault = ch->align.fault();
  uint32_t cf = 0;
  uint64_t cs = 0;
  for (size_t k = 0; k < ch->cov_re.size(); ++k) {
    cf |= pack_flags(ch->cov_re[k].sat_flags()) | pack_flags(ch->cov_im[k].sat_flags());
    cs += ch->cov_re[k].sat_count() + ch->cov_im[k].sat_count();
  }
  ch->st.cov_flags = cf;
  ch->st.cov_sat_steps = cs;
  return trunc ? RD_ETRUNC : RD_OK;
}

int orc_chain_flush_cov(orc_chain* ch, rd_output* out) {
  const unsigned N = ch->cfg.n_fft;
  const size_t P = ch->px.size();
  out->n_cov_windows = 0;
  if (ch->cov_re.empty()) return RD_OK;
  bool opened = false;
  for (unsigned bin = 0; bin < N; ++bin) {
    for (size_t p = 0; p < P; ++p) {
      const size_t k = static_cast<size_t>(bin) * P + p;
      covar::Result rr, ri;
      const bool er = ch->cov_re[k].step(ch->ccfg, false, 0, true, false, &rr);
      const bool ei = ch->cov_im[k].step(ch->ccfg, false, 0, true, false, &ri);
      if (er != ei) return RD_EDEVICE;
      if (!er) continue;
      if (!opened) {
        if (out->cap_cov_windows < 1) return RD_ETRUNC;
        rd_cov_window& h = out->cov_windows[0];
        std::memset(&h, 0, sizeof(h));
        h.window_id = rr.window_id;
        h.sample_count = rr.sample_count;
        h.end_frame = static_cast<uint32_t>(ch->frame);
        h.flushed = rr.flushed;
        h.truncated = rr.truncated;
        out->n_cov_windows = 1;
        opened = true;
      }
      if (out->cov_acc) {
        int64_t* acc = out->cov_acc + (static_cast<size_t>(bin) * P + p) * 2;
        acc[0] = rr.acc;
        acc[1] = ri.acc;
      }
    }
  }
  return RD_OK;
}

int orc_chain_stats(const orc_chain* ch, rd_stats* st) {
  *st = ch->st;
  return RD_OK;
}

int orc_chain_set_history_depth(orc_chain* ch, uint32_t frames) {
  ch->hist.request_depth(frames);  // lands at once: no antenna is mid-frame
  ch->st.hist_frames_done = ch->hist.frames_done();
  ch->st.hist_depth = ch->hist.depth();
  ch->st.hist_epoch = ch->hist.epoch();
  return RD_OK;
}

int orc_chain_read_history(orc_chain* ch, uint32_t bin, uint32_t frame_off,
                           rd_cplx16* vec, uint32_t* frame_id, uint32_t* flags) {
  const hist::Response r = ch->hist.read(bin, frame_off);
  for (size_t a = 0; a < r.vec.size(); ++a) vec[a] = r.vec[a].packed();
  *frame_id = r.frame_id;
  *flags = r.flags;
  ch->st.hist_reads = ch->hist.read_count();
  ch->st.hist_errors = ch->hist.error_count();
  ch->st.hist_collisions = ch->hist.collision_count();
  return RD_OK;
}

// ---- per-block -------------------------------------------------------------

int orc_pfb_run(uint32_t phases, uint32_t taps, const rd_cplx16* coeff,
                rd_cplx16* state, const rd_cplx16* in, uint32_t beats,
                rd_cplx16* out, uint8_t* flags_out) {
  std::vector<Complex> cf(phases * taps);
  for (size_t i = 0; i < cf.size(); ++i) cf[i] = cx(coeff[i]);
  pfb::PfbModel m(phases, taps, cf);
  std::vector<Complex> beat(phases);
  // Load the delay line by replaying it, oldest first: state[k] = x[n-1-k].
  for (int k = static_cast<int>(taps) - 2; k >= 0; --k) {
    for (unsigned p = 0; p < phases; ++p) beat[p] = cx(state[k * phases + p]);
    (void)m.step(beat);
  }
  for (uint32_t t = 0; t < beats; ++t) {
    for (unsigned p = 0; p < phases; ++p) beat[p] = cx(in[t * phases + p]);
    const pfb::BeatResult r = m.step(beat);
    for (unsigned p = 0; p < phases; ++p) {
      out[t * phases + p] = r.y[p].packed();
      if (flags_out)
        flags_out[t * phases + p] = static_cast<uint8_t>(
            (r.flags_re[p].packed() << 2) | r.flags_im[p].packed());
    }
  }
  // New delay line from the concatenated sequence.
  if (taps > 1) {
    std::vector<rd_cplx16> seq;
    for (int k = static_cast<int>(taps) - 2; k >= 0; --k)
      for (unsigned p = 0; p < phases; ++p) seq.push_back(state[k * phases + p]);
    for (uint32_t t = 0; t < beats; ++t)
      for (unsigned p = 0; p < phases; ++p) seq.push_back(in[t * phases + p]);
    const size_t total_beats = seq.size() / phases;
    for (unsigned k = 0; k + 1 < taps; ++k)
      for (unsigned p = 0; p < phases; ++p)
        state[k * phases + p] = seq[(total_beats - 1 - k) * phases + p];
  }
  return RD_OK;
}

int orc_fft_run(uint32_t n_fft, uint32_t spc, uint32_t scale_sched, int reorder,
                const rd_cplx16* in, uint32_t frames, rd_cplx16* out,
                rd_cplx16* bins, uint8_t* stage_flags) {
  fft::Config c;
  c.n_fft = n_fft;
  c.spc = spc;
  c.scale_sched = scale_sched;
  c.reorder = reorder != 0;
  if (!c.valid()) return RD_EINVAL;
  const unsigned stages = fft::total_stages(n_fft);
  std::vector<Complex> x(n_fft);
  for (uint32_t f = 0; f < frames; ++f) {
    for (unsigned i = 0; i < n_fft; ++i) x[i] = cx(in[f * n_fft + i]);
    const fft::Result r = fft::transform(c, x);
    for (unsigned i = 0; i < n_fft; ++i) {
      if (out) out[f * n_fft + i] = r.out[i].packed();
      if (bins) bins[f * n_fft + i] = r.bins[i].packed();
    }
    if (stage_flags)
      for (unsigned s = 0; s < stages; ++s)
        stage_flags[f * stages + s] = static_cast<uint8_t>(r.stage_flags[s].packed());
  }
  return RD_OK;
}

int orc_bf_run(uint32_t n_ant, uint32_t n_beams, const rd_cplx16* w,
               const rd_cplx16* x, uint64_t n_vec, rd_cplx16* y, int64_t* acc,
               uint8_t* flags) {
  std::vector<Complex> wc(n_ant * n_beams), xc(n_ant);
  for (size_t i = 0; i < wc.size(); ++i) wc[i] = cx(w[i]);
  for (uint64_t v = 0; v < n_vec; ++v) {
    for (unsigned a = 0; a < n_ant; ++a) xc[a] = cx(x[v * n_ant + a]);
    for (unsigned b = 0; b < n_beams; ++b) {
      const bf::DotResult d = bf::dot(xc.data(), &wc[bf::weight_index(n_ant, b, 0)], n_ant);
      y[v * n_beams + b] = d.y.packed();
      if (acc) {
        acc[(v * n_beams + b) * 2 + 0] = d.acc_re;
        acc[(v * n_beams + b) * 2 + 1] = d.acc_im;
      }
      if (flags)
        flags[v * n_beams + b] = static_cast<uint8_t>((d.f_re.packed() << 2) | d.f_im.packed());
    }
  }
  return RD_OK;
}

int orc_power_run(const rd_cplx16* x, uint64_t n, int64_t* power) {
  for (uint64_t i = 0; i < n; ++i) power[i] = covar::power(cx(x[i]));
  return RD_OK;
}

int orc_cross_power_run(const rd_cplx16* x, const rd_cplx16* y, uint64_t n,
                        int64_t* cross) {
  for (uint64_t i = 0; i < n; ++i) {
    const covar::Cross a = covar::cross_power_direct(cx(x[i]), cx(y[i]));
    const covar::Cross b = covar::cross_power_swap(cx(x[i]), cx(y[i]));
    if (a != b) return RD_EDEVICE;  // the two wirings must agree
    cross[2 * i] = b.re;
    cross[2 * i + 1] = b.im;
  }
  return RD_OK;
}

int orc_cfar_run(const int64_t* cells, uint32_t n, uint32_t frames,
                 const rd_config* c, const uint32_t* frame_ids,
                 rd_event* events, uint64_t cap, uint64_t* n_events) {
  cfar::Config cc;
  cc.enable = c->cfar_enable != 0;
  cc.mode = c->cfar_mode == RD_CFAR_GO ? cfar::Mode::kGO : cfar::Mode::kCA;
  cc.out_mode = c->cfar_out_mode == RD_CFAR_DENSE ? cfar::OutMode::kDense
                                                  : cfar::OutMode::kEvents;
  cc.guard_lead = c->guard_lead;
  cc.guard_lag = c->guard_lag;
  cc.ref_lead = c->ref_lead;
  cc.ref_lag = c->ref_lag;
  cc.alpha = c->alpha;
  uint64_t k = 0;
  std::vector<uint64_t> bins(n);
  for (uint32_t f = 0; f < frames; ++f) {
    for (uint32_t i = 0; i < n; ++i) bins[i] = cfar::clamp_cell(cells[f * n + i]);
    const std::vector<cfar::Event> ev =
        cfar::run_frame(bins, cc, c->max_guard, c->max_ref, frame_ids[f]);
    for (const cfar::Event& e : ev) {
      if (k < cap) events[k] = pack_event(e, frame_ids[f], static_cast<uint16_t>(f));
      ++k;
    }
  }
  *n_events = k;
  return k > cap ? RD_ETRUNC : RD_OK;
}

int orc_packetize(const rd_event* ev, uint64_t n, uint32_t packet_w,
                  uint32_t src_id, uint32_t dest, uint32_t vc, uint32_t seq0,
                  uint32_t* flits) {
  const unsigned words = rd_flit_words(packet_w);
  const unsigned nfl = rd_detection_flits(packet_w);
  for (uint64_t i = 0; i < n; ++i)
    packet_flits(ev[i], packet_w, src_id, dest, vc,
                 static_cast<unsigned>((seq0 + i) & 0xFFFFu),
                 flits + i * nfl * words);
  return RD_OK;
}

int orc_fxp_apply(const uint32_t* op, const int64_t* a, const int64_t* b,
                  const uint32_t* sh, const uint32_t* w, uint64_t n, int64_t* y,
                  uint8_t* flags) {
  // RD_OP_* order -> fxp::ops opcode (fxp_ops.hpp op table).
  for (uint64_t i = 0; i < n; ++i) {
    unsigned code = 0;
    switch (op[i]) {
      case RD_OP_SAT: code = fxp::ops::kSat; break;
      case RD_OP_TRUNC: code = fxp::ops::kTrunc; break;
      case RD_OP_ROUND_EVEN: code = fxp::ops::kRoundEven; break;
      case RD_OP_ROUND_HALF_UP: code = fxp::ops::kRoundHalfUp; break;
      case RD_OP_ROUND: code = fxp::ops::kRound; break;
      case RD_OP_ROUND_SAT: code = fxp::ops::kRoundSat; break;
      case RD_OP_ADD_SAT: code = fxp::ops::kAddSat; break;
      case RD_OP_SUB_SAT: code = fxp::ops::kSubSat; break;
      case RD_OP_NEG_SAT: code = fxp::ops::kNegSat; break;
      case RD_OP_MUL_Q15: code = fxp::ops::kMulQ15; break;
      case RD_OP_MUL_Q15_RS: code = fxp::ops::kMulQ15Rs; break;
      case RD_OP_CMUL_RE: code = fxp::ops::kCmulRe; break;
      case RD_OP_CMUL_IM: code = fxp::ops::kCmulIm; break;
      case RD_OP_ACC_W: code = fxp::ops::kAccW; break;
      case RD_OP_GROWTH_BITS: code = fxp::ops::kGrowthBits; break;
      default: return RD_EINVAL;
    }
    const fxp::ops::Result r = fxp::ops::apply(code, a[i], b[i], sh[i], w[i]);
    y[i] = r.y;
    flags[i] = static_cast<uint8_t>(r.flags.packed());
  }
  return RD_OK;
}

// The reference's packet_model::Scoreboard over whole packets injected as
// flit rows and flits observed at egress ports (ref leg only; it pins the
// Python restatement of the scoreboard). counts: delivered, lost, duplicated,
// misrouted, corrupted, reordered, framing, parity, unexpected; log: the
// delivery log, one entry per line.
int orc_ref_scoreboard(uint32_t packet_w, uint32_t radix, uint32_t stages,
                       const uint32_t* inj, uint64_t n_inj_flits, const uint32_t* obs_port,
                       const uint32_t* obs, uint64_t n_obs, uint64_t* counts, char* log,
                       uint64_t log_cap) {
  if (packet_w < 64 || packet_w > 512 || packet_w % 32) return RD_EINVAL;
  packet_model::Scoreboard sb(packet_w, radix, stages);
  const unsigned words = rd_flit_words(packet_w);
  auto flit_at = [&](const uint32_t* rows, uint64_t i) {
    packet_model::Flit f;
    f.resize_for(packet_w);
    for (unsigned k = 0; k < words; ++k) f.w[k] = rows[i * words + k];
    return f;
  };
  for (uint64_t i = 0; i < n_inj_flits;) {
    packet_model::Packet p;
    p.hdr = flit_at(inj, i).header();
    const uint64_t n = p.hdr.length ? p.hdr.length : 1;
    if (i + n > n_inj_flits) return RD_EINVAL;
    for (uint64_t k = 1; k < n; ++k) {
      const packet_model::Flit f = flit_at(inj, i + k);
      std::vector<std::uint64_t> d;
      for (unsigned q = 0; q * 64 < packet_w; ++q) d.push_back(f.data64(q));
      p.payload.push_back(d);
    }
    sb.inject(p);
    i += n;
  }
  for (uint64_t i = 0; i < n_obs; ++i) sb.observe(obs_port[i], flit_at(obs, i));
  sb.finish();
  const packet_model::Counts& c = sb.counts();
  const std::size_t v[9] = {c.delivered, c.lost, c.duplicated, c.misrouted, c.corrupted,
                            c.reordered, c.framing, c.parity, c.unexpected};
  for (int k = 0; k < 9; ++k) counts[k] = v[k];
  std::string all;
  for (const std::string& e : sb.log()) all += e + "\n";
  if (log && log_cap) {
    const std::size_t k = std::min<std::size_t>(all.size(), log_cap - 1);
    std::memcpy(log, all.data(), k);
    log[k] = 0;
  }
  return all.size() < log_cap ? RD_OK : RD_ETRUNC;
}

// Shared geometry helpers (also exported by the product library).
uint32_t rd_flit_words(uint32_t packet_w) {
  return (packet_w + packet_model::kFlitCtrlW + 31) / 32;
}
uint32_t rd_detection_flits(uint32_t packet_w) {
  return packet_model::detection_flits(packet_w);
}

}  // extern "C"
