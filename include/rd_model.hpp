// rd_model.hpp - C++ facade with the call surface of the reference model
// (fpga-professional-association/agilex-7-radar-detect, model/cpp), computed
// on the GPU through the C ABI of rd_chain.h.
//
// The namespaces, class names and member signatures are the reference's, inside
// namespace rdgb so both can be included side by side:
//
//   reference (model/cpp)                       this facade
//   ------------------------------------------  -----------------------------
//   pfb::PfbModel(phases, taps, coeff)          rdgb::pfb::PfbModel
//     .step(beat) -> BeatResult  (pfb_model.hpp:207-251)
//   fft::transform(Config, in) -> Result        rdgb::fft::transform
//                                (fft_ref.hpp:199-240, 409-412)
//   bf::dot(x, w, n) -> DotResult               rdgb::bf::dot
//   bf::BeamformerModel(n_ant, n_beams, bin_par, w).step(beat)
//                                (beamformer_model.hpp:145-179, 255-303)
//   covar::power / cross_power                  rdgb::covar::power / cross_power
//                                (covar_model.hpp:99-151)
//   cfar::run_frame(bins, cfg, max_guard, max_ref, frame_id)
//                                (cfar_model.hpp:112-128, 179-217, 295-340)
//   packet_model::make_flit / hdr_pack          rdgb::packet_model::detection_packet
//                                (packet_model.hpp:132-260)
//   (no chained entry point in the reference)   rdgb::Chain (rd_chain_*)
//
// Every call runs CUDA kernels; errors throw std::runtime_error carrying
// rd_last_error(). The per-block classes move one call's data to the device
// and back; batch many beats or frames per call for throughput, or use
// rdgb::Chain, which keeps all stream state resident on the GPU.
#ifndef RD_MODEL_HPP_
#define RD_MODEL_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "rd_chain.h"

namespace rdgb {

inline void check(rd_status s, const char* what) {
  if (s != RD_OK) throw std::runtime_error(std::string(what) + ": " + rd_last_error());
}

namespace fxp {
struct Complex {
  int16_t re = 0;
  int16_t im = 0;
  uint32_t packed() const {
    return (static_cast<uint32_t>(static_cast<uint16_t>(im)) << 16) |
           static_cast<uint16_t>(re);
  }
  static Complex from_packed(uint32_t p) {
    return Complex{static_cast<int16_t>(static_cast<uint16_t>(p & 0xFFFFu)),
                   static_cast<int16_t>(static_cast<uint16_t>(p >> 16))};
  }
  bool operator==(const Complex& o) const { return re == o.re && im == o.im; }
};
struct Flags {
  bool sat_pos = false;
  bool sat_neg = false;
  unsigned packed() const { return (sat_pos ? 2u : 0u) | (sat_neg ? 1u : 0u); }
  static Flags from_packed(unsigned p) { return Flags{(p & 2u) != 0, (p & 1u) != 0}; }
  bool any() const { return sat_pos || sat_neg; }
};
inline std::vector<uint32_t> pack(const std::vector<Complex>& v) {
  std::vector<uint32_t> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = v[i].packed();
  return o;
}
}  // namespace fxp

namespace pfb {
using fxp::Complex;
using fxp::Flags;
struct BeatResult {
  std::vector<Complex> y;
  std::vector<Flags> flags_re, flags_im;
};
class PfbModel {
 public:
  PfbModel(unsigned phases, unsigned taps, const std::vector<Complex>& coeff)
      : phases_(phases), taps_(taps), coeff_(fxp::pack(coeff)),
        state_(static_cast<size_t>(taps > 1 ? taps - 1 : 0) * phases, 0u) {}
  // keeps the delay line (pfb_model.hpp:229-233)
  void swap_coeff(const std::vector<Complex>& coeff) { coeff_ = fxp::pack(coeff); }
  void reset() { std::fill(state_.begin(), state_.end(), 0u); }
  BeatResult step(const std::vector<Complex>& beat) { return step_many(beat, 1).front(); }
  // `beats` consecutive beats of `phases` samples each, one GPU call.
  std::vector<BeatResult> step_many(const std::vector<Complex>& x, unsigned beats) {
    const std::vector<uint32_t> in = fxp::pack(x);
    std::vector<uint32_t> out(in.size());
    std::vector<uint8_t> fl(in.size());
    check(rd_pfb_run(phases_, taps_, coeff_.data(), state_.data(), in.data(), beats, out.data(),
                     fl.data()),
          "rd_pfb_run");
    std::vector<BeatResult> r(beats);
    for (unsigned t = 0; t < beats; ++t) {
      r[t].y.resize(phases_);
      r[t].flags_re.resize(phases_);
      r[t].flags_im.resize(phases_);
      for (unsigned p = 0; p < phases_; ++p) {
        const size_t i = static_cast<size_t>(t) * phases_ + p;
        r[t].y[p] = Complex::from_packed(out[i]);
        r[t].flags_re[p] = Flags::from_packed(fl[i] >> 2);
        r[t].flags_im[p] = Flags::from_packed(fl[i] & 3u);
      }
    }
    return r;
  }
  unsigned phases() const { return phases_; }
  unsigned taps() const { return taps_; }

 private:
  unsigned phases_, taps_;
  std::vector<uint32_t> coeff_, state_;
};
}  // namespace pfb

namespace fft {
using fxp::Complex;
using fxp::Flags;
struct Config {
  unsigned n_fft = 64;
  unsigned spc = 2;
  unsigned scale_sched = 0xFFFFFFFFu;
  bool reorder = true;
};
struct Result {
  std::vector<Complex> out;        // beat order
  std::vector<Flags> stage_flags;  // one per sub-stage
  std::vector<Complex> bins;       // natural order
};
inline std::vector<Result> transform_many(const Config& c, const std::vector<Complex>& in,
                                          unsigned frames) {
  const std::vector<uint32_t> x = fxp::pack(in);
  std::vector<uint32_t> out(x.size()), bins(x.size());
  unsigned st = 0;
  while ((1u << st) < c.n_fft) ++st;
  std::vector<uint8_t> sf(static_cast<size_t>(frames) * st);
  check(rd_fft_run(c.n_fft, c.spc, c.scale_sched, c.reorder ? 1 : 0, x.data(), frames,
                   out.data(), bins.data(), sf.data()),
        "rd_fft_run");
  std::vector<Result> r(frames);
  for (unsigned f = 0; f < frames; ++f) {
    for (unsigned i = 0; i < c.n_fft; ++i) {
      r[f].out.push_back(Complex::from_packed(out[static_cast<size_t>(f) * c.n_fft + i]));
      r[f].bins.push_back(Complex::from_packed(bins[static_cast<size_t>(f) * c.n_fft + i]));
    }
    for (unsigned s = 0; s < st; ++s)
      r[f].stage_flags.push_back(Flags::from_packed(sf[static_cast<size_t>(f) * st + s]));
  }
  return r;
}
inline Result transform(const Config& c, const std::vector<Complex>& in) {
  return transform_many(c, in, 1).front();
}
}  // namespace fft

namespace bf {
using fxp::Complex;
using fxp::Flags;
struct DotResult {
  Complex y;
  Flags f_re, f_im;
  int64_t acc_re = 0, acc_im = 0;
};
// Y[v][b] for n_vec antenna vectors x[v][a], weights beam-major w[b][a].
inline std::vector<DotResult> dot_many(const std::vector<Complex>& x,
                                       const std::vector<Complex>& w, unsigned n_ant,
                                       unsigned n_beams,
                                       uint32_t form = RD_FORM_CUDA_CORE) {
  const std::vector<uint32_t> xp = fxp::pack(x), wp = fxp::pack(w);
  const uint64_t nv = xp.size() / n_ant;
  std::vector<uint32_t> y(nv * n_beams);
  std::vector<int64_t> acc(nv * n_beams * 2);
  std::vector<uint8_t> fl(nv * n_beams);
  check(rd_bf_run(n_ant, n_beams, wp.data(), xp.data(), nv, y.data(), acc.data(), fl.data(),
                  form),
        "rd_bf_run");
  std::vector<DotResult> r(nv * n_beams);
  for (size_t i = 0; i < r.size(); ++i) {
    r[i].y = Complex::from_packed(y[i]);
    r[i].f_re = Flags::from_packed(fl[i] >> 2);
    r[i].f_im = Flags::from_packed(fl[i] & 3u);
    r[i].acc_re = acc[2 * i];
    r[i].acc_im = acc[2 * i + 1];
  }
  return r;
}
inline DotResult dot(const Complex* x, const Complex* w, unsigned n_ant) {
  return dot_many(std::vector<Complex>(x, x + n_ant), std::vector<Complex>(w, w + n_ant),
                  n_ant, 1)
      .front();
}
struct BeamBeat {
  std::vector<std::vector<Complex>> y;  // [beam][bin]
};
class BeamformerModel {
 public:
  BeamformerModel(unsigned n_ant, unsigned n_beams, unsigned bin_par, const std::vector<Complex>& w)
      : n_ant_(n_ant), n_beams_(n_beams), bin_par_(bin_par), w_(w) {}
  void swap_weights(const std::vector<Complex>& w) { w_ = w; }
  BeamBeat step(const std::vector<std::vector<Complex>>& beat) const {
    std::vector<Complex> x;
    for (const auto& v : beat) x.insert(x.end(), v.begin(), v.end());
    const std::vector<DotResult> d = dot_many(x, w_, n_ant_, n_beams_);
    BeamBeat r;
    r.y.assign(n_beams_, std::vector<Complex>(bin_par_));
    for (unsigned j = 0; j < bin_par_; ++j)
      for (unsigned b = 0; b < n_beams_; ++b) r.y[b][j] = d[j * n_beams_ + b].y;
    return r;
  }

 private:
  unsigned n_ant_, n_beams_, bin_par_;
  std::vector<Complex> w_;
};
}  // namespace bf

namespace covar {
using fxp::Complex;
struct Cross {
  int64_t re = 0, im = 0;
};
inline std::vector<int64_t> power(const std::vector<Complex>& s) {
  const std::vector<uint32_t> x = fxp::pack(s);
  std::vector<int64_t> p(x.size());
  check(rd_power_run(x.data(), x.size(), p.data()), "rd_power_run");
  return p;
}
inline std::vector<Cross> cross_power(const std::vector<Complex>& x, const std::vector<Complex>& y) {
  const std::vector<uint32_t> a = fxp::pack(x), b = fxp::pack(y);
  std::vector<int64_t> c(2 * a.size());
  check(rd_cross_power_run(a.data(), b.data(), a.size(), c.data()), "rd_cross_power_run");
  std::vector<Cross> r(a.size());
  for (size_t i = 0; i < r.size(); ++i) r[i] = Cross{c[2 * i], c[2 * i + 1]};
  return r;
}
}  // namespace covar

namespace cfar {
enum class Mode : unsigned { kCA = 0, kGO = 1 };
enum class OutMode : unsigned { kEvents = 0, kDense = 1 };
struct Config {
  bool enable = true;
  Mode mode = Mode::kCA;
  OutMode out_mode = OutMode::kEvents;
  unsigned guard_lead = 2, guard_lag = 2, ref_lead = 8, ref_lag = 8;
  unsigned alpha = 1u << 8;
};
struct Event {
  unsigned kind = 3, bin = 0, frame_id = 0, ref_count = 0, alpha = 0;
  unsigned det_count = 0, sup_count = 0;
  uint64_t cut_power = 0, noise_sum = 0;
  bool sof = false, eof = false;
  rd_event raw{};
};
inline uint64_t field(const rd_event& e, unsigned lsb, unsigned n) {
  uint64_t v = 0;
  for (unsigned i = 0; i < n; ++i) {
    const unsigned b = lsb + i;
    if ((e.w[b / 64] >> (b % 64)) & 1ull) v |= 1ull << i;
  }
  return v;
}
// frames of n cells each (signed, clamped at zero as clamp_cell does)
inline std::vector<Event> run_frames(const std::vector<int64_t>& cells, unsigned n,
                                     const Config& c, unsigned max_guard, unsigned max_ref,
                                     const std::vector<uint32_t>& frame_ids) {
  rd_config k;
  rd_config_default(&k);
  k.cfar_enable = c.enable;
  k.cfar_mode = static_cast<uint32_t>(c.mode);
  k.cfar_out_mode = static_cast<uint32_t>(c.out_mode);
  k.guard_lead = c.guard_lead;
  k.guard_lag = c.guard_lag;
  k.ref_lead = c.ref_lead;
  k.ref_lag = c.ref_lag;
  k.alpha = c.alpha;
  k.max_guard = max_guard;
  k.max_ref = max_ref;
  const uint32_t frames = static_cast<uint32_t>(frame_ids.size());
  std::vector<rd_event> ev(static_cast<size_t>(frames) * (n + 1));
  uint64_t ne = 0;
  check(rd_cfar_run(cells.data(), n, frames, &k, frame_ids.data(), ev.data(), ev.size(), &ne),
        "rd_cfar_run");
  std::vector<Event> r(ne);
  for (uint64_t i = 0; i < ne; ++i) {
    const rd_event& e = ev[i];
    r[i].raw = e;
    r[i].kind = static_cast<unsigned>(field(e, 0, 2));
    r[i].bin = static_cast<unsigned>(field(e, 2, 16));
    r[i].frame_id = static_cast<unsigned>(field(e, 18, 16));
    r[i].ref_count = static_cast<unsigned>(field(e, 34, 7));
    r[i].alpha = static_cast<unsigned>(field(e, 41, 16));
    r[i].det_count = static_cast<unsigned>(field(e, 57, 16));
    r[i].sup_count = static_cast<unsigned>(field(e, 73, 16));
    r[i].cut_power = field(e, 89, 40);
    r[i].noise_sum = field(e, 129, 47);
    r[i].sof = (e.framing & 1u) != 0;
    r[i].eof = (e.framing & 2u) != 0;
  }
  return r;
}
inline std::vector<Event> run_frame(const std::vector<uint64_t>& bins, const Config& c,
                                    unsigned max_guard, unsigned max_ref, unsigned frame_id) {
  std::vector<int64_t> cells(bins.begin(), bins.end());
  return run_frames(cells, static_cast<unsigned>(bins.size()), c, max_guard, max_ref,
                    {frame_id});
}
}  // namespace cfar

namespace packet_model {
// One detection packet per event, flits of rd_flit_words(packet_w) words.
inline std::vector<uint32_t> detection_packets(const std::vector<rd_event>& ev, unsigned packet_w,
                                               unsigned src, unsigned dest, unsigned vc,
                                               unsigned seq0) {
  std::vector<uint32_t> fl(ev.size() * rd_detection_flits(packet_w) * rd_flit_words(packet_w));
  check(rd_packetize(ev.data(), ev.size(), packet_w, src, dest, vc, seq0, fl.data()),
        "rd_packetize");
  return fl;
}
}  // namespace packet_model

// The whole chain of one stream, with every piece of state on the GPU.
class Chain {
 public:
  Chain(const rd_config& cfg, const std::vector<rd_cplx16>& coeff,
        const std::vector<rd_cplx16>& weights) {
    check(rd_chain_create(&cfg, &h_), "rd_chain_create");
    check(rd_chain_set_coeff(h_, coeff.data()), "rd_chain_set_coeff");
    check(rd_chain_set_weights(h_, weights.data()), "rd_chain_set_weights");
  }
  ~Chain() { rd_chain_destroy(h_); }
  Chain(const Chain&) = delete;
  Chain& operator=(const Chain&) = delete;
  rd_status process(const rd_cplx16* adc, uint64_t n, uint64_t ld, rd_output* out) {
    return rd_chain_process(h_, adc, n, ld, out);
  }
  rd_stats stats() const {
    rd_stats s;
    check(rd_chain_stats(h_, &s), "rd_chain_stats");
    return s;
  }
  rd_chain* handle() { return h_; }

 private:
  rd_chain* h_ = nullptr;
};

}  // namespace rdgb

#endif  // RD_MODEL_HPP_
