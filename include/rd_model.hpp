// rd_model.hpp - C++ facade with the call surface of the reference model
// (fpga-professional-association/agilex-7-radar-detect, model/cpp), computed
// on the GPU through the C ABI of rd_chain.h.
//
// The namespaces, class names, member names and signatures are the
// reference's, inside namespace rdgb so both can be included side by side. A
// caller of the reference switches by changing the include and adding
// `rdgb::`:
//
//   reference (model/cpp)                          this facade
//   ---------------------------------------------  -----------------------------
//   pfb::PfbModel(phases, taps, coeff)             rdgb::pfb::PfbModel
//     .set_coeff / .swap_coeff / .reset / .step    (pfb_model.hpp:207-258)
//   pfb::BeatResult {y, flags_re, flags_im}        rdgb::pfb::BeatResult
//   pfb::load_coeff / load_io, CoeffHeader,        rdgb::pfb::load_coeff / load_io
//     IoHeader, IoVector, coeff_index, acc_w       (pfb_model.hpp:82-111, 273-544)
//   fft::Config, fft::Result, fft::transform       rdgb::fft::* (fft_ref.hpp:199-240,
//                                                  409-412)
//   bf::DotResult, bf::dot                         rdgb::bf::* (beamformer_model.hpp:
//                                                  145-184)
//   bf::BeamBeat, bf::OutBeatExp,                  rdgb::bf::* (:230-303)
//     bf::BeamformerModel(n_ant, n_beams, bin_par, w)
//   bf::split_beat, beam_mux, seq_shift,           rdgb::bf::* (:127-139, 331-427)
//     weight_index, unit_weights,
//     unit_weight_expect, zero_weights,
//     max_weights, permute_weights
//   covar::power / cross_power, covar::Cross       rdgb::covar::* (covar_model.hpp:
//                                                  99-151)
//   cfar::Config, cfar::Event, clamp_config,       rdgb::cfar::* (cfar_model.hpp:
//     run_frame                                    112-217, 295-340)
//   packet_model::Header, hdr_pack, hdr_unpack,    rdgb::packet_model::*
//     Flit, total_flits, detection_flits           (packet_model.hpp:110-260)
//   (composed only in RTL in the reference)        rdgb::Chain (rd_chain_*)
//
// Deliberately absent: bf::dot_float / step_float (a double-precision
// cross-check of the model against itself, not part of the data path); the
// FFT, beamformer and CFAR latency and register-width helpers (RTL timing,
// no arithmetic); cfar::decide (the per-bin body of run_frame, which runs on
// the GPU inside run_frame here); covar::Integrator / Engine, hist::Model and
// algn::Model as separate objects (rdgb::Chain keeps their state on the GPU and
// returns their results and counters); packet_model::make_flit and Scoreboard
// as host objects (detection packets are built on the GPU by
// detection_packets; the fabric merge is rd_egress_merge).
//
// Errors. Like the reference, nothing here throws. Every call that can fail
// records its status; rdgb::last_status() and rdgb::last_error() return the
// last failure of the calling thread (RD_OK when the last call succeeded),
// and a failed call returns an empty or default result. The loaders return
// bool and fill `err`, as the reference's do.
//
// Every compute call runs CUDA kernels. The per-block classes move one call's
// data to the device and back; batch many beats or frames per call
// (step_many, transform_many, run_frames) for throughput, or use rdgb::Chain,
// which keeps all stream state resident on the GPU.
#ifndef RD_MODEL_HPP_
#define RD_MODEL_HPP_

#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "rd_chain.h"

namespace rdgb {

namespace detail {
inline rd_status& status_slot() {
  static thread_local rd_status s = RD_OK;
  return s;
}
// records the outcome of a call; true on success
inline bool record(rd_status s) {
  status_slot() = s;
  return s == RD_OK;
}
}  // namespace detail

// The status of the calling thread's last facade call, and its description.
inline rd_status last_status() { return detail::status_slot(); }
inline const char* last_error() {
  return detail::status_slot() == RD_OK ? "" : rd_last_error();
}

// ---------------------------------------------------------------------------
// fixed-point types (fxp.hpp:148-150, 279-297)
// ---------------------------------------------------------------------------
namespace fxp {
using i16 = int16_t;
using wide_t = int64_t;
struct Complex {
  i16 re = 0;
  i16 im = 0;
  uint32_t packed() const {
    return (static_cast<uint32_t>(static_cast<uint16_t>(im)) << 16) | static_cast<uint16_t>(re);
  }
  static Complex from_packed(uint32_t p) {
    return Complex{static_cast<i16>(static_cast<uint16_t>(p & 0xFFFFu)),
                   static_cast<i16>(static_cast<uint16_t>(p >> 16))};
  }
  bool operator==(const Complex& o) const { return re == o.re && im == o.im; }
  bool operator!=(const Complex& o) const { return !(*this == o); }
};
struct Flags {
  bool sat_pos = false;
  bool sat_neg = false;
  unsigned packed() const { return (sat_pos ? 2u : 0u) | (sat_neg ? 1u : 0u); }
  static Flags from_packed(unsigned p) { return Flags{(p & 2u) != 0, (p & 1u) != 0}; }
  bool any() const { return sat_pos || sat_neg; }
  bool operator==(const Flags& o) const { return sat_pos == o.sat_pos && sat_neg == o.sat_neg; }
};
inline Flags flags_merge(Flags a, Flags b) { return Flags{a.sat_pos || b.sat_pos, a.sat_neg || b.sat_neg}; }
constexpr i16 q15_max() { return 32767; }
constexpr i16 q15_min() { return -32768; }
inline std::vector<uint32_t> pack(const std::vector<Complex>& v) {
  std::vector<uint32_t> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = v[i].packed();
  return o;
}
inline std::vector<Complex> unpack(const std::vector<uint32_t>& v) {
  std::vector<Complex> o(v.size());
  for (size_t i = 0; i < v.size(); ++i) o[i] = Complex::from_packed(v[i]);
  return o;
}
}  // namespace fxp

// ---------------------------------------------------------------------------
// PFB (pfb_model.hpp)
// ---------------------------------------------------------------------------
namespace pfb {
using fxp::Complex;
using fxp::Flags;
using fxp::i16;

constexpr int kSchemaVersion = 1;
constexpr size_t coeff_index(unsigned taps, unsigned phase, unsigned tap) {
  return static_cast<size_t>(phase) * taps + tap;
}
// the accumulator width the model declares for a bank: 32 + ceil(log2(2 taps))
inline unsigned acc_w(unsigned taps) {
  unsigned g = 0;
  while ((1u << g) < 2u * taps) ++g;
  return 32u + g;
}

struct BeatResult {
  std::vector<Complex> y;
  std::vector<Flags> flags_re;
  std::vector<Flags> flags_im;
  Flags merged() const {
    Flags m;
    for (size_t i = 0; i < flags_re.size(); ++i)
      m = fxp::flags_merge(m, fxp::flags_merge(flags_re[i], flags_im[i]));
    return m;
  }
};

class PfbModel {
 public:
  PfbModel() = default;
  // `coeff`: phases * taps entries, phase-major, tap-minor (coeff_index)
  PfbModel(unsigned phases, unsigned taps, const std::vector<Complex>& coeff)
      : phases_(phases), taps_(taps),
        state_(static_cast<size_t>(taps > 1 ? taps - 1 : 1) * phases, 0u) {
    set_coeff(coeff);
  }
  // a new bank with the history cleared
  void set_coeff(const std::vector<Complex>& coeff) {
    coeff_ = fxp::pack(coeff);
    coeff_.resize(static_cast<size_t>(phases_) * taps_, 0u);
    reset();
  }
  // a new bank, the history kept (a mid-stream bank swap)
  void swap_coeff(const std::vector<Complex>& coeff) {
    coeff_ = fxp::pack(coeff);
    coeff_.resize(static_cast<size_t>(phases_) * taps_, 0u);
  }
  void reset() { std::fill(state_.begin(), state_.end(), 0u); }
  unsigned phases() const { return phases_; }
  unsigned taps() const { return taps_; }

  BeatResult step(const std::vector<Complex>& beat) {
    std::vector<BeatResult> r = step_many(beat, 1);
    return r.empty() ? BeatResult{} : r.front();
  }
  // `beats` consecutive beats of phases() samples each in one GPU call.
  std::vector<BeatResult> step_many(const std::vector<Complex>& x, unsigned beats) {
    std::vector<uint32_t> in = fxp::pack(x);
    in.resize(static_cast<size_t>(beats) * phases_, 0u);
    std::vector<uint32_t> out(in.size());
    std::vector<uint8_t> fl(in.size());
    if (!detail::record(rd_pfb_run(phases_, taps_, coeff_.data(), state_.data(), in.data(), beats,
                                   out.data(), fl.data())))
      return {};
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

 private:
  unsigned phases_ = 0, taps_ = 0;
  std::vector<uint32_t> coeff_, state_;
};

// ---- the .coeff / .vec file formats (pfb_model.hpp:262-544) ----------------
// Line oriented ASCII: `# key: value` header lines, other `#` lines comments,
// then records of whitespace-separated integers. Counts and geometry are
// checked against the header.
struct CoeffHeader {
  int schema = 0;
  std::string kind, set, window, rounding_mode;
  unsigned phases = 0, taps = 0, coeff_w = 0, frac_w = 0;
  uint64_t seed = 0;
  size_t declared_count = 0;
};
struct IoHeader {
  int schema = 0;
  std::string kind, set, coeff_file, rounding_mode;
  unsigned phases = 0, taps = 0, acc_w = 0;
  uint64_t seed = 0;
  size_t declared_count = 0;
};
struct IoVector {
  size_t beat = 0;
  std::vector<Complex> x, y;
  std::vector<unsigned> f_re, f_im;
};

namespace detail {
inline std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}
// `# key: value` -> (key, value); false for any other line
inline bool key_value(const std::string& line, std::string* k, std::string* v) {
  if (line.empty() || line[0] != '#') return false;
  const size_t c = line.find(':');
  if (c == std::string::npos) return false;
  *k = trim(line.substr(1, c - 1));
  *v = trim(line.substr(c + 1));
  return true;
}
inline bool all_ints(const std::string& line, std::vector<long long>* out) {
  std::istringstream is(line);
  std::string tok;
  out->clear();
  while (is >> tok) {
    char* end = nullptr;
    const long long v = std::strtoll(tok.c_str(), &end, 10);
    if (end == tok.c_str() || *end != '\0') return false;
    out->push_back(v);
  }
  return true;
}
inline unsigned to_u(const std::string& s) {
  return static_cast<unsigned>(std::strtoul(s.c_str(), nullptr, 10));
}
// the body lines of a file, with every header key collected
template <class OnKey>
inline bool read_lines(const std::string& path, OnKey on_key, std::vector<std::string>* body,
                       std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open " + path;
    return false;
  }
  std::string line, k, v;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (key_value(line, &k, &v)) {
      on_key(k, v);
      continue;
    }
    if (line.empty() || line[0] == '#') continue;
    body->push_back(line);
  }
  return true;
}
}  // namespace detail

inline bool load_coeff(const std::string& path, std::vector<Complex>* out, CoeffHeader* header,
                       std::string* err) {
  CoeffHeader h;
  std::vector<std::string> body;
  auto on_key = [&](const std::string& k, const std::string& v) {
    if (k == "schema") h.schema = static_cast<int>(detail::to_u(v));
    else if (k == "kind") h.kind = v;
    else if (k == "set") h.set = v;
    else if (k == "window") h.window = v;
    else if (k == "rounding_mode") h.rounding_mode = v;
    else if (k == "phases") h.phases = detail::to_u(v);
    else if (k == "taps") h.taps = detail::to_u(v);
    else if (k == "coeff_w") h.coeff_w = detail::to_u(v);
    else if (k == "frac_w") h.frac_w = detail::to_u(v);
    else if (k == "seed") h.seed = std::strtoull(v.c_str(), nullptr, 10);
    else if (k == "count") h.declared_count = detail::to_u(v);
  };
  if (!detail::read_lines(path, on_key, &body, err)) return false;
  std::vector<Complex> vals;
  std::vector<long long> f;
  for (size_t r = 0; r < body.size(); ++r) {
    if (!detail::all_ints(body[r], &f) || f.size() != 5) {
      *err = path + ": expected 5 integer fields in \"" + body[r] + "\"";
      return false;
    }
    // index, phase, tap, re, im; the index must follow the row order and
    // agree with (phase, tap)
    if (static_cast<size_t>(f[0]) != r ||
        (h.taps && static_cast<size_t>(f[0]) !=
                       coeff_index(h.taps, static_cast<unsigned>(f[1]), static_cast<unsigned>(f[2])))) {
      *err = path + ": row " + std::to_string(r) + " declares index " + std::to_string(f[0]);
      return false;
    }
    vals.push_back(Complex{static_cast<i16>(f[3]), static_cast<i16>(f[4])});
  }
  if (h.schema != kSchemaVersion || h.kind != "pfb_coeff") {
    *err = path + ": not a schema " + std::to_string(kSchemaVersion) + " pfb_coeff file";
    return false;
  }
  if (h.declared_count != vals.size() || static_cast<size_t>(h.phases) * h.taps != vals.size()) {
    *err = path + ": " + std::to_string(vals.size()) + " records against count " +
           std::to_string(h.declared_count) + " and a " + std::to_string(h.phases) + "x" +
           std::to_string(h.taps) + " bank";
    return false;
  }
  *out = vals;
  if (header) *header = h;
  return true;
}

inline bool load_io(const std::string& path, std::vector<IoVector>* out, IoHeader* header,
                    std::string* err) {
  IoHeader h;
  std::vector<std::string> body;
  auto on_key = [&](const std::string& k, const std::string& v) {
    if (k == "schema") h.schema = static_cast<int>(detail::to_u(v));
    else if (k == "kind") h.kind = v;
    else if (k == "set") h.set = v;
    else if (k == "coeff_file") h.coeff_file = v;
    else if (k == "rounding_mode") h.rounding_mode = v;
    else if (k == "phases") h.phases = detail::to_u(v);
    else if (k == "taps") h.taps = detail::to_u(v);
    else if (k == "acc_w") h.acc_w = detail::to_u(v);
    else if (k == "seed") h.seed = std::strtoull(v.c_str(), nullptr, 10);
    else if (k == "count") h.declared_count = detail::to_u(v);
  };
  if (!detail::read_lines(path, on_key, &body, err)) return false;
  std::vector<IoVector> vals;
  std::vector<long long> f;
  const size_t want = 1 + 6u * h.phases;  // beat, x and y pairs, flag pairs
  for (const std::string& line : body) {
    if (h.phases == 0 || !detail::all_ints(line, &f) || f.size() != want) {
      *err = path + ": expected " + std::to_string(want) + " integer fields";
      return false;
    }
    IoVector r;
    r.beat = static_cast<size_t>(f[0]);
    size_t c = 1;
    for (unsigned p = 0; p < h.phases; ++p, c += 2)
      r.x.push_back(Complex{static_cast<i16>(f[c]), static_cast<i16>(f[c + 1])});
    for (unsigned p = 0; p < h.phases; ++p, c += 2)
      r.y.push_back(Complex{static_cast<i16>(f[c]), static_cast<i16>(f[c + 1])});
    for (unsigned p = 0; p < h.phases; ++p, c += 2) {
      r.f_re.push_back(static_cast<unsigned>(f[c]));
      r.f_im.push_back(static_cast<unsigned>(f[c + 1]));
    }
    vals.push_back(std::move(r));
  }
  if (h.schema != kSchemaVersion || h.kind != "pfb_io") {
    *err = path + ": not a schema " + std::to_string(kSchemaVersion) + " pfb_io file";
    return false;
  }
  if (h.declared_count != vals.size()) {
    *err = path + ": declares " + std::to_string(h.declared_count) + " beats, holds " +
           std::to_string(vals.size());
    return false;
  }
  if (h.acc_w != 0 && h.acc_w != acc_w(h.taps)) {
    *err = path + ": acc_w " + std::to_string(h.acc_w) + " against " + std::to_string(acc_w(h.taps));
    return false;
  }
  *out = vals;
  if (header) *header = h;
  return true;
}
}  // namespace pfb

// ---------------------------------------------------------------------------
// FFT (fft_ref.hpp)
// ---------------------------------------------------------------------------
namespace fft {
using fxp::Complex;
using fxp::Flags;
constexpr unsigned kSchedAll = 0xFFFFFFFFu;
struct Config {
  unsigned n_fft = 64;
  unsigned spc = 2;
  unsigned scale_sched = kSchedAll;
  bool reorder = true;
  unsigned stages() const {
    unsigned s = 0;
    while ((1u << s) < n_fft) ++s;
    return s;
  }
  bool valid() const {
    const bool p2 = n_fft && !(n_fft & (n_fft - 1));
    return p2 && n_fft >= 8 && n_fft <= 1024 && (spc == 1 || spc == 2) && n_fft / spc >= 4;
  }
};
struct Result {
  std::vector<Complex> out;        // beat order (fft_ref.hpp:223-227)
  std::vector<Flags> stage_flags;  // one per butterfly sub-stage
  std::vector<Complex> bins;       // natural bin order
};
// `frames` transforms of n_fft samples each in one GPU call
inline std::vector<Result> transform_many(const Config& c, const std::vector<Complex>& in,
                                          unsigned frames) {
  std::vector<uint32_t> x = fxp::pack(in);
  x.resize(static_cast<size_t>(frames) * c.n_fft, 0u);
  std::vector<uint32_t> out(x.size()), bins(x.size());
  const unsigned st = c.stages();
  std::vector<uint8_t> sf(static_cast<size_t>(frames) * st);
  if (!detail::record(rd_fft_run(c.n_fft, c.spc, c.scale_sched, c.reorder ? 1 : 0, x.data(), frames,
                                 out.data(), bins.data(), sf.data())))
    return {};
  std::vector<Result> r(frames);
  for (unsigned f = 0; f < frames; ++f) {
    const size_t o = static_cast<size_t>(f) * c.n_fft;
    for (unsigned i = 0; i < c.n_fft; ++i) {
      r[f].out.push_back(Complex::from_packed(out[o + i]));
      r[f].bins.push_back(Complex::from_packed(bins[o + i]));
    }
    for (unsigned s = 0; s < st; ++s)
      r[f].stage_flags.push_back(Flags::from_packed(sf[static_cast<size_t>(f) * st + s]));
  }
  return r;
}
inline Result transform(const Config& c, const std::vector<Complex>& in) {
  std::vector<Result> r = transform_many(c, in, 1);
  return r.empty() ? Result{} : r.front();
}
}  // namespace fft

// ---------------------------------------------------------------------------
// Beamformer (beamformer_model.hpp)
// ---------------------------------------------------------------------------
namespace bf {
using fxp::Complex;
using fxp::Flags;
using fxp::wide_t;

inline size_t weight_index(unsigned n_ant, unsigned beam, unsigned ant) {
  return static_cast<size_t>(beam) * n_ant + ant;
}
inline unsigned beam_mux(unsigned n_beams, unsigned beam_par) {
  return beam_par == 0u ? 1u : n_beams / beam_par;
}
// ceil(log2(mux)) bits of output beat index appended to the sequence number
inline unsigned seq_shift(unsigned mux) {
  unsigned l = 0;
  while ((1u << l) < mux) ++l;
  return mux <= 1u ? 0u : l;
}

struct DotResult {
  Complex y;
  Flags f_re, f_im;
  wide_t acc_re = 0, acc_im = 0;
  Flags merged() const { return fxp::flags_merge(f_re, f_im); }
  bool saturating() const { return merged().any(); }
};

// Y[v][b] for n_vec antenna vectors x[v][a] and beam-major weights w[b][a],
// one GPU call; result index v * n_beams + b. `form` picks the contraction
// (RD_FORM_*); every form gives the same bits.
inline std::vector<DotResult> dot_many(const std::vector<Complex>& x, const std::vector<Complex>& w,
                                       unsigned n_ant, unsigned n_beams,
                                       uint32_t form = RD_FORM_CUDA_CORE) {
  const std::vector<uint32_t> xp = fxp::pack(x), wp = fxp::pack(w);
  const uint64_t nv = n_ant ? xp.size() / n_ant : 0;
  std::vector<uint32_t> y(nv * n_beams);
  std::vector<int64_t> acc(nv * n_beams * 2);
  std::vector<uint8_t> fl(nv * n_beams);
  if (!detail::record(rd_bf_run(n_ant, n_beams, wp.data(), xp.data(), nv, y.data(), acc.data(),
                                fl.data(), form)))
    return {};
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
  std::vector<DotResult> r = dot_many(std::vector<Complex>(x, x + n_ant),
                                      std::vector<Complex>(w, w + n_ant), n_ant, 1);
  return r.empty() ? DotResult{} : r.front();
}
inline DotResult dot(const std::vector<Complex>& x, const std::vector<Complex>& w) {
  return dot(x.data(), w.data(), static_cast<unsigned>(x.size()));
}

// every beam of every bin of one input beat: [beam][bin]
struct BeamBeat {
  std::vector<std::vector<Complex>> y;
  std::vector<std::vector<Flags>> f_re, f_im;
  std::vector<std::vector<wide_t>> acc_re, acc_im;
  bool saturating = false;
  unsigned n_beams() const { return static_cast<unsigned>(y.size()); }
  unsigned n_bins() const { return y.empty() ? 0u : static_cast<unsigned>(y[0].size()); }
};

// one output beat: beam_par beams x bin_par bins of one beam group
struct OutBeatExp {
  std::vector<Complex> data;  // [k * bins + j]
  uint32_t seq = 0;
  uint32_t user = 0;  // the beam group
  bool sof = false, eof = false;
  uint32_t stream_id = 0;
  bool saturating = false;
};

class BeamformerModel {
 public:
  BeamformerModel() = default;
  // `w`: n_beams * n_ant weights, beam-major (weight_index)
  BeamformerModel(unsigned n_ant, unsigned n_beams, unsigned bin_par, const std::vector<Complex>& w,
                  uint32_t form = RD_FORM_CUDA_CORE)
      : n_ant_(n_ant), n_beams_(n_beams), bin_par_(bin_par), w_(w), form_(form) {
    w_.resize(static_cast<size_t>(n_beams) * n_ant);
  }
  unsigned n_ant() const { return n_ant_; }
  unsigned n_beams() const { return n_beams_; }
  unsigned bin_par() const { return bin_par_; }
  const std::vector<Complex>& weights() const { return w_; }
  // the next beat is computed entirely with the new bank
  void swap_weights(const std::vector<Complex>& w) {
    w_ = w;
    w_.resize(static_cast<size_t>(n_beams_) * n_ant_);
  }
  // `beat`: x[bin][antenna], bin_par x n_ant
  BeamBeat step(const std::vector<std::vector<Complex>>& beat) const {
    std::vector<Complex> x;
    x.reserve(static_cast<size_t>(bin_par_) * n_ant_);
    for (unsigned j = 0; j < bin_par_; ++j) {
      std::vector<Complex> v = j < beat.size() ? beat[j] : std::vector<Complex>();
      v.resize(n_ant_);
      x.insert(x.end(), v.begin(), v.end());
    }
    const std::vector<DotResult> d = dot_many(x, w_, n_ant_, n_beams_, form_);
    BeamBeat r;
    if (d.size() != static_cast<size_t>(bin_par_) * n_beams_) return r;
    r.y.assign(n_beams_, std::vector<Complex>(bin_par_));
    r.f_re.assign(n_beams_, std::vector<Flags>(bin_par_));
    r.f_im.assign(n_beams_, std::vector<Flags>(bin_par_));
    r.acc_re.assign(n_beams_, std::vector<wide_t>(bin_par_));
    r.acc_im.assign(n_beams_, std::vector<wide_t>(bin_par_));
    for (unsigned j = 0; j < bin_par_; ++j)
      for (unsigned b = 0; b < n_beams_; ++b) {
        const DotResult& e = d[static_cast<size_t>(j) * n_beams_ + b];
        r.y[b][j] = e.y;
        r.f_re[b][j] = e.f_re;
        r.f_im[b][j] = e.f_im;
        r.acc_re[b][j] = e.acc_re;
        r.acc_im[b][j] = e.acc_im;
        r.saturating = r.saturating || e.saturating();
      }
    return r;
  }

 private:
  unsigned n_ant_ = 0, n_beams_ = 0, bin_par_ = 0;
  std::vector<Complex> w_;
  uint32_t form_ = RD_FORM_CUDA_CORE;
};

// One beat's beams into the output beats of beam_par beams each: group g
// carries beams g beam_par .. + beam_par - 1, its sequence number is seq_in
// with the group index appended (seq_shift bits), sof on the first group and
// eof on the last.
inline std::vector<OutBeatExp> split_beat(const BeamBeat& r, unsigned beam_par, uint32_t seq_in,
                                          uint32_t stream_id, bool sof_in, bool eof_in) {
  const unsigned bins = r.n_bins(), mux = beam_mux(r.n_beams(), beam_par), sh = seq_shift(mux);
  std::vector<OutBeatExp> out(mux);
  for (unsigned g = 0; g < mux; ++g) {
    OutBeatExp& o = out[g];
    o.data.resize(static_cast<size_t>(beam_par) * bins);
    o.seq = sh ? ((seq_in << sh) | g) : seq_in;
    o.user = g;
    o.sof = sof_in && g == 0u;
    o.eof = eof_in && g + 1u == mux;
    o.stream_id = stream_id;
    for (unsigned k = 0; k < beam_par; ++k)
      for (unsigned j = 0; j < bins; ++j) {
        const unsigned b = g * beam_par + k;
        o.data[static_cast<size_t>(k) * bins + j] = r.y[b][j];
        o.saturating = o.saturating || r.f_re[b][j].any() || r.f_im[b][j].any();
      }
  }
  return out;
}

// ---- the directed weight sets (beamformer_model.hpp:375-427) ----
// beam b passes antenna sel[b % sel.size()] % n_ant with gain 0x7FFF
inline std::vector<Complex> unit_weights(unsigned n_ant, unsigned n_beams,
                                         const std::vector<unsigned>& sel) {
  std::vector<Complex> w(static_cast<size_t>(n_beams) * n_ant);
  for (unsigned b = 0; b < n_beams && !sel.empty(); ++b)
    w[weight_index(n_ant, b, sel[b % sel.size()] % n_ant)] = Complex{fxp::q15_max(), 0};
  return w;
}
// the sample a unit-weight beam passes: x times 0x7FFF, rounded and saturated once
inline Complex unit_weight_expect(Complex x) {
  const Complex w{fxp::q15_max(), 0};
  return dot(&x, &w, 1u).y;
}
inline std::vector<Complex> zero_weights(unsigned n_ant, unsigned n_beams) {
  return std::vector<Complex>(static_cast<size_t>(n_beams) * n_ant);
}
// every weight -1 - 1j, the extreme of a complex product
inline std::vector<Complex> max_weights(unsigned n_ant, unsigned n_beams) {
  return std::vector<Complex>(static_cast<size_t>(n_beams) * n_ant,
                              Complex{fxp::q15_min(), fxp::q15_min()});
}
// w_out[b][p[a]] = w_in[b][a]
inline std::vector<Complex> permute_weights(const std::vector<Complex>& w, unsigned n_ant,
                                            unsigned n_beams, const std::vector<unsigned>& p) {
  std::vector<Complex> out(w.size());
  for (unsigned b = 0; b < n_beams; ++b)
    for (unsigned a = 0; a < n_ant; ++a) out[weight_index(n_ant, b, p[a])] = w[weight_index(n_ant, b, a)];
  return out;
}
}  // namespace bf

// ---------------------------------------------------------------------------
// Power and cross power (covar_model.hpp:99-151)
// ---------------------------------------------------------------------------
namespace covar {
using fxp::Complex;
struct Cross {
  int64_t re = 0, im = 0;
  bool operator==(const Cross& o) const { return re == o.re && im == o.im; }
};
inline std::vector<int64_t> power(const std::vector<Complex>& s) {
  const std::vector<uint32_t> x = fxp::pack(s);
  std::vector<int64_t> p(x.size());
  if (!detail::record(rd_power_run(x.data(), x.size(), p.data()))) return {};
  return p;
}
inline int64_t power(Complex s) {
  const std::vector<int64_t> p = power(std::vector<Complex>{s});
  return p.empty() ? 0 : p[0];
}
inline std::vector<Cross> cross_power(const std::vector<Complex>& x, const std::vector<Complex>& y) {
  const std::vector<uint32_t> a = fxp::pack(x), b = fxp::pack(y);
  std::vector<int64_t> c(2 * a.size());
  if (a.size() != b.size() ||
      !detail::record(rd_cross_power_run(a.data(), b.data(), a.size(), c.data())))
    return {};
  std::vector<Cross> r(a.size());
  for (size_t i = 0; i < r.size(); ++i) r[i] = Cross{c[2 * i], c[2 * i + 1]};
  return r;
}
inline Cross cross_power(Complex x, Complex y) {
  const std::vector<Cross> r = cross_power(std::vector<Complex>{x}, std::vector<Complex>{y});
  return r.empty() ? Cross{} : r[0];
}
}  // namespace covar

// ---------------------------------------------------------------------------
// CFAR (cfar_model.hpp)
// ---------------------------------------------------------------------------
namespace cfar {
enum class Mode : unsigned { kCA = 0, kGO = 1 };
enum class OutMode : unsigned { kEvents = 0, kDense = 1 };
enum : unsigned { kEvDetect = RD_EV_DETECT, kEvBin = RD_EV_BIN, kEvSuppressed = RD_EV_SUPPRESSED,
                  kEvSummary = RD_EV_SUMMARY };
constexpr unsigned kAlphaOne = 1u << 8;
struct Config {
  bool enable = true;
  Mode mode = Mode::kCA;
  OutMode out_mode = OutMode::kEvents;
  unsigned guard_lead = 2, guard_lag = 2, ref_lead = 8, ref_lag = 8;
  unsigned alpha = kAlphaOne;
  bool operator==(const Config& o) const {
    return enable == o.enable && mode == o.mode && out_mode == o.out_mode &&
           guard_lead == o.guard_lead && guard_lag == o.guard_lag && ref_lead == o.ref_lead &&
           ref_lag == o.ref_lag && alpha == o.alpha;
  }
  bool operator!=(const Config& o) const { return !(*this == o); }
};
// the geometry as the detector latches it: guards and references at most
// the elaborated maxima
inline Config clamp_config(const Config& c, unsigned max_guard, unsigned max_ref) {
  Config o = c;
  o.guard_lead = std::min(c.guard_lead, max_guard);
  o.guard_lag = std::min(c.guard_lag, max_guard);
  o.ref_lead = std::min(c.ref_lead, max_ref);
  o.ref_lag = std::min(c.ref_lag, max_ref);
  return o;
}
struct Event {
  unsigned kind = kEvSummary;
  unsigned bin = 0;  // the frame length on a summary
  unsigned frame_id = 0, ref_count = 0, alpha = 0;
  unsigned det_count = 0, sup_count = 0;  // summary only
  uint64_t cut_power = 0, noise_sum = 0;
  bool sof = false, eof = false;
  bool operator==(const Event& o) const {
    return kind == o.kind && bin == o.bin && frame_id == o.frame_id && ref_count == o.ref_count &&
           alpha == o.alpha && det_count == o.det_count && sup_count == o.sup_count &&
           cut_power == o.cut_power && noise_sum == o.noise_sum && sof == o.sof && eof == o.eof;
  }
  bool operator!=(const Event& o) const { return !(*this == o); }
};
// bits [lsb, lsb + n) of the 176-bit event word (cfar_model.hpp:75-84)
inline uint64_t event_field(const rd_event& e, unsigned lsb, unsigned n) {
  uint64_t v = 0;
  for (unsigned i = 0; i < n; ++i) {
    const unsigned b = lsb + i;
    if ((e.w[b / 64] >> (b % 64)) & 1ull) v |= 1ull << i;
  }
  return v;
}
inline Event decode(const rd_event& e) {
  Event r;
  r.kind = static_cast<unsigned>(event_field(e, 0, 2));
  r.bin = static_cast<unsigned>(event_field(e, 2, 16));
  r.frame_id = static_cast<unsigned>(event_field(e, 18, 16));
  r.ref_count = static_cast<unsigned>(event_field(e, 34, 7));
  r.alpha = static_cast<unsigned>(event_field(e, 41, 16));
  r.det_count = static_cast<unsigned>(event_field(e, 57, 16));
  r.sup_count = static_cast<unsigned>(event_field(e, 73, 16));
  r.cut_power = event_field(e, 89, 40);
  r.noise_sum = event_field(e, 129, 47);
  r.sof = (e.framing & 1u) != 0;
  r.eof = (e.framing & 2u) != 0;
  return r;
}
// `frame_ids.size()` frames of n cells each in one GPU call (cells signed,
// clamped at zero as the model's cell clamp does); the raw events as the
// chain emits them, or decoded
inline std::vector<rd_event> run_frames_raw(const std::vector<int64_t>& cells, unsigned n,
                                            const Config& c, unsigned max_guard, unsigned max_ref,
                                            const std::vector<uint32_t>& frame_ids) {
  rd_config k;
  rd_config_default(&k);
  k.cfar_enable = c.enable ? 1u : 0u;
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
  std::vector<rd_event> ev(static_cast<size_t>(frames) * (n + 1) + 1);
  uint64_t ne = 0;
  if (!detail::record(rd_cfar_run(cells.data(), n, frames, &k, frame_ids.data(), ev.data(), ev.size(),
                                  &ne)))
    return {};
  ev.resize(ne);
  return ev;
}
inline std::vector<Event> run_frames(const std::vector<int64_t>& cells, unsigned n, const Config& c,
                                     unsigned max_guard, unsigned max_ref,
                                     const std::vector<uint32_t>& frame_ids) {
  const std::vector<rd_event> raw = run_frames_raw(cells, n, c, max_guard, max_ref, frame_ids);
  std::vector<Event> r(raw.size());
  for (size_t i = 0; i < raw.size(); ++i) r[i] = decode(raw[i]);
  return r;
}
inline std::vector<Event> run_frame(const std::vector<uint64_t>& bins, const Config& written,
                                    unsigned max_guard, unsigned max_ref, unsigned frame_id) {
  const std::vector<int64_t> cells(bins.begin(), bins.end());
  return run_frames(cells, static_cast<unsigned>(bins.size()), written, max_guard, max_ref,
                    {frame_id});
}
}  // namespace cfar

// ---------------------------------------------------------------------------
// Packets (packet_model.hpp)
// ---------------------------------------------------------------------------
namespace packet_model {
constexpr unsigned kDestW = 4, kSrcW = 5, kVcW = 2, kTypeW = 3, kLenW = 6, kSeqW = 16;
constexpr unsigned kHdrW = kDestW + kSrcW + kVcW + kTypeW + kLenW + kSeqW;  // 36
constexpr unsigned kFlitCtrlW = 5;                                          // parity, vc, sof, eof
constexpr unsigned kFlitParityLsb = 0, kFlitVcLsb = 1, kFlitSofLsb = 3, kFlitEofLsb = 4,
                   kFlitDataLsb = 5;
constexpr unsigned kDetectionPayloadW = 176;
enum PacketType : unsigned { kTypeDetection = 0, kTypePower, kTypeCovar, kTypeError, kTypeCounter,
                             kTypeRaw };
inline unsigned payload_flits(unsigned bits, unsigned packet_w) {
  return packet_w ? (bits + packet_w - 1) / packet_w : 0u;
}
inline unsigned total_flits(unsigned bits, unsigned packet_w) { return 1 + payload_flits(bits, packet_w); }
inline unsigned detection_flits(unsigned packet_w) { return rd_detection_flits(packet_w); }

struct Header {
  unsigned dest = 0, src = 0, vc = 0, ptype = 0;
  unsigned length = 1;  // total flits, header included
  unsigned seq = 0;
  bool operator==(const Header& o) const {
    return dest == o.dest && src == o.src && vc == o.vc && ptype == o.ptype && length == o.length &&
           seq == o.seq;
  }
};
// fields packed LSB first: dest, src, vc, type, length, seq
constexpr unsigned kHdrWidths[6] = {kDestW, kSrcW, kVcW, kTypeW, kLenW, kSeqW};
inline uint64_t hdr_pack(const Header& h) {
  const unsigned v[6] = {h.dest, h.src, h.vc, h.ptype, h.length, h.seq};
  uint64_t p = 0;
  for (unsigned i = 0, at = 0; i < 6; at += kHdrWidths[i], ++i)
    p |= (static_cast<uint64_t>(v[i]) & ((1ull << kHdrWidths[i]) - 1ull)) << at;
  return p;
}
inline Header hdr_unpack(uint64_t p) {
  unsigned v[6];
  for (unsigned i = 0, at = 0; i < 6; at += kHdrWidths[i], ++i)
    v[i] = static_cast<unsigned>((p >> at) & ((1ull << kHdrWidths[i]) - 1ull));
  return Header{v[0], v[1], v[2], v[3], v[4], v[5]};
}

// One flit: packet_w payload bits above the 5 control bits, in 32-bit words.
struct Flit {
  std::vector<uint32_t> w;
  unsigned packet_w = 64;
  unsigned flit_w() const { return packet_w + kFlitCtrlW; }
  bool bit(unsigned i) const { return i / 32 < w.size() && ((w[i / 32] >> (i % 32)) & 1u); }
  uint64_t field(unsigned lsb, unsigned n) const {
    uint64_t v = 0;
    for (unsigned i = 0; i < n; ++i)
      if (bit(lsb + i)) v |= 1ull << i;
    return v;
  }
  unsigned vc() const { return static_cast<unsigned>(field(kFlitVcLsb, kVcW)); }
  bool sof() const { return bit(kFlitSofLsb); }
  bool eof() const { return bit(kFlitEofLsb); }
  bool parity_bit() const { return bit(kFlitParityLsb); }
  bool parity_ok() const {  // odd parity over the whole flit
    unsigned n = 0;
    for (unsigned i = 0; i < flit_w(); ++i) n += bit(i) ? 1u : 0u;
    return (n & 1u) != 0;
  }
  uint64_t data64(unsigned k) const {
    const unsigned lo = k * 64;
    if (lo >= packet_w) return 0;
    return field(kFlitDataLsb + lo, packet_w - lo >= 64 ? 64 : packet_w - lo);
  }
  Header header() const { return hdr_unpack(data64(0) & ((1ull << kHdrW) - 1ull)); }
};

// The detection packets of n events (header flit, then the 176-bit event LS
// word first), built on the GPU; event i carries sequence seq0 + i.
inline std::vector<Flit> detection_packets(const std::vector<rd_event>& ev, unsigned packet_w,
                                           unsigned src, unsigned dest, unsigned vc, unsigned seq0) {
  const unsigned nfl = rd_detection_flits(packet_w), words = rd_flit_words(packet_w);
  std::vector<uint32_t> fl(ev.size() * nfl * words);
  if (!detail::record(rd_packetize(ev.data(), ev.size(), packet_w, src, dest, vc, seq0, fl.data())))
    return {};
  std::vector<Flit> r(ev.size() * nfl);
  for (size_t i = 0; i < r.size(); ++i) {
    r[i].packet_w = packet_w;
    r[i].w.assign(fl.begin() + static_cast<long>(i * words), fl.begin() + static_cast<long>((i + 1) * words));
  }
  return r;
}
}  // namespace packet_model

// ---------------------------------------------------------------------------
// The whole chain of one stream, every piece of state on the GPU.
// ---------------------------------------------------------------------------
class Chain {
 public:
  Chain(const rd_config& cfg, const std::vector<rd_cplx16>& coeff,
        const std::vector<rd_cplx16>& weights) {
    if (!detail::record(rd_chain_create(&cfg, &h_))) return;
    if (!detail::record(rd_chain_set_coeff(h_, coeff.data())) ||
        !detail::record(rd_chain_set_weights(h_, weights.data()))) {
      rd_chain_destroy(h_);
      h_ = nullptr;
    }
  }
  ~Chain() { rd_chain_destroy(h_); }
  Chain(const Chain&) = delete;
  Chain& operator=(const Chain&) = delete;
  bool valid() const { return h_ != nullptr; }
  rd_status set_coeff(const std::vector<rd_cplx16>& c) { return status(rd_chain_set_coeff(h_, c.data())); }
  rd_status set_weights(const std::vector<rd_cplx16>& w) {
    return status(rd_chain_set_weights(h_, w.data()));
  }
  rd_status set_pairs(const std::vector<uint32_t>& x, const std::vector<uint32_t>& y) {
    return status(rd_chain_set_pairs(h_, x.data(), y.data(), static_cast<uint32_t>(x.size())));
  }
  rd_status process(const rd_cplx16* adc, uint64_t n, uint64_t ld, rd_output* out) {
    return status(rd_chain_process(h_, adc, n, ld, out));
  }
  rd_status flush_cov(rd_output* out) { return status(rd_chain_flush_cov(h_, out)); }
  // hist::Model::request_depth (history_model.hpp:260-266): lands at once
  rd_status request_depth(uint32_t frames) {
    return status(rd_chain_set_history_depth(h_, frames));
  }
  rd_status reset() { return status(rd_chain_reset(h_, nullptr)); }
  // checkpoint / resume: the stream's state as bytes, and back into a chain
  // of the same configuration (empty on failure; see rdgb::last_status)
  std::vector<uint8_t> save_state() {
    std::vector<uint8_t> b(h_ ? rd_chain_state_size(h_) : 0u);
    if (!h_ || status(rd_chain_save_state(h_, b.data(), b.size())) != RD_OK) b.clear();
    return b;
  }
  rd_status load_state(const std::vector<uint8_t>& b) {
    return status(rd_chain_load_state(h_, b.data(), b.size()));
  }
  rd_stats stats() const {
    rd_stats s{};
    detail::record(rd_chain_stats(h_, &s));
    return s;
  }
  rd_chain* handle() { return h_; }

 private:
  rd_status status(rd_status s) {
    detail::record(h_ ? s : RD_EINVAL);
    return h_ ? s : RD_EINVAL;
  }
  rd_chain* h_ = nullptr;
};

}  // namespace rdgb

#endif  // RD_MODEL_HPP_
