// facade_check.cpp - drives the C++ facade (include/rd_model.hpp) the way a
// caller of the reference model's C++ API would, on inputs a test writes to
// a directory, and writes every result back there as raw little-endian
// arrays for the test to compare with the CPU oracle.
//
//   facade_check loaders <dir> <name>...   parses <dir>/<name>.coeff and
//                                          <name>.vec (no GPU needed)
//   facade_check gpu <dir>                 every facade class on the GPU
//
// Inputs: <dir>/params.txt ("key value" lines) and raw arrays <name>.bin.
// A failed call shows up as a missing output and a "fail" line in
// <dir>/status.txt; nothing throws.
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "rd_model.hpp"

namespace {

std::string g_dir;
std::map<std::string, long long> g_par;
std::ofstream g_status;

template <class T>
std::vector<T> get(const std::string& name) {
  std::ifstream f(g_dir + "/" + name + ".bin", std::ios::binary | std::ios::ate);
  std::vector<T> v(f ? static_cast<size_t>(f.tellg()) / sizeof(T) : 0);
  f.seekg(0);
  f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
  return v;
}
template <class T>
void put(const std::string& name, const std::vector<T>& v) {
  std::ofstream f(g_dir + "/" + name + ".out", std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}
unsigned par(const std::string& k) { return static_cast<unsigned>(g_par.at(k)); }
void note(const std::string& what, bool ok) {
  g_status << what << " " << (ok ? "ok" : "fail") << " " << rdgb::last_error() << "\n";
}

using rdgb::fxp::Complex;

std::vector<Complex> cplx(const std::vector<uint32_t>& v) { return rdgb::fxp::unpack(v); }

void check_pfb() {
  namespace pfb = rdgb::pfb;
  const unsigned P = par("pfb_phases"), T = par("pfb_taps"), beats = par("pfb_beats");
  const std::vector<Complex> c1 = cplx(get<uint32_t>("pfb_coeff")), c2 = cplx(get<uint32_t>("pfb_coeff2"));
  const std::vector<Complex> x = cplx(get<uint32_t>("pfb_x"));
  pfb::PfbModel m(P, T, c1);
  std::vector<uint32_t> y;
  std::vector<uint8_t> fl;
  auto keep = [&](const pfb::BeatResult& r) {
    for (unsigned p = 0; p < r.y.size(); ++p) {
      y.push_back(r.y[p].packed());
      fl.push_back(static_cast<uint8_t>(r.flags_re[p].packed() << 2 | r.flags_im[p].packed()));
    }
  };
  const unsigned half = beats / 2;
  // the first half beat by beat, then a bank swap that keeps the history and
  // the second half in one call
  for (unsigned t = 0; t < half; ++t)
    keep(m.step(std::vector<Complex>(x.begin() + t * P, x.begin() + (t + 1) * P)));
  m.swap_coeff(c2);
  for (const pfb::BeatResult& r :
       m.step_many(std::vector<Complex>(x.begin() + half * P, x.end()), beats - half))
    keep(r);
  note("pfb", y.size() == static_cast<size_t>(beats) * P);
  put("pfb_y", y);
  put("pfb_f", fl);
}

void check_fft() {
  namespace fft = rdgb::fft;
  fft::Config c;
  c.n_fft = par("fft_n");
  c.spc = par("fft_spc");
  c.scale_sched = par("fft_sched");
  c.reorder = par("fft_reorder") != 0;
  const unsigned frames = par("fft_frames");
  const std::vector<Complex> x = cplx(get<uint32_t>("fft_x"));
  const std::vector<fft::Result> r = fft::transform_many(c, x, frames);
  std::vector<uint32_t> out, bins;
  std::vector<uint8_t> sf;
  for (const fft::Result& f : r) {
    for (const Complex& v : f.out) out.push_back(v.packed());
    for (const Complex& v : f.bins) bins.push_back(v.packed());
    for (const rdgb::fxp::Flags& g : f.stage_flags) sf.push_back(static_cast<uint8_t>(g.packed()));
  }
  // the single-frame call gives frame 0 again
  const fft::Result one = fft::transform(c, std::vector<Complex>(x.begin(), x.begin() + c.n_fft));
  bool same = !r.empty() && one.bins == r[0].bins && one.out == r[0].out;
  note("fft", r.size() == frames && c.valid() && same);
  put("fft_out", out);
  put("fft_bins", bins);
  put("fft_sf", sf);
  // an invalid geometry is an error status and an empty result, not an exception
  fft::Config bad = c;
  bad.n_fft = 12;
  const fft::Result e = fft::transform(bad, x);
  note("fft_invalid_status", e.bins.empty() && rdgb::last_status() == RD_EINVAL && !bad.valid());
}

void check_bf() {
  namespace bf = rdgb::bf;
  const unsigned A = par("bf_ant"), B = par("bf_beams"), J = par("bf_binpar"), beats = par("bf_beats");
  const unsigned form = par("bf_form"), beam_par = par("bf_beam_par");
  const std::vector<Complex> w1 = cplx(get<uint32_t>("bf_w")), w2 = cplx(get<uint32_t>("bf_w2"));
  const std::vector<Complex> x = cplx(get<uint32_t>("bf_x"));  // [beat][bin][ant]
  bf::BeamformerModel m(A, B, J, w1, form);
  std::vector<uint32_t> y;
  std::vector<int64_t> acc;
  std::vector<uint8_t> fl;
  std::vector<uint32_t> split;  // per output beat: seq, user, sof, eof, saturating, data...
  bool sat_ok = true;
  for (unsigned t = 0; t < beats; ++t) {
    if (t == beats / 2) m.swap_weights(w2);
    std::vector<std::vector<Complex>> beat(J);
    for (unsigned j = 0; j < J; ++j) {
      const size_t o = (static_cast<size_t>(t) * J + j) * A;
      beat[j].assign(x.begin() + static_cast<long>(o), x.begin() + static_cast<long>(o + A));
    }
    const bf::BeamBeat r = m.step(beat);
    bool any = false;
    for (unsigned b = 0; b < r.n_beams(); ++b)
      for (unsigned j = 0; j < r.n_bins(); ++j) {
        y.push_back(r.y[b][j].packed());
        acc.push_back(r.acc_re[b][j]);
        acc.push_back(r.acc_im[b][j]);
        fl.push_back(static_cast<uint8_t>(r.f_re[b][j].packed() << 2 | r.f_im[b][j].packed()));
        any = any || r.f_re[b][j].any() || r.f_im[b][j].any();
      }
    sat_ok = sat_ok && any == r.saturating;
    for (const bf::OutBeatExp& o : bf::split_beat(r, beam_par, 100u + t, 7u, t == 0, t + 1 == beats)) {
      split.push_back(o.seq);
      split.push_back(o.user);
      split.push_back(o.sof);
      split.push_back(o.eof);
      split.push_back(o.saturating);
      for (const Complex& v : o.data) split.push_back(v.packed());
    }
  }
  note("bf", y.size() == static_cast<size_t>(beats) * B * J && sat_ok);
  put("bf_y", y);
  put("bf_acc", acc);
  put("bf_f", fl);
  put("bf_split", split);
  // the directed weight sets, as the reference builds them
  std::vector<unsigned> sel(B), perm(A);
  for (unsigned b = 0; b < B; ++b) sel[b] = (3u * b + 1u) % A;
  for (unsigned a = 0; a < A; ++a) perm[a] = (a * 5u + 3u) % A;  // a permutation when gcd(5, A) = 1
  put("bf_unit_w", rdgb::fxp::pack(bf::unit_weights(A, B, sel)));
  put("bf_zero_w", rdgb::fxp::pack(bf::zero_weights(A, B)));
  put("bf_max_w", rdgb::fxp::pack(bf::max_weights(A, B)));
  put("bf_perm_w", rdgb::fxp::pack(bf::permute_weights(w1, A, B, perm)));
  // unit weights pass a sample scaled by 0x7FFF, which unit_weight_expect predicts
  bool unit_ok = true;
  const std::vector<bf::DotResult> d = bf::dot_many(std::vector<Complex>(x.begin(), x.begin() + A),
                                                    bf::unit_weights(A, B, sel), A, B, form);
  for (unsigned b = 0; b < B && !d.empty(); ++b)
    unit_ok = unit_ok && d[b].y == bf::unit_weight_expect(x[sel[b] % A]);
  note("bf_unit", !d.empty() && unit_ok);
}

void check_covar() {
  namespace covar = rdgb::covar;
  const std::vector<Complex> x = cplx(get<uint32_t>("cv_x")), y = cplx(get<uint32_t>("cv_y"));
  const std::vector<int64_t> p = covar::power(x);
  std::vector<int64_t> c;
  for (const covar::Cross& e : covar::cross_power(x, y)) {
    c.push_back(e.re);
    c.push_back(e.im);
  }
  note("covar", p.size() == x.size() && c.size() == 2 * x.size() &&
                    covar::power(x[0]) == p[0] && covar::cross_power(x[1], y[1]).re == c[2]);
  put("cv_power", p);
  put("cv_cross", c);
}

void check_cfar_packets() {
  namespace cfar = rdgb::cfar;
  namespace pk = rdgb::packet_model;
  const unsigned n = par("cf_n");
  cfar::Config c;
  c.mode = static_cast<cfar::Mode>(par("cf_mode"));
  c.out_mode = static_cast<cfar::OutMode>(par("cf_out"));
  c.guard_lead = par("cf_gl");
  c.guard_lag = par("cf_gg");
  c.ref_lead = par("cf_rl");
  c.ref_lag = par("cf_rg");
  c.alpha = par("cf_alpha");
  const unsigned mg = par("cf_max_guard"), mr = par("cf_max_ref");
  const std::vector<int64_t> cells = get<int64_t>("cf_cells");
  const std::vector<uint32_t> fid = get<uint32_t>("cf_fid");
  const std::vector<rd_event> raw = cfar::run_frames_raw(cells, n, c, mg, mr, fid);
  // run_frame of frame 0 decodes to the same events as the batched call's first frame
  const std::vector<uint64_t> f0(cells.begin(), cells.begin() + n);
  const std::vector<cfar::Event> one = cfar::run_frame(f0, c, mg, mr, fid[0]);
  bool same = one.size() <= raw.size();
  for (size_t i = 0; same && i < one.size(); ++i) same = one[i] == cfar::decode(raw[i]);
  note("cfar", !raw.empty() && same);
  put("cf_events", raw);
  // the events' detection packets
  const unsigned pw = par("pk_w");
  const std::vector<pk::Flit> fl = pk::detection_packets(raw, pw, par("pk_src"), par("pk_dest"),
                                                         par("pk_vc"), par("pk_seq0"));
  std::vector<uint32_t> words;
  bool parse_ok = fl.size() == raw.size() * pk::detection_flits(pw);
  for (size_t i = 0; i < fl.size(); ++i) {
    words.insert(words.end(), fl[i].w.begin(), fl[i].w.end());
    parse_ok = parse_ok && fl[i].parity_ok();
    if (i % pk::detection_flits(pw) == 0) {  // a header flit
      const pk::Header h = fl[i].header();
      parse_ok = parse_ok && fl[i].sof() && h.src == par("pk_src") && h.dest == par("pk_dest") &&
                 h.length == pk::detection_flits(pw) && pk::hdr_unpack(pk::hdr_pack(h)) == h;
    }
  }
  note("packets", parse_ok);
  put("pk_flits", words);
}

void check_chain() {
  rd_config cfg;
  rd_config_default(&cfg);
  cfg.n_chan = par("ch_chan");
  cfg.n_fft = par("ch_n");
  cfg.taps = par("ch_taps");
  cfg.n_beams = par("ch_beams");
  cfg.cov_window = par("ch_window");
  cfg.guard_lead = cfg.guard_lag = 1;
  cfg.ref_lead = cfg.ref_lag = 4;
  cfg.alpha = 0x800;
  cfg.max_frames = par("ch_max_frames");
  cfg.form = par("ch_form");
  const std::vector<rd_cplx16> coeff = get<uint32_t>("ch_coeff"), w = get<uint32_t>("ch_w");
  const std::vector<rd_cplx16> adc = get<uint32_t>("ch_adc");
  const uint64_t n = adc.size() / cfg.n_chan;
  rdgb::Chain ch(cfg, coeff, w);
  const uint64_t cap = (n / cfg.n_fft) * cfg.n_beams * (cfg.n_fft + 1);
  std::vector<rd_event> ev(cap);
  std::vector<uint32_t> fl(cap * rd_detection_flits(cfg.packet_w) * rd_flit_words(cfg.packet_w));
  const uint32_t nw = static_cast<uint32_t>(n / cfg.n_fft / cfg.cov_window + 2);
  const uint32_t pairs = rd_cov_pairs(&cfg);
  std::vector<rd_cov_window> win(nw);
  std::vector<int64_t> acc(static_cast<size_t>(nw) * cfg.n_fft * pairs * 2);
  rd_output o{};
  o.events = ev.data();
  o.cap_events = cap;
  o.flits = fl.data();
  o.cap_flits = cap * rd_detection_flits(cfg.packet_w);
  o.cov_windows = win.data();
  o.cap_cov_windows = nw;
  o.cov_acc = acc.data();
  const bool ok = ch.valid() && ch.process(adc.data(), n, n, &o) == RD_OK;
  ev.resize(o.n_events);
  fl.resize(o.n_flits * rd_flit_words(cfg.packet_w));
  acc.resize(static_cast<size_t>(o.n_cov_windows) * cfg.n_fft * pairs * 2);
  note("chain", ok && ch.stats().frames == n / cfg.n_fft);
  put("ch_events", ev);
  put("ch_flits", fl);
  put("ch_cov", acc);

  // checkpoint: one chain takes the first half, saves, a new chain loads the
  // state and takes the rest (its events go out for comparison)
  const uint64_t h = (n / cfg.n_fft / 2) * cfg.n_fft;
  rdgb::Chain c1(cfg, coeff, w), c2(cfg, coeff, w);
  std::vector<rd_event> ev2(cap);
  std::vector<uint32_t> fl2(fl.capacity());
  std::vector<rd_cov_window> win2(nw);
  std::vector<int64_t> acc2(static_cast<size_t>(nw) * cfg.n_fft * pairs * 2);
  rd_output o2{};
  o2.events = ev2.data();
  o2.cap_events = cap;
  o2.flits = fl2.data();
  o2.cap_flits = cap * rd_detection_flits(cfg.packet_w);
  o2.cov_windows = win2.data();
  o2.cap_cov_windows = nw;
  o2.cov_acc = acc2.data();
  bool ck = c1.valid() && c2.valid() && c1.process(adc.data(), h, n, &o2) == RD_OK;
  const std::vector<uint8_t> blob = c1.save_state();
  ck = ck && !blob.empty() && c2.load_state(blob) == RD_OK;
  ck = ck && c2.process(adc.data() + h, n - h, n, &o2) == RD_OK;
  ev2.resize(ck ? o2.n_events : 0);
  note("checkpoint", ck && c2.stats().frames == n / cfg.n_fft);
  put("ck_events", ev2);
}

int loaders(int argc, char** argv) {
  for (int i = 3; i < argc; ++i) {
    const std::string base = g_dir + "/" + argv[i];
    std::vector<Complex> coeff;
    rdgb::pfb::CoeffHeader ch;
    std::vector<rdgb::pfb::IoVector> io;
    rdgb::pfb::IoHeader ih;
    std::string err;
    const bool ok = rdgb::pfb::load_coeff(base + ".coeff", &coeff, &ch, &err) &&
                    rdgb::pfb::load_io(base + ".vec", &io, &ih, &err);
    g_status << argv[i] << " " << (ok ? "ok" : "fail") << " " << err << "\n";
    if (!ok) continue;
    std::vector<uint32_t> c = rdgb::fxp::pack(coeff), x, y, f;
    for (const rdgb::pfb::IoVector& v : io) {
      for (const Complex& s : v.x) x.push_back(s.packed());
      for (const Complex& s : v.y) y.push_back(s.packed());
      for (size_t p = 0; p < v.f_re.size(); ++p) f.push_back(v.f_re[p] << 2 | v.f_im[p]);
    }
    std::vector<uint32_t> geo = {ch.phases, ch.taps, ih.phases, ih.taps, ih.acc_w,
                                 static_cast<uint32_t>(io.size())};
    put(std::string(argv[i]) + "_coeff", c);
    put(std::string(argv[i]) + "_x", x);
    put(std::string(argv[i]) + "_y", y);
    put(std::string(argv[i]) + "_f", f);
    put(std::string(argv[i]) + "_geo", geo);
    // a truncated file is an error with a diagnosis, not a short load
    std::ifstream in(base + ".coeff");
    std::ofstream cut(base + "_cut.coeff");
    std::string line;
    for (int k = 0; std::getline(in, line) && k < 20; ++k) cut << line << "\n";
    cut.close();
    const bool refused = !rdgb::pfb::load_coeff(base + "_cut.coeff", &coeff, &ch, &err) && !err.empty();
    g_status << argv[i] << "_truncated " << (refused ? "ok" : "fail") << " " << err << "\n";
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: facade_check loaders|gpu <dir> [names]\n");
    return 2;
  }
  const std::string mode = argv[1];
  g_dir = argv[2];
  g_status.open(g_dir + "/status.txt");
  if (mode == "loaders") return loaders(argc, argv);
  std::ifstream pf(g_dir + "/params.txt");
  std::string k;
  long long v;
  while (pf >> k >> v) g_par[k] = v;
  check_pfb();
  check_fft();
  check_bf();
  check_covar();
  check_cfar_packets();
  check_chain();
  return 0;
}
