"""CPU oracle pinning: the plain-C restatement (oracle/orc_port.c) against the
reference's own golden vectors, against chain fixtures produced by the
reference's model headers, and against those headers directly on seeded
random cases. No GPU."""
import numpy as np
import pytest

from conftest import load_chain_fixture
from helpers import (CHAIN_KEYS, TAP_KEYS, accum_replay, banks, cfar_config, cfg_from_fixture,
                     check_delayed, clutter_edge_cells, delayed_input, diff, diff_stats,
                     event_fields, fixture_stats, hadamard_case, orthogonal_pair, rnd, rne15,
                     weight_sets)
from rdgb import abi, scenario as sc
from rdgb.twiddle import DIGEST, TWIDDLES


def test_twiddle_table(port):
    # fft_twiddle_table.hpp:40-43: digest c756048fbc00d64f, axis points exact
    assert DIGEST == "c756048fbc00d64f"
    t = port.twiddles()
    assert np.array_equal(t, np.array(TWIDDLES, np.uint32))
    re, im = sc.unpack(t)
    assert (re[0], im[0]) == (32767, 0)
    assert (re[256], im[256]) == (0, -32768)
    assert (re[512], im[512]) == (-32768, 0)


def test_twiddle_matches_reference(refo):
    assert np.array_equal(refo.twiddles(), np.array(TWIDDLES, np.uint32))


def test_fxp_ops_vectors(port, blockvec):
    z = blockvec
    y, fl = port.fxp(z["fxp_op"], z["fxp_a"], z["fxp_b"], z["fxp_sh"], z["fxp_w"])
    assert len(y) == 1457
    assert np.array_equal(y, z["fxp_y"])
    assert np.array_equal(fl, z["fxp_flags"])


def test_fxp_accum_vectors(port, blockvec):
    # fxp_accum.vec: 19 sequences, 251 steps, widths 16-40, climbs into either
    # rail, recoveries, the acc_w growth policy's edge cases
    z = blockvec
    y, fl, st, ct = accum_replay(port.fxp, z)
    assert len(y) == 251
    assert np.array_equal(y, z["accum_y"])
    assert np.array_equal(fl, z["accum_step_flags"])
    assert np.array_equal(st, z["accum_sticky"])
    assert np.array_equal(ct, z["accum_count"])
    assert (ct > 0).any() and (z["accum_sticky"] == 1).any() and (z["accum_sticky"] == 2).any()


def test_cmult_vectors(port, blockvec):
    z = blockvec
    a, b = z["cmult_a"], z["cmult_b"]
    n = len(a)
    ops = np.concatenate([np.full(n, abi.OP_CODE["cmul_re"]), np.full(n, abi.OP_CODE["cmul_im"])])
    y, fl = port.fxp(ops, np.concatenate([a, a]).astype(np.int64),
                     np.concatenate([b, b]).astype(np.int64), np.zeros(2 * n), np.zeros(2 * n))
    yre, yim = sc.unpack(z["cmult_y"])
    assert np.array_equal(y[:n], yre) and np.array_equal(y[n:], yim)
    assert np.array_equal(fl[:n], z["cmult_f_re"]) and np.array_equal(fl[n:], z["cmult_f_im"])
    # X * conj(Y) with Y = conj(b) is the exact 33-bit product p of cmult.vec
    bre, bim = sc.unpack(b)
    c = port.cross_power(a, sc.pack(bre, -bim)).reshape(n, 2)
    ok = bim != -32768  # conj of -32768j is not representable
    assert np.array_equal(c[ok, 0], z["cmult_p_re"][ok])
    assert np.array_equal(c[ok, 1], z["cmult_p_im"][ok])


def test_fft64_vectors(port, blockvec):
    z = blockvec
    n, spc = int(z["fft_n"]), int(z["fft_spc"])
    for r in range(len(z["fft_sched"])):
        out, _, sf = port.fft(n, spc, int(z["fft_sched"][r]), int(z["fft_reorder"][r]), z["fft_x"][r])
        assert np.array_equal(out, z["fft_y"][r]), f"record {r}"
        assert np.array_equal(sf, z["fft_stage_flags"][r]), f"record {r} flags"


def test_fft_reorder_property(port):
    # test_fft_ref.cpp check 2: reorder on/off relate by bitrev of the beat
    rng = np.random.default_rng(1)
    for n, spc in ((64, 2), (256, 2), (1024, 1), (16, 2), (8, 2)):
        x = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
        o1, b1, _ = port.fft(n, spc, 0xFFFFFFFF, 1, x)
        o0, b0, _ = port.fft(n, spc, 0xFFFFFFFF, 0, x)
        assert np.array_equal(b1, b0)
        m, nl = n // spc, int(np.log2(n // spc))
        for j in range(m):
            src = int(format(j, f"0{nl}b")[::-1], 2)
            assert np.array_equal(o1[j * spc:(j + 1) * spc], o0[src * spc:(src + 1) * spc])


@pytest.mark.parametrize("idx", range(10))
def test_pfb_vectors(port, blockvec, idx):
    z = blockvec
    name = str(z["pfb_sets"][idx])
    P, T = int(z[f"{name}_P"]), int(z[f"{name}_T"])
    x = z[f"{name}_x"]
    y, fl, _ = port.pfb(P, T, z[f"{name}_coeff"], np.zeros((T - 1) * P, np.uint32), x)
    assert np.array_equal(y.reshape(x.shape), z[f"{name}_y"]), name
    assert np.array_equal((fl >> 2).reshape(x.shape), z[f"{name}_f_re"]), name
    assert np.array_equal((fl & 3).reshape(x.shape), z[f"{name}_f_im"]), name


def test_pfb_state_carry(port):
    # two calls with the returned delay line equal one call (swap-free stream)
    rng = np.random.default_rng(2)
    P, T = 8, 16
    c = rng.integers(0, 2**32, size=P * T, dtype=np.uint64).astype(np.uint32)
    x = rng.integers(0, 2**32, size=40 * P, dtype=np.uint64).astype(np.uint32)
    y_all, _, _ = port.pfb(P, T, c, np.zeros((T - 1) * P, np.uint32), x)
    y1, _, st = port.pfb(P, T, c, np.zeros((T - 1) * P, np.uint32), x[:3 * P])
    y2, _, _ = port.pfb(P, T, c, st, x[3 * P:])
    assert np.array_equal(np.concatenate([y1, y2]), y_all)


CHAIN_FIXTURES = ["tiny", "tiny_calls", "ref_tiny", "medium_slice", "tiny_go_dense", "tiny_sat"]


@pytest.mark.parametrize("name", CHAIN_FIXTURES)
def test_port_chain_fixture(port, name):
    z = load_chain_fixture(name)
    cfg = cfg_from_fixture(z)
    ch = port.chain(cfg, z["coeff"], z["weights"], z["px"], z["py"])
    n_fft = cfg.n_fft
    f0 = 0
    for i, nf in enumerate(z["calls"]):
        r = ch.process(z["adc"][:, f0 * n_fft:(f0 + nf) * n_fft], taps=f"c{i}_tap_pfb" in z,
                       threads=4)
        want = {k[len(f"c{i}_"):]: z[k] for k in z.files if k.startswith(f"c{i}_")}
        assert diff(r, want, CHAIN_KEYS + TAP_KEYS) == []
        assert diff_stats(ch.stats(), fixture_stats(z, i)) == []
        f0 += nf
    fl = ch.flush_cov()
    assert np.array_equal(fl["cov_windows"], z["flush_cov_windows"])
    assert np.array_equal(fl["cov_acc"], z["flush_cov_acc"])


def test_port_matches_reference_random(port, refo):
    rng = np.random.default_rng(11)
    for trial in range(4):
        name = ["tiny", "ref_tiny", "tiny", "medium"][trial]
        p = sc.preset(name)
        cfg = sc.make_config(p)
        cfg.cfar_mode = int(rng.integers(0, 2))
        cfg.cfar_out_mode = int(rng.integers(0, 2)) if name != "medium" else 0
        cfg.alpha = int(rng.integers(0, 4096))
        cfg.guard_lead, cfg.guard_lag = (int(v) for v in rng.integers(0, 4, 2))
        cfg.ref_lead, cfg.ref_lag = (int(v) for v in rng.integers(0, 9, 2))
        cfg.scale_sched = int(rng.integers(0, 2**32))
        px, py = sc.pair_table(p)
        coeff = rng.integers(0, 2**32, size=p.n_fft * p.taps, dtype=np.uint64).astype(np.uint32)
        w = rng.integers(0, 2**32, size=p.n_chan * p.n_beams, dtype=np.uint64).astype(np.uint32)
        frames = 20 if name == "medium" else 50
        x = rng.integers(0, 2**32, size=(p.n_chan, frames * p.n_fft), dtype=np.uint64).astype(np.uint32)
        a = port.chain(cfg, coeff, w, px, py)
        b = refo.chain(cfg, coeff, w, px, py)
        ra, rb = a.process(x, taps=True, threads=3), b.process(x, taps=True)
        assert diff(ra, rb, CHAIN_KEYS + TAP_KEYS) == [], trial
        assert diff_stats(a.stats(), b.stats()) == [], trial


def test_history_reads(port, refo):
    p = sc.preset("tiny")
    cfg = sc.make_config(p)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    a = port.chain(cfg, coeff, w, px, py)
    b = refo.chain(cfg, coeff, w, px, py)
    # before any frame: out of range, frame id wraps, zeros
    va, fa, ga = a.read_history(3, 0)
    vb, fb, gb = b.read_history(3, 0)
    assert (np.array_equal(va, vb), fa, ga) == (True, fb, gb)
    x = sc.adc(p, 11 * p.n_fft)
    a.process(x), b.process(x)
    for off in range(0, 10):
        for bin_ in (0, 5, 15, 16, 70000):
            assert [np.asarray(v).tolist() for v in a.read_history(bin_, off)] == \
                   [np.asarray(v).tolist() for v in b.read_history(bin_, off)]
    assert a.stats()["hist_reads"] == b.stats()["hist_reads"]


@pytest.mark.parametrize("case", ["full_slice", "medium_exp_go", "medium_saturating_block"])
def test_port_matches_reference_modes(port, refo, case):
    # the restatement against the reference model's own chain on the full
    # geometry (64 channels, 1024 bins, 64 beams, 2080 pairs, 512-bit packets)
    # and on the covariance and CFAR modes the presets leave at their defaults
    rng = np.random.default_rng(len(case))
    if case == "full_slice":
        p = sc.preset("full", cov_window=2)
        cfg = sc.make_config(p)
        frames = 5
        coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
        x = sc.adc(p, frames * p.n_fft)
    else:
        p = sc.preset("medium", cov_window=7)
        cfg = sc.make_config(p)
        frames = 24
        coeff = sc.coefficients(p.n_fft, p.taps)
        w = rng.integers(0, 2**32, size=p.n_chan * p.n_beams, dtype=np.uint64).astype(np.uint32)
        x = rng.integers(0, 2**32, size=(p.n_chan, frames * p.n_fft),
                         dtype=np.uint64).astype(np.uint32)
        if case == "medium_exp_go":
            cfg.cov_mode, cfg.cov_exp_k, cfg.cov_acc_w = abi.RD_COV_EXP, 3, 40
            cfg.cfar_mode, cfg.cfar_out_mode = abi.RD_CFAR_GO, abi.RD_CFAR_DENSE
        else:  # an unscaled FFT fills the spectrum; 7-frame block sums pass
            cfg.scale_sched = 0  # 33-bit integrators, which saturate
            cfg.cov_acc_w = 33
    px, py = sc.pair_table(p)
    a = port.chain(cfg, coeff, w, px, py)
    b = refo.chain(cfg, coeff, w, px, py)
    ra, rb = a.process(x, taps=True, threads=4), b.process(x, taps=True)
    assert diff(ra, rb, CHAIN_KEYS + TAP_KEYS) == [], case
    assert diff_stats(a.stats(), b.stats()) == [], case
    fa, fb = a.flush_cov(), b.flush_cov()
    assert diff(fa, fb, ("cov_windows", "cov_acc")) == [], case
    if case == "medium_saturating_block":
        assert a.stats()["cov_sat_steps"] > 0


@pytest.mark.parametrize("name", ["tiny", "medium"])
def test_port_matches_reference_bank_swaps(port, refo, name):
    # mid-stream coefficient and weight swaps (pfb_model.hpp:225-233,
    # beamformer_model.hpp:271-279) between calls of uneven length, inside
    # covariance windows: the restatement against the reference's own models
    rng = np.random.default_rng(len(name))
    p = sc.preset(name, cov_window=6)
    cfg = sc.make_config(p, max_frames=7)
    px, py = sc.pair_table(p)
    cb, ws = banks(p, rng), weight_sets(p, rng)
    a = port.chain(cfg, cb[0], ws[0], px, py)
    b = refo.chain(cfg, cb[0], ws[0], px, py)
    start = 0
    for k, (nf, c, w) in enumerate([(4, None, None), (9, 1, None), (2, None, 1), (9, 2, None),
                                    (5, 3, 2), (1, 1, 0), (6, None, None)]):
        for ch in (a, b):
            if c is not None:
                ch.set_coeff(cb[c])
            if w is not None:
                ch.set_weights(ws[w])
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        ra, rb = a.process(x, taps=True, threads=4), b.process(x, taps=True)
        assert diff(ra, rb, CHAIN_KEYS + TAP_KEYS) == [], (name, k)
        start += nf
    assert diff_stats(a.stats(), b.stats()) == []
    fa, fb = a.flush_cov(), b.flush_cov()
    assert diff(fa, fb, ("cov_windows", "cov_acc")) == []


def _depth_script(a, b, p, step_reads):
    """Frames, depth changes and reads applied to two chains alike; every read
    and the statistics after every step must agree."""
    H = p.hist_frames
    start = 0
    for what in (("proc", 11), ("depth", 4), ("read",), ("proc", 1), ("read",), ("proc", 6),
                 ("depth", 1), ("read",), ("proc", 3), ("depth", 2), ("proc", 5),
                 ("depth", H + 9), ("read",), ("proc", 13), ("depth", 0), ("depth", 3),
                 ("proc", 2)):
        if what[0] == "proc":
            x = sc.adc(p, what[1] * p.n_fft, start=start * p.n_fft)
            a.process(x), b.process(x)
            start += what[1]
        elif what[0] == "depth":
            a.set_history_depth(what[1]), b.set_history_depth(what[1])
        step_reads(what)
        assert diff_stats(a.stats(), b.stats()) == [], what


def test_history_depth_changes(port, refo):
    # hist::Model::request_depth (history_model.hpp:260-266, 435-451): the
    # restatement against the reference's own model through depth changes
    # (to 4, 1, 2, above the maximum, 0, 3) between frames - reads right
    # after a change (no frame done: slot 0 as an earlier epoch left it), the
    # epoch, depth and frame counters, collisions and stale flags
    p = sc.preset("tiny")
    cfg = sc.make_config(p)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    a = port.chain(cfg, coeff, w, px, py)
    b = refo.chain(cfg, coeff, w, px, py)

    def reads(_):
        for off in range(0, p.hist_frames + 1):
            for bin_ in (0, 7, p.n_fft - 1):
                assert [np.asarray(v).tolist() for v in a.read_history(bin_, off)] == \
                       [np.asarray(v).tolist() for v in b.read_history(bin_, off)], (bin_, off)

    _depth_script(a, b, p, reads)
    s = a.stats()
    assert (s["hist_depth"], s["hist_epoch"]) == (3, 6)


def _engine_case(case, rng):
    """(preset, config, weights, input) for the beat-stream engine's checks."""
    if case == "tiny":
        p = sc.preset("tiny")
        cfg = sc.make_config(p)
        cfg.engine_pairs = 1
        return p, cfg, sc.steering_weights(p.n_chan, p.n_beams), sc.adc(p, 37 * p.n_fft)
    if case == "medium":
        p = sc.preset("medium")
        cfg = sc.make_config(p)
        cfg.engine_pairs = 5
        return p, cfg, sc.steering_weights(p.n_chan, p.n_beams), sc.adc(p, 9 * p.n_fft)
    # 1024 points, no FFT scaling and full-scale noise put the spectrum at
    # 16-bit full scale; every beam is channel 0 (weight 32767), so a pair's
    # cross power is |x|^2 ~ 2^31 a beat and 1024 beats pass the 40-bit
    # integrators' range; 3 beams make the pair table wrap
    p = sc.preset("full", n_chan=4, n_beams=3, taps=4, cov_source=abi.RD_COV_OFF)
    cfg = sc.make_config(p)
    cfg.scale_sched = 0
    cfg.engine_pairs = 7  # clamped to n_beams / 2 = 1
    w = np.zeros(p.n_beams * p.n_chan, np.uint32)
    w[::p.n_chan] = sc.pack(32767, 0)
    x = rng.integers(0, 2**32, size=(p.n_chan, 6 * p.n_fft), dtype=np.uint64).astype(np.uint32)
    return p, cfg, w, x


@pytest.mark.parametrize("case", ["tiny", "medium", "saturating"])
def test_engine_port_matches_reference(port, refo, case):
    # the RTL's beat-stream covariance engine (covar::Engine run as
    # benchmark_sim_top.sv:1124-1200 wires it, inside the reference-backed
    # oracle) against its restatement in the C oracle: the telemetry after
    # every call of a stream cut into uneven calls
    rng = np.random.default_rng(5)
    p, cfg, w, x = _engine_case(case, rng)
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    a = port.chain(cfg, coeff, w, px, py)
    b = refo.chain(cfg, coeff, w, px, py)
    frames = x.shape[1] // p.n_fft
    cuts = [0] + sorted(rng.choice(np.arange(1, frames), size=min(3, frames - 1),
                                   replace=False).tolist()) + [frames]
    for lo, hi in zip(cuts, cuts[1:]):
        xs = np.ascontiguousarray(x[:, lo * p.n_fft:hi * p.n_fft])
        a.process(xs, taps=False), b.process(xs, taps=False)
        sa, sb = a.stats(), b.stats()
        assert [sa[k] for k in ("engine_window", "engine_samples", "engine_sat")] == \
               [sb[k] for k in ("engine_window", "engine_samples", "engine_sat")], (lo, hi)
        assert diff_stats(sa, sb) == [], (lo, hi)
    s = a.stats()
    beats = frames * p.n_fft // 2
    assert s["engine_samples"] == (p.n_fft if beats >= p.n_fft else 0)
    assert s["engine_window"] == (beats // p.n_fft - 1 if beats >= p.n_fft else 0)
    if case == "saturating":
        assert s["engine_sat"] == 1


@pytest.mark.parametrize("seed", range(4))
def test_depth_and_engine_random_vs_reference(port, refo, seed):
    # random streams through both oracles with the beat-stream engine on
    # (random pair counts, beams and window lengths) and random history depth
    # changes between uneven calls: every read, every counter and the
    # engine's telemetry agree with the reference's own models
    rng = np.random.default_rng(900 + seed)
    name = ["tiny", "ref_tiny", "medium", "tiny"][seed]
    p = sc.preset(name)
    cfg = sc.make_config(p)
    cfg.engine_pairs = int(rng.integers(1, p.n_beams + 3))
    if seed == 3:
        cfg.scale_sched = 0  # unscaled FFT: large beams
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    a = port.chain(cfg, coeff, w, px, py)
    b = refo.chain(cfg, coeff, w, px, py)
    start = 0
    for _ in range(6):
        if rng.integers(0, 2):
            d = int(rng.integers(0, p.hist_frames + 3))
            a.set_history_depth(d), b.set_history_depth(d)
        nf = int(rng.integers(1, 20 if p.n_fft <= 64 else 6))
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        ra, rb = a.process(x, taps=False), b.process(x, taps=False)
        assert diff(ra, rb, CHAIN_KEYS) == []
        assert diff_stats(a.stats(), b.stats()) == []
        for off in (0, 1, p.hist_frames - 1, p.hist_frames + 2):
            assert [np.asarray(v).tolist() for v in a.read_history(3, off)] == \
                   [np.asarray(v).tolist() for v in b.read_history(3, off)], off
        start += nf


# ---- directed and metamorphic cases of the reference's block tests, on the
# oracle (their GPU twins are in test_gpu_blocks.py and test_gpu_chain.py)

def test_hadamard_bank_directed(port):
    # test_beamformer.cpp's orthogonal bank: each input is one bank row, so
    # one beam carries it and the others are exactly zero
    A, frames = 16, 200
    w, x, row, s = hadamard_case(A, frames, np.random.default_rng(21))
    y, _, fl = port.bf(A, A, w, x)
    yr, yi = sc.unpack(y.reshape(frames, A))
    want = np.zeros((frames, A), np.int64)
    want[np.arange(frames), row] = rne15(A * 32767 * s)
    assert np.array_equal(yr, want) and not yi.any() and not fl.any()


def test_cfar_clutter_edge_ca_vs_go(port):
    cells = clutter_edge_cells()
    ca = event_fields(port.cfar(cells, 128, cfar_config(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS,
                                                        2, 2, 8, 8, 384), [0]))
    go = event_fields(port.cfar(cells, 128, cfar_config(abi.RD_CFAR_GO, abi.RD_CFAR_EVENTS,
                                                        2, 2, 8, 8, 384), [0]))
    det_ca = set(ca["bin"][ca["kind"] == 0].tolist())
    assert det_ca and det_ca <= set(range(64, 72))
    assert not (go["kind"] == 0).any()


@pytest.mark.parametrize("mode", [abi.RD_CFAR_CA, abi.RD_CFAR_GO])
def test_cfar_halving_invariance(port, mode):
    # test_pipeline_metamorphic.cpp: exact halving of every cell leaves the
    # detections as they are (the threshold test is homogeneous)
    rng = np.random.default_rng(22 + mode)
    n, frames = 256, 12
    half = rng.integers(0, 4000, frames * n).astype(np.int64)
    half[rng.integers(0, half.size, 60)] *= 30
    cfg = cfar_config(mode, abi.RD_CFAR_DENSE, 2, 3, 8, 12, 900)
    a = event_fields(port.cfar(half, n, cfg, np.arange(frames)))
    b = event_fields(port.cfar(2 * half, n, cfg, np.arange(frames)))
    assert (a["kind"] == 0).sum() > 20
    for k in ("kind", "bin", "frame_id", "ref_cnt", "det", "sup"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(2 * a["cut"], b["cut"]) and np.array_equal(2 * a["sum"], b["sum"])


def test_cross_power_orthogonal(port):
    rng = np.random.default_rng(23)
    x = rnd(rng, 4000)
    re, im = sc.unpack(x)
    x = sc.pack(re, np.where(im == -32768, 0, im))
    c = port.cross_power(x, orthogonal_pair(x)).reshape(-1, 2)
    assert not c[:, 0].any() and np.array_equal(c[:, 1], -port.power(x))


def test_exp_covariance_every_k_vs_reference(port, refo):
    # test_covariance.cpp sweeps the exponential mode's k = 0..15
    p = sc.preset("tiny", cov_window=5)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    px, py = sc.pair_table(p)
    x = sc.adc(p, 40 * p.n_fft)
    for k in range(16):
        cfg = sc.make_config(p)
        cfg.cov_mode, cfg.cov_exp_k, cfg.cov_acc_w = abi.RD_COV_EXP, k, 40
        a, b = port.chain(cfg, coeff, w, px, py), refo.chain(cfg, coeff, w, px, py)
        ra, rb = a.process(x, threads=2), b.process(x)
        assert diff(ra, rb) == [], k
        assert diff_stats(a.stats(), b.stats()) == [], k
        assert diff(a.flush_cov(), b.flush_cov(), ("cov_windows", "cov_acc")) == [], k


def test_delay_invariance(port):
    # test_pipeline_metamorphic.cpp: the input behind zero frames
    p = sc.preset("tiny", cov_window=8)
    cfg = sc.make_config(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    px, py = sc.pair_table(p)
    x = sc.adc(p, 60 * p.n_fft)
    a = port.chain(cfg, coeff, w, px, py).process(x)
    b = port.chain(cfg, coeff, w, px, py).process(delayed_input(x, 16, p.n_fft))
    assert (event_fields(a["events"])["kind"] == 0).any()
    check_delayed(a, b, 16, p.n_beams, 8)
