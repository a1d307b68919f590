"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

from rdgb import abi, scenario as sc

CHAIN_KEYS = ("events", "flits", "cov_windows", "cov_acc")
TAP_KEYS = ("tap_pfb", "tap_spectrum", "tap_beams", "tap_power")
STAT_KEYS = ("frames", "pfb_flags", "pfb_sat_samples", "fft_stage_flags", "bf_flags",
             "bf_sat_samples", "cov_flags", "cov_sat_steps", "hist_frames_done",
             "hist_write_beats", "hist_reads", "hist_collisions", "hist_errors",
             "hist_overwrites", "hist_skew", "align_beats", "align_missing", "align_dup",
             "align_orphan", "align_timeout", "align_fault", "cfar_det", "cfar_sup",
             "cfar_frames", "packets", "flits", "next_seq", "hist_depth", "hist_epoch",
             "engine_window", "engine_samples", "engine_sat")


def cfg_from_fixture(z) -> abi.RdConfig:
    c = abi.RdConfig()
    for name, _ in abi.RdConfig._fields_:
        key = f"cfg_{name}"
        if key in z.files:  # (fields added after a fixture was written stay 0: off)
            setattr(c, name, int(z[key]))
    return c


def diff(a: dict, b: dict, keys=CHAIN_KEYS) -> list[str]:
    bad = []
    for k in keys:
        if k not in a or k not in b:
            continue
        if not np.array_equal(np.asarray(a[k]), np.asarray(b[k])):
            bad.append(k)
    return bad


def diff_stats(a: dict, b: dict) -> list[str]:
    # (the golden fixtures predate hist_depth / hist_epoch: a key one side
    # lacks is not compared)
    return [k for k in STAT_KEYS if k in a and k in b and a[k] != b[k]]


def fixture_stats(z, i: int) -> dict:
    keys = list(z[f"c{i}_stats_keys"])
    vals = list(z[f"c{i}_stats_vals"])
    d = {str(k): int(v) for k, v in zip(keys, vals)}
    d["fft_stage_flags"] = [int(v) for v in z[f"c{i}_fft_stage_flags"]]
    return d


def scenario_inputs(name: str, frames: int, **over):
    p = sc.preset(name, **over)
    cfg = sc.make_config(p, max_frames=over.get("max_frames", None) if False else None)
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, frames * p.n_fft)
    return p, cfg, (px, py), coeff, w, x


def event_fields(ev: np.ndarray) -> dict:
    """Decodes the 176-bit events (cfar_model.hpp:75-84) into columns."""
    w = ev["w"].astype(object)
    v = [int(a) | (int(b) << 64) | (int(c) << 128) for a, b, c in w]

    def f(lsb, n):
        return np.array([(x >> lsb) & ((1 << n) - 1) for x in v], dtype=np.int64)

    return {"kind": f(0, 2), "bin": f(2, 16), "frame_id": f(18, 16), "ref_cnt": f(34, 7),
            "alpha": f(41, 16), "det": f(57, 16), "sup": f(73, 16), "cut": f(89, 40),
            "sum": f(129, 47)}


def accum_replay(fxp, z) -> tuple:
    """Replays the saturating-accumulator sequences of fxp_accum.vec (fxp::Acc,
    fxp.hpp:384-420: wrap-add, then saturate and flag at the accumulator
    width; sticky flags OR'd, a count of flagged steps - the step
    covar::Integrator takes in block mode, covar_model.hpp:204-262) through an
    add-and-saturate primitive `fxp` (the oracle's or the GPU's, the call
    signature of rd_fxp_apply). Every sequence starts from a cleared
    accumulator; step k of all sequences goes in one call. Returns the value,
    step flags, sticky flags and count after every row."""
    seq, step, w, x = z["accum_seq"], z["accum_step"], z["accum_w"], z["accum_x"]
    n = len(x)
    assert all(step[i] == (step[i - 1] + 1 if seq[i] == seq[i - 1] else 0) for i in range(1, n))
    n_seq = len(z["accum_names"])
    acc = np.zeros(n_seq, np.int64)
    sticky = np.zeros(n_seq, np.uint8)
    cnt = np.zeros(n_seq, np.uint32)
    y, fl = np.zeros(n, np.int64), np.zeros(n, np.uint8)
    st, ct = np.zeros(n, np.uint8), np.zeros(n, np.uint32)
    for k in range(int(step.max()) + 1):
        rows = np.nonzero(step == k)[0]
        s = seq[rows]
        op = np.full(len(rows), abi.OP_CODE["add_sat"], np.uint32)
        yk, fk = fxp(op, acc[s], x[rows], np.zeros(len(rows), np.uint32), w[rows])
        acc[s] = yk
        sticky[s] |= fk
        cnt[s] += (fk != 0).astype(np.uint32)  # saturates at 2^32 - 1; never near here
        y[rows], fl[rows], st[rows], ct[rows] = yk, fk, sticky[s], cnt[s]
    return y, fl, st, ct


def rnd(rng, n):
    return rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)


# ---- directed and metamorphic cases of the reference's block tests ---------
# (sim/tests/test_beamformer.cpp, test_cfar.cpp, test_covariance.cpp and
# test_pipeline_metamorphic.cpp name them; the values below are this suite's)

def rne15(v):
    """round_sat(v, 15, 16) with ties to even (fxp.hpp:198-231), |v| < 2^47."""
    v = np.asarray(v, np.int64)
    q, rem = v >> 15, v & 0x7FFF
    return np.clip(q + (rem > 0x4000) + ((rem == 0x4000) & (q & 1)), -32768, 32767)


def hadamard_case(n_ant: int, frames: int, rng) -> tuple:
    """A Sylvester-Hadamard weight bank (real, +-32767; beams = antennas) and
    inputs that are each one bank row times a small s: the row's beam gets
    round_sat(A x 32767 x s, 15, 16) and every other beam exactly 0 (the rows
    are orthogonal and every product is exact). Returns (w, x, row, s)."""
    h = np.array([[1]], np.int64)
    while len(h) < n_ant:
        h = np.block([[h, h], [h, -h]])
    assert len(h) == n_ant
    w = sc.pack((h * 32767).reshape(-1), np.zeros(n_ant * n_ant, np.int64))
    row = rng.integers(0, n_ant, frames)
    s = rng.integers(-400, 401, frames)
    x = sc.pack((h[row] * s[:, None]).reshape(-1), np.zeros(frames * n_ant, np.int64))
    return w, x, row, s


def cfar_config(mode, out, gl, gg, rl, rg, alpha, mg=4, mr=16, enable=1) -> abi.RdConfig:
    c = sc.make_config(sc.preset("tiny"))
    c.cfar_mode, c.cfar_out_mode, c.cfar_enable = mode, out, enable
    c.guard_lead, c.guard_lag, c.ref_lead, c.ref_lag = gl, gg, rl, rg
    c.alpha, c.max_guard, c.max_ref = alpha, mg, mr
    return c


def clutter_edge_cells(n: int = 128, edge: int = 64, lo: int = 100, hi: int = 2000) -> np.ndarray:
    """A clutter step: `lo` below bin `edge`, `hi` from it on. With guard 2,
    reference 8 per side and alpha 1.5, CA-CFAR averages both sides and
    detects the first high cells (their lagging reference cells are low);
    GO-CFAR takes the greater mean (cfar_model.hpp:268-273) and detects
    nothing."""
    c = np.full(n, lo, np.int64)
    c[edge:] = hi
    return c


def delayed_input(x: np.ndarray, frames: int, n_fft: int) -> np.ndarray:
    """The ADC input [C][n] behind `frames` frames of zeros."""
    return np.concatenate([np.zeros((x.shape[0], frames * n_fft), np.uint32), x], axis=1)


def check_delayed(a: dict, b: dict, d: int, n_beams: int, window: int) -> None:
    """Delay invariance (test_pipeline_metamorphic.cpp): `b` is the chain's
    output for its input behind d zero frames, `a` for the input alone. The
    delay line starts at zero, so the zero frames leave no trace: they add
    one CFAR summary event per beam and frame (no detection, cfar_model.hpp
    run_frame) and all-zero covariance windows (d a multiple of the window);
    after them every event and window equals `a`'s with the frame ids, end
    frames and window ids moved on by the delay."""
    fa, fb = event_fields(a["events"]), event_fields(b["events"])
    lead = d * n_beams
    assert len(fb["kind"]) == len(fa["kind"]) + lead
    assert (fb["kind"][:lead] == 3).all() and not fb["det"][:lead].any()
    for k in fa:
        if k != "frame_id":
            assert np.array_equal(fa[k], fb[k][lead:]), k
    assert np.array_equal((fa["frame_id"] + d) & 0xFFFF, fb["frame_id"][lead:])
    assert d % window == 0
    nz = d // window
    assert not b["cov_acc"][:nz].any()
    assert np.array_equal(a["cov_acc"], b["cov_acc"][nz:])
    wa, wb = a["cov_windows"], b["cov_windows"][nz:]
    for k in ("sample_count", "flushed", "truncated", "sat_flags"):
        assert np.array_equal(wa[k], wb[k]), k
    assert np.array_equal(wa["end_frame"] + d, wb["end_frame"])
    assert np.array_equal((wa["window_id"] + nz) & 0xFFFF, wb["window_id"])


def orthogonal_pair(x: np.ndarray) -> np.ndarray:
    """j x for packed {im, re} samples whose imaginary part is not -32768:
    x conj(j x) = -j |x|^2, a cross power with real part 0."""
    re, im = sc.unpack(x)
    assert (im != -32768).all()
    return sc.pack(-im, re)


def banks(p, rng):
    """Coefficient banks that take the PFB's three integer paths: a small-norm
    bank (byte-limb dot products), a full-range random one (int64 sums), one
    holding an imaginary -32768 (int32 multiplies), then the first again."""
    n = p.n_fft * p.taps
    small = sc.coefficients(p.n_fft, p.taps)
    re, im = sc.unpack(sc.coefficients(p.n_fft, p.taps, window="hamming"))
    im[1::p.taps] = -32768  # no int8 high limb for its negation
    re[::p.taps] = 0
    return [small, rnd(rng, n), sc.pack(re, im), small]


def weight_sets(p, rng):
    """Steering weights (int32 beam sums), full-range random weights
    (limb-split sums) and weaker steering weights."""
    return [sc.steering_weights(p.n_chan, p.n_beams), rnd(rng, p.n_chan * p.n_beams),
            sc.steering_weights(p.n_chan, p.n_beams, gain=0.5)]
