"""Chain parity on the GPU, through the C ABI: the committed fixtures made by
the reference's own model headers, and the CPU oracle on seeded inputs,
including chunking across launches, multiple calls, device-resident input,
history reads and the covariance flush. Bit-exact."""
import numpy as np
import pytest

from conftest import load_chain_fixture
from helpers import (CHAIN_KEYS, TAP_KEYS, cfg_from_fixture, check_delayed, delayed_input, diff,
                     diff_stats, event_fields, fixture_stats)
from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu

FIXTURES = ["tiny", "tiny_calls", "ref_tiny", "medium_slice", "tiny_go_dense", "tiny_sat"]


@pytest.mark.parametrize("name", FIXTURES)
def test_chain_fixture(gpulib, name):
    z = load_chain_fixture(name)
    cfg = cfg_from_fixture(z)
    ch = gc.Chain(cfg, z["coeff"], z["weights"], (z["px"], z["py"]))
    n_fft = cfg.n_fft
    f0 = 0
    for i, nf in enumerate(z["calls"]):
        taps = f"c{i}_tap_pfb" in z
        r = ch.process(z["adc"][:, f0 * n_fft:(f0 + nf) * n_fft], taps=taps,
                       cap_events=int(nf) * cfg.n_beams * (n_fft + 1))
        want = {k[len(f"c{i}_"):]: z[k] for k in z.files if k.startswith(f"c{i}_")}
        assert diff(r, want, CHAIN_KEYS + TAP_KEYS) == [], (name, i)
        assert diff_stats(ch.stats(), fixture_stats(z, i)) == [], (name, i)
        f0 += nf
    fl = ch.flush_cov()
    assert np.array_equal(fl["cov_windows"], z["flush_cov_windows"])
    assert np.array_equal(fl["cov_acc"], z["flush_cov_acc"])


@pytest.mark.parametrize("name", ["tiny", "ref_tiny"])
def test_history_reads_fixture(gpulib, name):
    z = load_chain_fixture(name)
    cfg = cfg_from_fixture(z)
    ch = gc.Chain(cfg, z["coeff"], z["weights"], (z["px"], z["py"]))
    ch.process(z["adc"])
    p = {"tiny": sc.preset("tiny"), "ref_tiny": sc.preset("ref_tiny")}[name]
    got = [ch.read_history(b, off) for off in range(0, min(p.hist_frames, 6))
           for b in (0, 1, p.n_fft - 1)]
    assert np.array_equal(np.array([g[0] for g in got]), z["hist_vec"])
    assert np.array_equal(np.array([g[1] for g in got], np.uint32), z["hist_fid"])
    assert np.array_equal(np.array([g[2] for g in got], np.uint32), z["hist_flags"])


def _random_cfg(rng, name, max_frames):
    p = sc.preset(name)
    cfg = sc.make_config(p, max_frames=max_frames)
    cfg.cfar_mode = int(rng.integers(0, 2))
    cfg.cfar_out_mode = int(rng.integers(0, 2)) if p.n_fft <= 64 else 0
    cfg.alpha = int(rng.integers(200, 4096))
    cfg.scale_sched = int(rng.integers(0, 2**32)) | 0xFFFFFF00
    cfg.cov_window = int(rng.integers(1, 40))
    if rng.integers(0, 2):
        cfg.cov_mode, cfg.cov_exp_k, cfg.cov_acc_w = abi.RD_COV_EXP, int(rng.integers(0, 16)), 40
    return p, cfg


@pytest.mark.parametrize("seed", range(6))
def test_chain_random_vs_oracle(gpulib, port, seed):
    rng = np.random.default_rng(100 + seed)
    name = ["tiny", "ref_tiny", "tiny", "medium", "ref_tiny", "tiny"][seed]
    p, cfg = _random_cfg(rng, name, max_frames=int(rng.integers(3, 40)))
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps) if seed % 2 else \
        rng.integers(0, 2**32, size=p.n_fft * p.taps, dtype=np.uint64).astype(np.uint32)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)
    start = 0
    for call in range(3):
        nf = int(rng.integers(1, 70 if p.n_fft <= 64 else 25))
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        rg = g.process(x, taps=True, cap_events=nf * p.n_beams * (p.n_fft + 1))
        ro = o.process(x, taps=True, threads=4)
        assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == [], (seed, call)
        assert diff_stats(g.stats(), o.stats()) == [], (seed, call)
        start += nf
    fg, fo = g.flush_cov(), o.flush_cov()
    assert diff(fg, fo, ("cov_windows", "cov_acc")) == []


@pytest.mark.parametrize("name,max_frames,calls", [("medium", 3, (1, 2, 5, 9, 1)),
                                                    ("full", 4, (1, 3, 6, 2))])
def test_chain_short_chunks_delay_line(gpulib, port, name, max_frames, calls):
    # launches shorter than the PFB delay line (taps - 1 frames): the next
    # delay line keeps part of the old one, the rest comes from the chunk
    p = sc.preset(name, cov_window=8)
    cfg = sc.make_config(p, max_frames=max_frames)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)
    start = 0
    for nf in calls:
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        rg = g.process(x, taps=True)
        ro = o.process(x, taps=True, threads=8)
        assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == [], (name, nf)
        start += nf
    assert diff_stats(g.stats(), o.stats()) == []


def _pinned_alloc(torch):
    def alloc(shape, dtype):
        dt = np.dtype(dtype)
        k = int(np.prod(shape)) * dt.itemsize
        a = torch.empty(max(k, 1), dtype=torch.uint8, pin_memory=True).numpy()[:k]
        a[:] = 0xA5  # anything not written by the call shows
        return a.view(dt).reshape(shape)
    return alloc


@pytest.mark.parametrize("window", [16, 100])
def test_process_into_pinned_buffers(gpulib, window):
    # page-locked result buffers fill chunk by chunk while later chunks
    # compute; the results equal the ones read at the end into pageable ones
    torch = pytest.importorskip("torch")
    p = sc.preset("medium", cov_window=window)
    cfg = sc.make_config(p, max_frames=64)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 700 * p.n_fft)
    a, b = gc.Chain(cfg, coeff, w, (px, py)), gc.Chain(cfg, coeff, w, (px, py))
    for lo, hi in ((0, 400), (400, 700)):  # the second call reuses the drain state
        xs = x[:, lo * p.n_fft:hi * p.n_fft]
        want = a.process(xs)
        got = b.process(xs, alloc=_pinned_alloc(torch))
        assert diff(got, want) == [], (lo, hi)
        assert len(want["events"]) > 1000 and len(want["cov_windows"]) >= 2


def test_fetch_after_pinned_process(gpulib):
    # results copied chunk by chunk into one call's page-locked buffers are
    # read again in full by a later fetch into other buffers
    torch = pytest.importorskip("torch")
    p = sc.preset("medium", cov_window=32)
    cfg = sc.make_config(p, max_frames=64)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 300 * p.n_fft)
    ch = gc.Chain(cfg, coeff, w, (px, py))
    first = ch.process(x, alloc=_pinned_alloc(torch))
    again = ch.fetch(300)
    assert diff(again, first) == []


def test_process_into_pinned_buffers_truncated(gpulib):
    # an event capacity below the call's events: both buffers keep the first
    # cap events and packets, and the call reports the truncation
    torch = pytest.importorskip("torch")
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=64)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = gc._u32(sc.adc(p, 300 * p.n_fft))
    outs = []
    for alloc in (np.zeros, _pinned_alloc(torch)):
        ch = gc.Chain(cfg, coeff, w, (px, py))
        o = gc.Outputs(cfg, 300, ch.n_pairs, False, 777, alloc=alloc)
        st = ch.L.rd_chain_process(ch.h, gc.ptr(x), x.shape[1], x.shape[1], gc.C.byref(o.c))
        assert st == abi.RD_ETRUNC
        outs.append(o)
    a, b = outs
    assert a.c.n_events == b.c.n_events > 777
    assert np.array_equal(a.events[:777], b.events[:777])
    nfl = len(a.flits) // 777
    assert np.array_equal(a.flits[:777 * nfl], b.flits[:777 * nfl])


@pytest.mark.parametrize("extreme", [False, True])
def test_pfb_small_bank_paths(gpulib, port, extreme):
    # a bank whose phase norms keep the PFB sums in int32 runs the byte-limb
    # dot products; one holding an imaginary -32768 (its negation has no int8
    # high limb) runs the plain int32 multiplies - both bit-exact
    rng = np.random.default_rng(31 + extreme)
    p = sc.preset("medium")
    re = rng.integers(-800, 800, p.n_fft * p.taps)
    im = rng.integers(-800, 800, p.n_fft * p.taps)
    re[::p.taps] = 16000
    im[1::p.taps] = -32768 if extreme else -32767
    re[2::p.taps], im[2::p.taps] = 0, 0
    l1 = (np.abs(re) + np.abs(im)).reshape(p.n_fft, p.taps).sum(1).max()
    assert l1 <= 65535  # the int32 PFB sums hold
    coeff = sc.pack(re, im)
    cfg = sc.make_config(p, max_frames=40)
    px, py = sc.pair_table(p)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 90 * p.n_fft)
    rg = gc.Chain(cfg, coeff, w, (px, py)).process(x, taps=True)
    ro = port.chain(cfg, coeff, w, px, py).process(x, taps=True, threads=8)
    assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == []


@pytest.mark.parametrize("packet_w", [64, 96, 128, 160, 256, 480, 512])
def test_chain_packet_widths(gpulib, port, packet_w):
    # the CFAR emit's packet layouts: fixed at compile time for 64/128/256/512,
    # computed at run time for the other widths - the same flits as the model
    p = sc.preset("tiny")
    cfg = sc.make_config(p, max_frames=16)
    cfg.packet_w = packet_w
    cfg.src_id, cfg.dest, cfg.vc = 5, 9, 2
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 60 * p.n_fft)
    rg = gc.Chain(cfg, coeff, w, (px, py)).process(x)
    ro = port.chain(cfg, coeff, w, px, py).process(x, taps=False, threads=4)
    assert diff(rg, ro) == []
    assert len(rg["flits"]) == len(rg["events"]) * (1 + -(-176 // packet_w))


def test_chain_medium_cpi_vs_oracle(gpulib, port):
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=100)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, p.cpi_samples)
    rg = gc.Chain(cfg, coeff, w, (px, py)).process(x)
    ro = port.chain(cfg, coeff, w, px, py).process(x, taps=False, threads=8)
    assert diff(rg, ro) == []
    assert len(rg["cov_windows"]) == 1 and rg["cov_windows"][0]["sample_count"] == 256
    assert (event_fields(rg["events"][:50])["alpha"] == p.alpha).all()


def test_medium_bench_step_vs_oracle(gpulib, port):
    # the medium workload at the bench's size: 64 CPIs of 65536 samples on
    # each of 16 channels (16384 frames, 64 covariance windows, 1.3 M events)
    # in the bench's 1024-frame launches, bit-exact against the oracle
    import os

    p = sc.preset("medium")
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 64 * p.cpi_samples)
    g = gc.Chain(sc.make_config(p, max_frames=1024), coeff, w, (px, py))
    rg = g.process(x)
    o = port.chain(sc.make_config(p, max_frames=1024), coeff, w, px, py)
    ro = o.process(x, taps=False, threads=os.cpu_count() or 1)
    assert len(rg["cov_windows"]) == 64 and len(rg["events"]) > 16384 * p.n_beams
    assert diff(rg, ro) == []
    assert diff_stats(g.stats(), o.stats()) == []


def test_chain_full_geometry_slice_vs_oracle(gpulib, port):
    # the full workload's geometry (64 ch, 1024-point PFB x 16 taps, 64 beams,
    # 2080 covariance pairs), 20 frames with an 8-frame window
    p = sc.preset("full", cov_window=8)
    cfg = sc.make_config(p, max_frames=12)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 20 * p.n_fft)
    g = gc.Chain(cfg, coeff, w, (px, py))
    rg = g.process(x, taps=True)
    o = port.chain(cfg, coeff, w, px, py)
    ro = o.process(x, taps=True, threads=8)
    assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == []
    assert diff_stats(g.stats(), o.stats()) == []


def test_device_input_and_chunking_invariance(gpulib):
    torch = pytest.importorskip("torch")
    p = sc.preset("medium")
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    n = 2 * p.cpi_samples
    x = sc.adc(p, n)
    d = torch.from_numpy(x.view(np.int32)).cuda()
    results = []
    for mf in (512, 100, 37):
        cfg = sc.make_config(p, max_frames=mf)
        ch = gc.Chain(cfg, coeff, w, (px, py))
        ch.process_device(d.data_ptr(), n, n, torch.cuda.current_stream().cuda_stream)
        results.append((ch.fetch(n // p.n_fft), ch.stats()))
        ch.close()
    host = gc.Chain(sc.make_config(p, max_frames=512), coeff, w, (px, py)).process(x)
    for r, st in results:
        assert diff(r, host) == []
        assert diff_stats(st, results[0][1]) == []


def test_zero_input(gpulib):
    p = sc.preset("tiny")
    cfg = sc.make_config(p)
    px, py = sc.pair_table(p)
    ch = gc.Chain(cfg, sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams),
                  (px, py))
    r = ch.process(np.zeros((p.n_chan, 64 * p.n_fft), np.uint32), taps=True)
    assert not r["tap_power"].any() and not r["tap_spectrum"].any()
    f = event_fields(r["events"])
    assert (f["kind"] == 3).all() and len(r["events"]) == 64 * p.n_beams
    assert not r["cov_acc"].any() if len(r["cov_acc"]) else True


def test_empty_call_and_bad_sizes(gpulib):
    p = sc.preset("tiny")
    cfg = sc.make_config(p)
    ch = gc.Chain(cfg, sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams))
    r = ch.process(np.zeros((p.n_chan, 0), np.uint32))
    assert r["n_frames"] == 0 and len(r["events"]) == 0
    with pytest.raises(RuntimeError, match="RD_EINVAL"):
        ch.process(np.zeros((p.n_chan, p.n_fft + 3), np.uint32))


def test_event_truncation_reports(gpulib, port):
    p = sc.preset("tiny")
    cfg = sc.make_config(p)
    cfg.cfar_out_mode = abi.RD_CFAR_DENSE
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 10 * p.n_fft)
    ch = gc.Chain(cfg, coeff, w, (px, py))
    with pytest.raises(RuntimeError, match="RD_ETRUNC"):
        ch.process(x, cap_events=5)


@pytest.mark.parametrize("name,split,rest", [("tiny", 37, 50), ("medium", 45, 70)])
def test_checkpoint_resume(gpulib, port, name, split, rest):
    # a stream saved after `split` frames (inside a covariance window, with
    # the delay line and history full) and restored into a new chain of the
    # same configuration continues bit for bit: the next call's events,
    # packets, windows and counters equal the oracle's uninterrupted stream,
    # and so do the history reads and the Doppler map of the restored ring
    p = sc.preset(name, cov_window=16)
    cfg = sc.make_config(p, max_frames=32)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    o = port.chain(cfg, coeff, w, px, py)
    x1 = sc.adc(p, split * p.n_fft)
    x2 = sc.adc(p, rest * p.n_fft, start=split * p.n_fft)
    o.process(x1, taps=False, threads=8)
    want = o.process(x2, taps=False, threads=8)
    a = gc.Chain(cfg, coeff, w, (px, py))
    a.process(x1)
    blob = a.save_state()
    assert len(blob) == gpulib.rd_chain_state_size(a.h)
    a.close()
    b = gc.Chain(cfg, coeff, w, (px, py))
    b.load_state(blob)
    got = b.process(x2)
    assert diff(got, want, CHAIN_KEYS) == []
    assert diff_stats(b.stats(), o.stats()) == []
    # the restored ring: the history reads and the Doppler map equal a
    # stream that never stopped
    c = gc.Chain(cfg, coeff, w, (px, py))
    c.process(x1)
    c.process(x2)
    H = cfg.hist_frames
    for bin_, off in ((0, 0), (p.n_fft - 1, 1), (3, H - 3)):
        vb, vc = b.read_history(bin_, off), c.read_history(bin_, off)
        assert all(np.array_equal(u, v) if isinstance(u, np.ndarray) else u == v
                   for u, v in zip(vb, vc)), (bin_, off)
    db, dc = b.doppler(H), c.doppler(H)
    assert np.array_equal(db[0], dc[0]) and np.array_equal(db[1], dc[1])
    # a blob of another configuration, or cut short, is refused
    cfg2 = sc.make_config(p, max_frames=16)
    d = gc.Chain(cfg2, coeff, w, (px, py))
    assert gpulib.rd_chain_load_state(d.h, blob, len(blob)) == abi.RD_EINVAL
    assert gpulib.rd_chain_load_state(b.h, blob, len(blob) - 1) == abi.RD_EINVAL
    bad = bytearray(blob)
    bad[0] ^= 1
    assert gpulib.rd_chain_load_state(b.h, bytes(bad), len(bad)) == abi.RD_EINVAL
    small = (gc.C.c_char * 16)()
    assert gpulib.rd_chain_save_state(b.h, small, 16) == abi.RD_EINVAL
    for ch in (b, c, d):
        ch.close()


def test_history_depth_changes(gpulib, port):
    # rd_chain_set_history_depth against the oracle (which the reference's
    # own history model pins, tests/test_oracle.py): depth changes between
    # calls, reads right after a change and after new frames, the counters,
    # the epoch; and every call's events and windows unchanged by them
    from test_oracle import _depth_script
    p = sc.preset("tiny")
    cfg = sc.make_config(p, max_frames=8)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)

    def reads(_):
        for off in range(0, p.hist_frames + 1):
            for bin_ in (0, 7, p.n_fft - 1):
                vg, fg, lg = g.read_history(bin_, off)
                vo, fo, lo = o.read_history(bin_, off)
                assert (np.array_equal(vg, vo), fg, lg) == (True, fo, lo), (bin_, off)

    _depth_script(g, o, p, reads)
    assert g.stats()["hist_epoch"] == 6
    # a reset returns the depth a new chain has
    g.L.rd_chain_reset(g.h, None)
    s = g.stats()
    assert (s["hist_depth"], s["hist_epoch"], s["hist_frames_done"]) == (p.hist_frames, 0, 0)
    g.close()


@pytest.mark.parametrize("case,form", [("tiny", abi.RD_FORM_CUDA_CORE),
                                       ("medium", abi.RD_FORM_CUDA_CORE),
                                       ("medium", abi.RD_FORM_TENSOR),
                                       ("saturating", abi.RD_FORM_CUDA_CORE)])
def test_beat_stream_engine(gpulib, port, case, form):
    # the RTL's beat-stream covariance engine against the oracle (pinned to
    # the reference's covar::Engine, tests/test_oracle.py) over a stream cut
    # into uneven calls and launches: pair 0's last window id and count and
    # the saturation flag after every call, the chain's own outputs unchanged;
    # then a checkpoint inside an open engine window resumes exactly
    from test_oracle import _engine_case
    rng = np.random.default_rng(5)
    p, cfg, w, x = _engine_case(case, rng)
    cfg.form = form
    cfg.max_frames = 3
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)
    frames = x.shape[1] // p.n_fft
    cuts = [0] + sorted(rng.choice(np.arange(1, frames), size=min(3, frames - 1),
                                   replace=False).tolist()) + [frames]
    keys = ("engine_window", "engine_samples", "engine_sat")
    for lo, hi in zip(cuts, cuts[1:]):
        xs = np.ascontiguousarray(x[:, lo * p.n_fft:hi * p.n_fft])
        rg, ro = g.process(xs), o.process(xs, taps=False, threads=8)
        assert diff(rg, ro, CHAIN_KEYS) == [], (lo, hi)
        sg, so = g.stats(), o.stats()
        assert [sg[k] for k in keys] == [so[k] for k in keys], (lo, hi)
        assert diff_stats(sg, so) == [], (lo, hi)
    if case == "saturating":
        assert g.stats()["engine_sat"] == 1
    # a checkpoint with an engine window open carries its accumulators
    g2 = gc.Chain(cfg, coeff, w, (px, py))
    o2 = port.chain(cfg, coeff, w, px, py)
    half = max(1, frames // 2)
    if (half * p.n_fft // 2) % p.n_fft == 0 and frames > half + 1:
        half += 1  # inside a window
    x1, x2 = np.ascontiguousarray(x[:, :half * p.n_fft]), np.ascontiguousarray(x[:, half * p.n_fft:])
    g2.process(x1), o2.process(x1, taps=False, threads=8)
    blob = g2.save_state()
    g3 = gc.Chain(cfg, coeff, w, (px, py))
    g3.load_state(blob)
    g3.process(x2), o2.process(x2, taps=False, threads=8)
    assert diff_stats(g3.stats(), o2.stats()) == []
    for ch in (g, g2, g3):
        ch.close()


@pytest.mark.parametrize("seed", range(4))
def test_depth_and_engine_random(gpulib, port, seed):
    # the random streams of test_oracle.py's reference check, on the GPU:
    # engine on, depth changes between uneven calls and launches, both forms
    rng = np.random.default_rng(900 + seed)
    name = ["tiny", "ref_tiny", "medium", "tiny"][seed]
    p = sc.preset(name)
    cfg = sc.make_config(p, max_frames=int(rng.integers(2, 9)),
                         form=abi.RD_FORM_TENSOR if seed == 2 else abi.RD_FORM_CUDA_CORE)
    cfg.engine_pairs = int(rng.integers(1, p.n_beams + 3))
    if seed == 3:
        cfg.scale_sched = 0
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)
    start = 0
    for _ in range(6):
        if rng.integers(0, 2):
            d = int(rng.integers(0, p.hist_frames + 3))
            g.set_history_depth(d), o.set_history_depth(d)
        nf = int(rng.integers(1, 20 if p.n_fft <= 64 else 6))
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        rg, ro = g.process(x), o.process(x, taps=False, threads=4)
        assert diff(rg, ro, CHAIN_KEYS) == []
        assert diff_stats(g.stats(), o.stats()) == []
        for off in (0, 1, p.hist_frames - 1, p.hist_frames + 2):
            vg, fg, lg = g.read_history(3, off)
            vo, fo, lo = o.read_history(3, off)
            assert (np.array_equal(vg, vo), fg, lg) == (True, fo, lo), off
        start += nf
    g.close()


@pytest.mark.parametrize("form", [abi.RD_FORM_CUDA_CORE, abi.RD_FORM_TENSOR])
def test_exp_covariance_every_k(gpulib, port, form):
    # the exponential covariance mode at every k = 0..15 (test_covariance.cpp
    # sweeps them), in two calls, against the oracle
    p = sc.preset("tiny", cov_window=5)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    px, py = sc.pair_table(p)
    x = sc.adc(p, 40 * p.n_fft)
    for k in range(16):
        cfg = sc.make_config(p, max_frames=16, form=form)
        cfg.cov_mode, cfg.cov_exp_k, cfg.cov_acc_w = abi.RD_COV_EXP, k, 40
        g, o = gc.Chain(cfg, coeff, w, (px, py)), port.chain(cfg, coeff, w, px, py)
        for lo, hi in ((0, 17), (17, 40)):
            xs = x[:, lo * p.n_fft:hi * p.n_fft]
            assert diff(g.process(xs), o.process(xs, threads=2)) == [], (k, lo)
            assert diff_stats(g.stats(), o.stats()) == [], (k, lo)
        assert diff(g.flush_cov(), o.flush_cov(), ("cov_windows", "cov_acc")) == [], k


def _run_calls(ch, x, n_fft, calls):
    """Runs x in calls of the given frame counts; the outputs concatenated."""
    outs, f0 = [], 0
    for nf in calls:
        outs.append(ch.process(x[:, f0 * n_fft:(f0 + nf) * n_fft]))
        f0 += nf
    assert f0 * n_fft == x.shape[1]
    return {k: np.concatenate([o[k] for o in outs]) for k in ("events", "cov_windows", "cov_acc")}


@pytest.mark.parametrize("name,form,calls", [("tiny", abi.RD_FORM_CUDA_CORE, (7, 30, 19)),
                                             ("medium", abi.RD_FORM_TENSOR, (5, 29, 22))])
def test_delay_invariance(gpulib, port, name, form, calls):
    # test_pipeline_metamorphic.cpp: the input behind 16 zero frames, run in
    # uneven calls over short launches, leaves every output as it was
    p = sc.preset(name, cov_window=8)
    cfg = sc.make_config(p, max_frames=12, form=form)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    px, py = sc.pair_table(p)
    x = sc.adc(p, 40 * p.n_fft)
    xd = delayed_input(x, 16, p.n_fft)
    a = gc.Chain(cfg, coeff, w, (px, py)).process(x)
    b = _run_calls(gc.Chain(cfg, coeff, w, (px, py)), xd, p.n_fft, calls)
    assert (event_fields(a["events"])["kind"] == 0).any()
    check_delayed(a, b, 16, p.n_beams, 8)
    o = port.chain(cfg, coeff, w, px, py).process(xd, threads=2)
    assert diff(b, o, ("events", "cov_windows", "cov_acc")) == []
