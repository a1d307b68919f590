"""The tensor-core form of the beamformer (RD_FORM_TENSOR) on the GPU, through
the C ABI: bit-exact against the CPU oracle and against the CUDA-core form,
per block (bf::dot, beamformer_model.hpp:162-179) and inside the chain
(the committed fixtures made by the reference's model headers, seeded random
chains, the full workload's geometry, one full-size CPI of it). The limb split makes every partial sum
an integer below 2^24, so any difference at all is a bug, not rounding."""
import numpy as np
import pytest

from conftest import load_chain_fixture
from helpers import CHAIN_KEYS, TAP_KEYS, cfg_from_fixture, diff, diff_stats, fixture_stats
from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu
TC = abi.RD_FORM_TENSOR


def rnd(rng, n):
    return rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)


FORMS = [abi.RD_FORM_TENSOR, abi.RD_FORM_TENSOR_WARP]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("A,B", [(1, 1), (4, 2), (16, 16), (64, 64), (5, 3), (63, 17),
                                 (65, 16), (128, 7), (127, 33), (2, 100)])
def test_bf_tensor_random_vs_oracle(gpulib, port, A, B, form):
    rng = np.random.default_rng(7 * A + B)
    w, x = rnd(rng, A * B), rnd(rng, 301 * A)
    want = port.bf(A, B, w, x)
    for a, b in zip(gc.bf(A, B, w, x, form=form), want):
        assert np.array_equal(a, b)
    for a, b in zip(gc.bf(A, B, w, x, form=form), gc.bf(A, B, w, x)):
        assert np.array_equal(a, b)


def test_bf_tensor_repeated_calls(gpulib):
    # many calls in a row, uneven sizes: any ordering gap between the tensor
    # core's writes and the threads' reads would show as a mismatch
    rng = np.random.default_rng(77)
    for it in range(40):
        A = int(rng.choice([4, 16, 33, 64, 128]))
        B = int(rng.integers(1, 70))
        n = int(rng.integers(1, 700))
        w, x = rnd(rng, A * B), rnd(rng, n * A)
        want = gc.bf(A, B, w, x)
        for a, b in zip(gc.bf(A, B, w, x, form=TC), want):
            assert np.array_equal(a, b), (it, A, B, n)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("A", [64, 128])
def test_bf_tensor_extremes(gpulib, port, A, form):
    # every limb at its extreme: -32768 (high limb -128, low 0), 32767
    # (127, 255), -1 (-1, 255), and mixed signs; at 128 channels the class
    # sums come within 0.4 % of 2^24, the most the fp32 accumulation holds
    B = 16
    vals = np.array([-32768, 32767, -1, 0, 255, -256, 128, -129], np.int64)
    rng = np.random.default_rng(11 + A)
    for trial in range(6):
        wr, wi = rng.choice(vals, A * B), rng.choice(vals, A * B)
        xr, xi = rng.choice(vals, 97 * A), rng.choice(vals, 97 * A)
        if trial == 0:
            wr[:] = wi[:] = -32768
            xr[:] = xi[:] = -32768
        if trial == 1:
            wr[:], wi[:] = 32767, -32768
            xr[:], xi[:] = -32768, 32767
        if trial == 2:  # the largest class-8 and class-0 sums: low limbs 255, high -128
            wr[:], wi[:] = -32768 + 255, 32767
            xr[:], xi[:] = -32768 + 255, -32768 + 255
        w, x = sc.pack(wr, wi), sc.pack(xr, xi)
        got, want = gc.bf(A, B, w, x, form=form), port.bf(A, B, w, x)
        for a, b in zip(got, want):
            assert np.array_equal(a, b), trial


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name", ["tiny", "ref_tiny", "medium_slice", "tiny_sat"])
def test_chain_tensor_fixture(gpulib, name, form):
    z = load_chain_fixture(name)
    cfg = cfg_from_fixture(z)
    cfg.form = form
    ch = gc.Chain(cfg, z["coeff"], z["weights"], (z["px"], z["py"]))
    n_fft, f0 = cfg.n_fft, 0
    for i, nf in enumerate(z["calls"]):
        taps = f"c{i}_tap_pfb" in z
        r = ch.process(z["adc"][:, f0 * n_fft:(f0 + nf) * n_fft], taps=taps,
                       cap_events=int(nf) * cfg.n_beams * (n_fft + 1))
        want = {k[len(f"c{i}_"):]: z[k] for k in z.files if k.startswith(f"c{i}_")}
        assert diff(r, want, CHAIN_KEYS + TAP_KEYS) == [], (name, i)
        assert diff_stats(ch.stats(), fixture_stats(z, i)) == [], (name, i)
        f0 += nf


def test_chain_tensor_full_geometry_vs_oracle(gpulib, port):
    # 64 channels, 1024 bins, 64 beams: four beam groups, one channel block
    p = sc.preset("full", cov_window=8)
    cfg = sc.make_config(p, max_frames=12, form=TC)
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 20 * p.n_fft)
    g = gc.Chain(cfg, coeff, w, (px, py))
    rg = g.process(x, taps=True)
    o = port.chain(cfg, coeff, w, px, py)
    ro = o.process(x, taps=True, threads=8)
    assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == []
    assert diff_stats(g.stats(), o.stats()) == []


def test_full_cpi_vs_oracle_both_forms(gpulib, port):
    # one CPI of the full workload at its full size (2^20 samples on each of
    # 64 channels: 1024 frames of 1024 bins, 64 beams, four 256-frame windows
    # of 2080 pairs, 512-bit packets): both forms, in launches of 1024 and of
    # 333 frames, bit-exact against the oracle on the same CPI
    import os

    p = sc.preset("full")
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, p.cpi_samples)
    o = port.chain(sc.make_config(p, max_frames=1024), coeff, w, px, py)
    ro = o.process(x, taps=False, threads=os.cpu_count() or 1)
    assert len(ro["cov_windows"]) == 4 and len(ro["events"]) > 1024 * p.n_beams
    for form, mf in ((abi.RD_FORM_CUDA_CORE, 1024), (TC, 1024), (TC, 333)):
        g = gc.Chain(sc.make_config(p, max_frames=mf, form=form), coeff, w, (px, py))
        rg = g.process(x)
        assert diff(rg, ro) == [], (form, mf)
        assert diff_stats(g.stats(), o.stats()) == [], (form, mf)
        g.close()


def test_full_bench_step_vs_oracle(gpulib, port):
    # the full workload at the bench's launch size: 2 CPIs of 2^20 samples on
    # each of 64 channels (2048 frames of 1024 bins, 64 beams, eight 256-frame
    # windows of 2080 pairs, 512-bit packets) in 1024-frame launches, both
    # forms, through the host-buffer call into page-locked result buffers (the
    # bench's end-to-end path), bit-exact against the oracle on the same input
    import os

    torch = pytest.importorskip("torch")
    p = sc.preset("full")
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, 2 * p.cpi_samples)
    frames = 2 * p.frames_per_cpi
    cap = frames * p.n_beams * (2 + p.n_fft // 16)
    o = port.chain(sc.make_config(p, max_frames=1024), coeff, w, px, py)
    ro = o.process(x, taps=False, threads=os.cpu_count() or 1, cap_events=cap)
    assert len(ro["cov_windows"]) == 8 and len(ro["events"]) > frames * p.n_beams

    def pinned(shape, dtype):
        dt = np.dtype(dtype)
        k = int(np.prod(shape)) * dt.itemsize
        return torch.empty(max(k, 1), dtype=torch.uint8, pin_memory=True).numpy()[:k] \
            .view(dt).reshape(shape)

    for form in (abi.RD_FORM_CUDA_CORE, TC):
        g = gc.Chain(sc.make_config(p, max_frames=1024, form=form), coeff, w, (px, py))
        rg = g.process(x, cap_events=cap, alloc=pinned)
        assert diff(rg, ro) == [], form
        assert diff_stats(g.stats(), o.stats()) == [], form
        g.close()


@pytest.mark.parametrize("seed", range(3))
def test_chain_tensor_equals_cuda_core(gpulib, seed):
    # random weights over the full int16 range and a medium CPI: both forms
    # give identical outputs and statistics
    rng = np.random.default_rng(300 + seed)
    p = sc.preset("medium")
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    w = rnd(rng, p.n_chan * p.n_beams) if seed else sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, p.cpi_samples // 4, start=seed * 1000 * p.n_fft)
    outs = []
    for form in (abi.RD_FORM_CUDA_CORE, TC):
        cfg = sc.make_config(p, max_frames=int(rng.integers(20, 200)), form=form)
        ch = gc.Chain(cfg, coeff, w, (px, py))
        outs.append((ch.process(x, taps=True), ch.stats()))
    assert diff(outs[0][0], outs[1][0], CHAIN_KEYS + TAP_KEYS) == []
    assert diff_stats(outs[0][1], outs[1][1]) == []


def _cov_chain_pair(p, cfg_over, pairs, x, coeff=None, w=None):
    coeff = sc.coefficients(p.n_fft, p.taps) if coeff is None else coeff
    w = sc.steering_weights(p.n_chan, p.n_beams) if w is None else w
    outs = []
    for form in (abi.RD_FORM_CUDA_CORE, TC):
        cfg = sc.make_config(p, max_frames=64, form=form)
        for k, v in cfg_over.items():
            setattr(cfg, k, v)
        ch = gc.Chain(cfg, coeff, w, pairs)
        r = ch.process(x, taps=True)
        outs.append((r, ch.stats(), ch.flush_cov()))
    return outs


@pytest.mark.parametrize("window", [1, 7, 64, 200, 1000])
def test_cov_tensor_windows_and_custom_pairs(gpulib, window):
    # the covariance on the tensor cores against the CUDA-core form: windows
    # shorter and longer than a launch, a pair table with lower-triangle,
    # diagonal and repeated-channel pairs, both sources
    rng = np.random.default_rng(window)
    p = sc.preset("medium")
    x = sc.adc(p, 300 * p.n_fft, start=window * p.n_fft)
    S = p.n_chan
    px = rng.integers(0, S, 40).astype(np.uint32)
    py = rng.integers(0, S, 40).astype(np.uint32)
    keep = np.unique(px * S + py, return_index=True)[1]
    px, py = px[np.sort(keep)], py[np.sort(keep)]
    for src in (abi.RD_COV_CHANNEL, abi.RD_COV_BEAM):
        a, b = _cov_chain_pair(p, {"cov_window": window, "cov_source": src, "cov_acc_w": 64},
                               (px, py), x)
        assert diff(a[0], b[0], CHAIN_KEYS + TAP_KEYS) == [], src
        assert diff_stats(a[1], b[1]) == [], src
        assert diff(a[2], b[2], ("cov_windows", "cov_acc")) == [], src


def test_cov_tensor_saturated_spectrum(gpulib):
    # a full-scale square wave on every channel drives the FFT into
    # saturation, so the covariance sees samples at -32768 and 32767: the
    # largest limb products the 128-frame fp32 accumulation has to hold
    p = sc.preset("full", cov_window=256)
    n = 300 * p.n_fft
    t = np.arange(n)
    sq = np.where((t // 3) % 2 == 0, 32767, -32768)
    x = np.tile(sc.pack(sq, -sq), (p.n_chan, 1))
    px, py = sc.pair_table(p)
    a, b = _cov_chain_pair(p, {"cov_acc_w": 64, "scale_sched": 0}, (px, py), x)
    re, im = sc.unpack(a[0]["tap_spectrum"])
    assert (re == -32768).any() and (im == 32767).any()
    assert diff(a[0], b[0], CHAIN_KEYS + TAP_KEYS) == []
    assert diff_stats(a[1], b[1]) == []
