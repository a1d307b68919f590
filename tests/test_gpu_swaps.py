"""Mid-stream coefficient and weight bank swaps on the GPU against the CPU
oracle, bit for bit.

pfb::PfbModel::swap_coeff (pfb_model.hpp:225-233) replaces the coefficient
bank and keeps every lane's delay line, so the next output mixes the new
bank with the old samples; bf::BeamformerModel::swap_weights
(beamformer_model.hpp:271-279) replaces the weight bank from the next step
on. Through the chain that is rd_chain_set_coeff / rd_chain_set_weights
between calls. The swaps below fall between calls of uneven length, inside
covariance windows, off the launch boundaries (the launch size is shorter
than some calls), and change which internal path runs: a small-norm bank
(byte-limb dot products), a bank with an imaginary -32768 (plain int32
multiplies), a full-range random bank (int64 sums), steering weights (int32
beam sums) and full-range random weights (limb-split sums).
"""
import numpy as np
import pytest

from helpers import CHAIN_KEYS, TAP_KEYS, banks, diff, diff_stats, rnd, weight_sets
from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu


CASES = [("tiny", 5, abi.RD_FORM_CUDA_CORE), ("tiny", 5, abi.RD_FORM_TENSOR),
         ("medium", 7, abi.RD_FORM_CUDA_CORE), ("medium", 7, abi.RD_FORM_TENSOR),
         ("full", 3, abi.RD_FORM_CUDA_CORE), ("full", 3, abi.RD_FORM_TENSOR)]


@pytest.mark.parametrize("name,max_frames,form", CASES)
def test_bank_swaps_vs_oracle(gpulib, port, name, max_frames, form):
    rng = np.random.default_rng(10 * len(name) + form)
    p = sc.preset(name, cov_window=6)
    cfg = sc.make_config(p, max_frames=max_frames, form=form)
    px, py = sc.pair_table(p)
    cb, ws = banks(p, rng), weight_sets(p, rng)
    g = gc.Chain(cfg, cb[0], ws[0], (px, py))
    o = port.chain(cfg, cb[0], ws[0], px, py)
    # (frames of the call, coefficient bank before it, weight set before it)
    plan = [(4, None, None), (9, 1, None), (2, None, 1), (max_frames + 2, 2, None),
            (5, 3, 2), (1, 1, 0), (6, None, None)]
    start = 0
    for k, (nf, c, w) in enumerate(plan):
        if c is not None:
            g.set_coeff(cb[c])
            o.set_coeff(cb[c])
        if w is not None:
            g.set_weights(ws[w])
            o.set_weights(ws[w])
        x = sc.adc(p, nf * p.n_fft, start=start * p.n_fft)
        rg = g.process(x, taps=True, cap_events=nf * p.n_beams * (p.n_fft + 1))
        ro = o.process(x, taps=True, threads=8)
        assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == [], (k, nf, c, w)
        start += nf
    assert diff_stats(g.stats(), o.stats()) == []
    fg, fo = g.flush_cov(), o.flush_cov()
    assert diff(fg, fo, ("cov_windows", "cov_acc")) == []


def test_swap_back_restores(gpulib):
    # banks swapped in and straight back out change only the frames computed
    # while they were in: the delay line holds samples, not products, so the
    # next frames' taps equal an unswapped chain's at once
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=16)
    rng = np.random.default_rng(5)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    a, b = gc.Chain(cfg, coeff, w), gc.Chain(cfg, coeff, w)
    x = sc.adc(p, 40 * p.n_fft)
    a.process(x[:, :10 * p.n_fft])
    b.process(x[:, :10 * p.n_fft])
    b.set_coeff(rnd(rng, p.n_fft * p.taps))
    b.set_weights(rnd(rng, p.n_chan * p.n_beams))
    ra, rb = a.process(x[:, 10 * p.n_fft:12 * p.n_fft], taps=True), \
        b.process(x[:, 10 * p.n_fft:12 * p.n_fft], taps=True)
    assert not np.array_equal(ra["tap_power"], rb["tap_power"])
    b.set_coeff(coeff)
    b.set_weights(w)
    ra, rb = a.process(x[:, 12 * p.n_fft:], taps=True), b.process(x[:, 12 * p.n_fft:], taps=True)
    for k in TAP_KEYS:
        assert np.array_equal(ra[k], rb[k]), k
