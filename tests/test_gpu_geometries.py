"""Every geometry the front-end kernel is compiled for, through the chain and
against the CPU oracle, bit for bit.

The front end (PFB + FFT + corner turn) is specialised at compile time per
FFT size and samples per cycle (16/2, 64/2, 64/1, 256/2, 256/1, 1024/2,
1024/1), per tap count (4, 8, 16, and one generic-tap kernel for the others)
and per scaling schedule (every sub-stage halving, or not). Each case below
reaches one of those kernels with the channel counts of the batching workload
(4, 16, 32, 64, and an odd 5 that takes the generic corner-turn path) and
beams = channels, and runs three calls through a chain whose launches are
shorter than some calls and than the PFB delay line:

  * a quiet call (12-bit tones and noise: every pass takes the bound-checked
    path that skips the saturation logic),
  * a loud call (the same samples times 16: passes whose PFB outputs pass
    the bound rerun with the exact saturation and per-sub-stage flags; with
    the first two sub-stages unscaled they saturate),
  * a short quiet call.

Events, packet flits, covariance windows, every tap (PFB output, spectrum,
beams, power) and every statistic must equal the oracle's. The forms
alternate between the CUDA-core and the tensor-core contractions.
"""
import numpy as np
import pytest

from helpers import CHAIN_KEYS, TAP_KEYS, diff, diff_stats
from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu

GEOMS = [(16, 2), (64, 2), (64, 1), (256, 2), (256, 1), (1024, 2), (1024, 1)]
TAPS = [4, 8, 16, 5]        # 5: the generic-tap kernel
CHANS = [4, 16, 32, 64, 5]


def _cases():
    out = []
    k = 0
    for N, spc in GEOMS:
        for T in TAPS:
            for sh1 in ((True, False) if T != 5 else (True,)):
                C = CHANS[k % len(CHANS)]
                if N == 1024 and C == 64 and T == 16:
                    C = 32  # the full workload's own geometry is tested elsewhere
                form = abi.RD_FORM_TENSOR if k % 2 else abi.RD_FORM_CUDA_CORE
                out.append(pytest.param(N, spc, T, sh1, C, form,
                                        id=f"N{N}-spc{spc}-T{T}-{'h' if sh1 else 'x'}-C{C}-f{form}"))
                k += 1
    return out


def _geometry(N, spc, T, C):
    ref = max(2, min(16, N // 8))
    guard = max(1, min(4, N // 64))
    return sc.Preset(f"g{N}_{spc}_{T}_{C}", C, N, T, spc, 8, C, (guard, guard), (ref, ref),
                     guard, ref, 0x0800, abi.RD_COV_CHANNEL, 4, 64, 128, 64 * N, 1, 3, False,
                     300 + N + T + C + spc)


@pytest.mark.parametrize("N,spc,T,sh1,C,form", _cases())
def test_front_geometry_vs_oracle(gpulib, port, N, spc, T, sh1, C, form):
    p = _geometry(N, spc, T, C)
    cfg = sc.make_config(p, max_frames=6, form=form)
    if not sh1:
        # the first two sub-stages do not halve: the schedule is a run-time
        # value, and the loud call saturates them
        cfg.scale_sched = 0xFFFFFFFF & ~3
    px, py = sc.pair_table(p)
    coeff, w = sc.coefficients(N, T), sc.steering_weights(C, C)
    g = gc.Chain(cfg, coeff, w, (px, py))
    o = port.chain(cfg, coeff, w, px, py)
    start = 0
    for nf, loud in ((T + 3, False), (T + 1, True), (3, False)):
        x = sc.adc(p, nf * N, start=start * N)
        if loud:
            re, im = sc.unpack(x)
            x = sc.pack(re * 16, im * 16)
        rg = g.process(x, taps=True, cap_events=nf * C * (N + 1))
        ro = o.process(x, taps=True, threads=8)
        assert diff(rg, ro, CHAIN_KEYS + TAP_KEYS) == [], (nf, loud)
        start += nf
    sg, so = g.stats(), o.stats()
    assert diff_stats(sg, so) == []
    if not sh1:  # the loud call saturated, and the exact path flagged it
        assert any(sg["fft_stage_flags"])
    g.close()
