"""Scene-level ingest on the GPU: each reference scene file runs through the
chain; the events are the oracle's, bit for bit, and pass the reference's
scene acceptance rule (every target detected within +/-1 bin, false alarms
within 6 per beam)."""
from pathlib import Path

import numpy as np
import pytest

from helpers import CHAIN_KEYS, diff
from rdgb import chain as gc, scene

pytestmark = pytest.mark.gpu

SCENES = sorted((Path(__file__).parent / "golden" / "scenes").glob("*.iq.gz"))


@pytest.mark.parametrize("path", SCENES, ids=lambda p: p.name)
def test_gpu_scene(gpulib, port, path):
    hdr, adc = scene.load_iq(path)
    truth = scene.load_truth(str(path).replace(".iq.gz", ".json"))
    cfg, coeff, w = scene.chain_setup(hdr)
    g = gc.Chain(cfg, coeff, w).process(adc)
    o = port.chain(cfg, coeff, w, np.zeros(0, np.uint32), np.zeros(0, np.uint32)).process(
        adc, taps=False, threads=4)
    assert diff(g, o, CHAIN_KEYS) == []
    rep = scene.check_detections(scene.detect_events(g["events"]), truth["targets"], cfg.n_beams)
    assert rep["passed"], rep


@pytest.mark.parametrize("path", SCENES, ids=lambda p: p.name)
def test_gpu_range_doppler(gpulib, port, path):
    # the slow-time transform of the resident history: bit-exact against the
    # oracle's fft::transform of the same vectors, and every target's peak
    # within one range and one Doppler bin of the ground truth (the
    # reference's range-Doppler check)
    hdr, adc = scene.load_iq(path)
    truth = scene.load_truth(str(path).replace(".iq.gz", ".json"))
    cfg, coeff, w = scene.chain_setup(hdr)
    H = int(hdr["HISTORY_FRAMES"])
    ch = gc.Chain(cfg, coeff, w)
    r = ch.process(adc, taps=True)
    rd, fl = ch.doppler(H)
    spec = r["tap_spectrum"]                      # [F][N][C]
    vec = np.ascontiguousarray(spec[-H:].transpose(2, 1, 0))  # [C][N][H]
    _, bins, sf = port.fft(H, 1, 0xFFFFFFFF, 1, vec.reshape(-1))
    assert np.array_equal(rd.reshape(-1), bins)
    assert np.array_equal(fl.reshape(-1), sf)
    from rdgb import scenario as sc
    re, im = sc.unpack(rd)
    peaks = scene.doppler_peaks(re + 1j * im, truth["targets"])
    assert all(p["passed"] for p in peaks), peaks
