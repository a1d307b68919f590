"""Scene-level ingest on the CPU: the iq_ascii_v1 loader on the scene files
the reference's generator wrote (tests/golden/make_scenes.py), its round trip
and its framing checks, and the reference's scene acceptance rule on the
oracle's events."""
import gzip
from pathlib import Path

import numpy as np
import pytest

from rdgb import scene
from rdgb import scenario as sc

SCENES = sorted((Path(__file__).parent / "golden" / "scenes").glob("*.iq.gz"))


def test_scenes_present():
    assert {p.name for p in SCENES} == {"three_targets_seed1.iq.gz",
                                        "three_targets_even_seed1.iq.gz",
                                        "mixed_parity_seed1.iq.gz"}


@pytest.mark.parametrize("path", SCENES, ids=lambda p: p.name)
def test_load_iq_fixture(path):
    hdr, adc = scene.load_iq(path)
    assert (hdr["FFT_SIZE"], hdr["N_ANTENNAS"], hdr["HISTORY_FRAMES"]) == ("256", "4", "16")
    assert adc.shape == (4, 16 * 256) and adc.dtype == np.uint32
    re, im = sc.unpack(adc)
    assert np.abs(im).max() > 100  # signal, not zeros
    truth = scene.load_truth(str(path).replace(".iq.gz", ".json"))
    assert truth["iq_format"] == "iq_ascii_v1" and len(truth["targets"]) >= 3


def test_write_load_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    adc = rng.integers(0, 2**32, size=(3, 5 * 64), dtype=np.uint64).astype(np.uint32)
    p = tmp_path / "x.iq.gz"
    scene.write_iq(p, adc, 64, 2, {"seed": 3})
    hdr, back = scene.load_iq(p)
    assert hdr["seed"] == "3" and np.array_equal(back, adc)


def test_framing_and_row_count_are_checked(tmp_path):
    adc = np.zeros((2, 2 * 16), np.uint32)
    p = tmp_path / "ok.iq"
    scene.write_iq(p, adc, 16, 2)
    lines = p.read_text().splitlines()
    bad = [ln for ln in lines]
    i = next(k for k, ln in enumerate(bad) if not ln.startswith("#"))
    t = bad[i].split()
    t[3] = "0"  # beat 0 without sof
    bad[i] = " ".join(t)
    (tmp_path / "sof.iq").write_text("\n".join(bad) + "\n")
    with pytest.raises(ValueError, match="framing"):
        scene.load_iq(tmp_path / "sof.iq")
    (tmp_path / "short.iq").write_text("\n".join(lines[:-1]) + "\n")
    with pytest.raises(ValueError, match="beat rows"):
        scene.load_iq(tmp_path / "short.iq")
    hdrless = [ln for ln in lines if "FFT_SIZE" not in ln]
    (tmp_path / "hdr.iq").write_text("\n".join(hdrless) + "\n")
    with pytest.raises(ValueError, match="FFT_SIZE"):
        scene.load_iq(tmp_path / "hdr.iq")


def test_check_detections_rule():
    t = [{"range_bin": 10}, {"range_bin": 50}]
    rep = scene.check_detections([(0, 0, 11), (3, 1, 49), (2, 0, 30)], t, n_beams=1,
                                 fa_per_beam=1)
    assert rep["detected"] == 2 and rep["false_alarms"] == 1 and rep["passed"]
    rep = scene.check_detections([(0, 0, 12)], t, n_beams=1)
    assert rep["missed"] == 2 and not rep["passed"]


@pytest.mark.parametrize("path", SCENES, ids=lambda p: p.name)
def test_oracle_scene_acceptance(path, port):
    # the reference's acceptance rule on the chain's events (the oracle's;
    # the GPU test checks the GPU's events equal these)
    hdr, adc = scene.load_iq(path)
    truth = scene.load_truth(str(path).replace(".iq.gz", ".json"))
    cfg, coeff, w = scene.chain_setup(hdr)
    r = port.chain(cfg, coeff, w, np.zeros(0, np.uint32), np.zeros(0, np.uint32)).process(
        adc, taps=False, threads=4)
    rep = scene.check_detections(scene.detect_events(r["events"]), truth["targets"], cfg.n_beams)
    assert rep["passed"], rep
    assert all(n >= 1 for n in rep["per_target"])
