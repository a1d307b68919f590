"""Scene-level ingest: the reference's ``iq_ascii_v1`` scenario files and
their ground truth, run through the chain, checked against the targets.

The file format is the one the reference's scene generator writes
(model/python/gen_target_iq.py:520-618) and its loaders read
(model/python/range_doppler.py:111-176, sim/verilator/harness/iq_loader.h):
a ``# key: value`` header, then one line per (frame, antenna, beat)

    frame antenna beat sof eof s0_re s0_im s1_re s1_im ...

with SAMPLES_PER_CYCLE Q1.15 pairs per line, frames of FFT_SIZE fast-time
samples. ``load_iq`` returns the samples as the chain's ADC input
(``[antenna][frame * FFT_SIZE + n]``, packed ``{im, re}``), checking the row
count and the sof/eof framing as the reference loader does.

``check_detections`` is the acceptance rule of the reference's scene test
(sim/tests/test_pipeline_scenario.cpp:104-258): a target is detected when
any frame of any beam produced a DETECT event within ``bin_tol`` of its range
bin; every DETECT outside all target windows is a false alarm, at most
``fa_per_beam`` per beam over the run. The chain runs CFAR on every bin of
every beam, so the expected CFAR bin is the FFT bin itself.
"""
from __future__ import annotations

import gzip
import json
import math
import re
from pathlib import Path

import numpy as np

from . import abi
from .scenario import pack

_KV = re.compile(r"([A-Za-z_][A-Za-z0-9_]*)\s*:\s*(.*)")


def _open(path: Path):
    path = Path(path)
    if path.suffix == ".gz":
        return gzip.open(path, "rt", encoding="utf-8")
    return path.open("r", encoding="utf-8")


def load_iq(path) -> tuple[dict, np.ndarray]:
    """(header, adc): adc is uint32 [N_ANTENNAS][HISTORY_FRAMES * FFT_SIZE]."""
    hdr: dict = {}
    rows = []
    with _open(path) as fh:
        for line in fh:
            s = line.strip()
            if not s:
                continue
            if s.startswith("#"):
                m = _KV.match(s.lstrip("#").strip())
                if m and m.group(1) not in hdr:
                    hdr[m.group(1)] = m.group(2).strip()
                continue
            rows.append(s)
    for key in ("FFT_SIZE", "HISTORY_FRAMES", "N_ANTENNAS", "SAMPLES_PER_CYCLE"):
        if key not in hdr:
            raise ValueError(f"IQ header missing key '{key}': {path}")
    n, h = int(hdr["FFT_SIZE"]), int(hdr["HISTORY_FRAMES"])
    a, p = int(hdr["N_ANTENNAS"]), int(hdr["SAMPLES_PER_CYCLE"])
    beats = n // p
    if len(rows) != h * a * beats:
        raise ValueError(f"IQ has {len(rows)} beat rows, expected {h * a * beats} "
                         f"({h} frames * {a} antennas * {beats} beats)")
    tab = np.array([r.split() for r in rows], dtype=np.int64)
    if tab.shape[1] != 5 + 2 * p:
        raise ValueError(f"IQ rows carry {(tab.shape[1] - 5) / 2} samples, expected {p}")
    f, ant, beat, sof, eof = tab[:, 0], tab[:, 1], tab[:, 2], tab[:, 3], tab[:, 4]
    bad = (sof != (beat == 0)) | (eof != (beat == beats - 1))
    if bad.any():
        i = int(np.argmax(bad))
        raise ValueError(f"IQ framing mismatch at frame {f[i]} antenna {ant[i]} beat {beat[i]}")
    if ((f < 0) | (f >= h) | (ant < 0) | (ant >= a) | (beat < 0) | (beat >= beats)).any():
        raise ValueError("IQ row index out of range")
    re_i = np.zeros((a, h * n), np.int64)
    im_i = np.zeros((a, h * n), np.int64)
    for slot in range(p):
        col = f * n + beat * p + slot
        re_i[ant, col] = tab[:, 5 + 2 * slot]
        im_i[ant, col] = tab[:, 6 + 2 * slot]
    return hdr, pack(re_i, im_i)


def write_iq(path, adc: np.ndarray, n_fft: int, spc: int, extra: dict | None = None) -> None:
    """The inverse of load_iq for [antenna][frame * n_fft + n] samples."""
    a, total = adc.shape
    h = total // n_fft
    re_i = (adc & 0xFFFF).astype(np.int64)
    re_i = np.where(re_i >= 0x8000, re_i - 0x10000, re_i)
    im_i = (adc >> 16).astype(np.int64)
    im_i = np.where(im_i >= 0x8000, im_i - 0x10000, im_i)
    lines = ["# format: iq_ascii_v1", f"# N_ANTENNAS: {a}", f"# SAMPLES_PER_CYCLE: {spc}",
             f"# FFT_SIZE: {n_fft}", f"# HISTORY_FRAMES: {h}"]
    for k, v in (extra or {}).items():
        lines.append(f"# {k}: {v}")
    beats = n_fft // spc
    for f in range(h):
        for ant in range(a):
            for b in range(beats):
                s = [f"{f} {ant} {b} {int(b == 0)} {int(b == beats - 1)}"]
                for slot in range(spc):
                    k = f * n_fft + b * spc + slot
                    s.append(f"{re_i[ant, k]} {im_i[ant, k]}")
                lines.append(" ".join(s))
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "wt", encoding="utf-8") as fh:
        fh.write("\n".join(lines) + "\n")


def load_truth(path) -> dict:
    with Path(path).open("r", encoding="utf-8") as fh:
        return json.load(fh)


def _q15(v: float) -> int:
    return int(max(-32768, min(32767, round(v * 32768.0))))


def chain_setup(hdr: dict, n_beams: int | None = None):
    """(rd_config, coefficients, weights) of the reference's scene test
    (test_pipeline_scenario.cpp:66-101): pass-through PFB (tap 0 = 0x7FFF),
    every FFT stage scaled, CA-CFAR guard 1 / reference 8 per side, alpha
    8.0 (UQ8.8 0x0800), history = the scene's frames. Beam b is steered at
    antenna-DFT angle b with 0.125 per lane: a target at angle index b sums
    coherently on beam b to half its amplitude, the gain the reference test
    gives its beam 0."""
    n, a = int(hdr["FFT_SIZE"]), int(hdr["N_ANTENNAS"])
    h, spc = int(hdr["HISTORY_FRAMES"]), int(hdr["SAMPLES_PER_CYCLE"])
    b = n_beams or a
    taps = 8
    c = abi.RdConfig()
    c.n_chan, c.n_fft, c.taps, c.spc = a, n, taps, spc
    c.scale_sched = 0xFFFFFFFF
    c.hist_frames = 1 << max(2, math.ceil(math.log2(max(h, 4))))
    c.n_beams = b
    c.cfar_enable, c.cfar_mode, c.cfar_out_mode = 1, abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS
    c.guard_lead = c.guard_lag = 1
    c.ref_lead = c.ref_lag = 8
    c.alpha, c.max_guard, c.max_ref = 0x0800, 2, 16
    c.cov_source = abi.RD_COV_OFF
    c.cov_acc_w, c.cov_window = 64, 256
    c.packet_w = 128
    c.max_frames = max(h, 1)
    c.form = abi.RD_FORM_CUDA_CORE
    coeff = np.zeros(n * taps, np.uint32)
    coeff[::taps] = pack(32767, 0)
    w = np.zeros(b * a, np.uint32)
    for bb in range(b):
        for aa in range(a):
            ph = -2.0 * math.pi * bb * aa / a
            w[bb * a + aa] = pack(_q15(0.125 * math.cos(ph)), _q15(0.125 * math.sin(ph)))
    return c, coeff, w


def detect_events(events: np.ndarray) -> list[tuple[int, int, int]]:
    """(frame, beam, bin) of every DETECT event (kind 0, bin = bits 17:2)."""
    w0 = events["w"][:, 0]
    kind = (w0 & 3).astype(int)
    bins = ((w0 >> 2) & 0xFFFF).astype(int)
    sel = kind == abi.RD_EV_DETECT
    return list(zip(events["frame"][sel].astype(int), events["beam"][sel].astype(int),
                    bins[sel]))


def check_detections(detects, targets: list[dict], n_beams: int, bin_tol: int = 1,
                     fa_per_beam: int = 6) -> dict:
    hits = [set() for _ in targets]
    false_alarms = 0
    for frame, beam, b in detects:
        which = -1
        for i, t in enumerate(targets):
            if abs(b - int(t["range_bin"])) <= bin_tol:
                which = i
                break
        if which >= 0:
            hits[which].add((frame, beam, b))
        else:
            false_alarms += 1
    detected = [bool(h) for h in hits]
    fa_max = fa_per_beam * n_beams
    return {"detected": sum(detected), "missed": len(targets) - sum(detected),
            "false_alarms": false_alarms, "false_alarm_max": fa_max,
            "events": len(detects), "per_target": [len(h) for h in hits],
            "passed": all(detected) and false_alarms <= fa_max}


def doppler_peaks(rd_map: np.ndarray, targets: list[dict], win: int = 2) -> list[dict]:
    """The reference's range-Doppler peak check (range_doppler.py:281-358):
    for each target, the argmax of |map| within +/-win range and Doppler bins
    of its ground truth (Doppler wrapping), all antennas; the target passes
    when the peak is within one bin on both axes. rd_map: [antenna][range]
    [Doppler] complex (unshifted Doppler axis)."""
    a, n, h = rd_map.shape
    mag = np.abs(rd_map)
    out = []
    for t in targets:
        r0, d0 = int(t["range_bin"]), int(t["doppler_bin"])
        rs = [r for r in range(r0 - win, r0 + win + 1) if 0 <= r < n]
        ds = [(d0 + k) % h for k in range(-win, win + 1)]
        sub = mag[:, rs][:, :, ds]
        ai, ri, di = np.unravel_index(int(np.argmax(sub)), sub.shape)
        pr, pd = rs[ri], ds[di]
        dd = (pd - d0 + h // 2) % h - h // 2
        out.append({"range": pr, "doppler": pd, "dr": pr - r0, "dd": int(dd),
                    "passed": abs(pr - r0) <= 1 and abs(dd) <= 1})
    return out
