"""Stream geometries and seeded synthetic inputs for the radar chain.

No public dataset is involved: the reference drives its chain with a synthetic
scene generator (model/python/gen_target_iq.py:437-517). The inputs here are
seeded stand-ins with the shapes the workloads name: complex int16 ADC samples
in a 12-bit range made of tones (plane waves across the array), an optional
linear chirp and Gaussian-like noise, windowed-sinc PFB coefficients and
DFT steering weights.

The ADC generator is integer-only (a phase-accumulator oscillator over the
Q1.15 twiddle table and a counter-based hash for the noise), so the same seed
gives the same samples on any machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

from . import abi
from .twiddle import TWIDDLES

BASE_SEED = 20261203

MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)


@dataclass(frozen=True)
class Preset:
    name: str
    n_chan: int
    n_fft: int
    taps: int
    spc: int
    hist_frames: int
    n_beams: int
    guard: tuple[int, int]   # (lead, lag)
    ref: tuple[int, int]     # (lead, lag)
    max_guard: int
    max_ref: int
    alpha: int               # UQ8.8
    cov_source: int
    cov_window: int
    cov_acc_w: int
    packet_w: int
    cpi_samples: int         # samples per channel per CPI
    n_cpi: int
    n_tones: int
    chirp: bool
    seed_index: int
    cov_pairs: tuple[tuple[int, int], ...] | None = None   # None: all i <= j
    window: str = "hann"
    cfar_mode: int = abi.RD_CFAR_CA
    out_mode: int = abi.RD_CFAR_EVENTS
    cov_mode: int = abi.RD_COV_BLOCK
    cov_exp_k: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def frames_per_cpi(self) -> int:
        return self.cpi_samples // self.n_fft

    @property
    def seed(self) -> int:
        return BASE_SEED + self.seed_index


# The workloads. tiny / medium / full follow the geometry of the three chain
# workloads (4/16/64 channels, 16/256/1024-channel PFB and FFT, 4/8/16 taps,
# 8/32/64-frame history, 2/16/64 beams). tiny's 16-bin frame cannot hold a
# 2-guard + 8-reference window on each side, so its "8 reference and 2 guard
# cells" are read as totals split over the two sides. "ref_tiny" is the
# reference's own config/tiny.json geometry (2 antennas, 64-point FFT, one
# sample per cycle, 4-frame history).
PRESETS = {
    "tiny": Preset("tiny", 4, 16, 4, 2, 8, 2, (1, 1), (4, 4), 2, 8, 0x0800,
                   abi.RD_COV_CHANNEL, 256, 64, 64, 4096, 1, 3, False, 0),
    "medium": Preset("medium", 16, 256, 8, 2, 32, 16, (4, 4), (16, 16), 4, 16, 0x0800,
                     abi.RD_COV_CHANNEL, 256, 64, 128, 65536, 64, 5, True, 1),
    "full": Preset("full", 64, 1024, 16, 2, 64, 64, (4, 4), (32, 32), 4, 32, 0x0800,
                   abi.RD_COV_CHANNEL, 256, 64, 512, 1 << 20, 16, 6, False, 2),
    "ref_tiny": Preset("ref_tiny", 2, 64, 4, 1, 4, 2, (2, 2), (8, 8), 2, 8, 0x0800,
                       abi.RD_COV_BEAM, 64, 40, 64, 4096, 1, 2, False, 5,
                       cov_pairs=((0, 1),)),
}


def preset(name: str, **over) -> Preset:
    p = PRESETS[name]
    return replace(p, **over) if over else p


def pair_table(p: Preset) -> tuple[np.ndarray, np.ndarray]:
    """Covariance pair table: every (i <= j) of the source vector by default
    (the Hermitian upper triangle), or the preset's explicit pairs."""
    if p.cov_pairs is not None:
        xs = np.array([a for a, _ in p.cov_pairs], dtype=np.uint32)
        ys = np.array([b for _, b in p.cov_pairs], dtype=np.uint32)
        return xs, ys
    n = p.n_chan if p.cov_source == abi.RD_COV_CHANNEL else p.n_beams
    iu = np.triu_indices(n)
    return iu[0].astype(np.uint32), iu[1].astype(np.uint32)


def make_config(p: Preset, max_frames: int | None = None,
                form: int = abi.RD_FORM_CUDA_CORE) -> abi.RdConfig:
    c = abi.RdConfig()
    c.n_chan, c.n_fft, c.taps, c.spc = p.n_chan, p.n_fft, p.taps, p.spc
    c.scale_sched = 0xFFFFFFFF
    c.hist_frames, c.n_beams = p.hist_frames, p.n_beams
    c.cfar_enable, c.cfar_mode, c.cfar_out_mode = 1, p.cfar_mode, p.out_mode
    c.guard_lead, c.guard_lag = p.guard
    c.ref_lead, c.ref_lag = p.ref
    c.alpha, c.max_guard, c.max_ref = p.alpha, p.max_guard, p.max_ref
    c.cov_source, c.cov_mode, c.cov_exp_k = p.cov_source, p.cov_mode, p.cov_exp_k
    c.cov_window, c.cov_acc_w = p.cov_window, p.cov_acc_w
    c.cov_n_pairs = len(pair_table(p)[0]) if p.cov_source != abi.RD_COV_OFF else 0
    c.packet_w, c.src_id, c.dest, c.vc = p.packet_w, 0, 0, 0
    c.max_frames = max_frames if max_frames else min(p.frames_per_cpi * p.n_cpi, 1024)
    c.form = form
    return c


# ---------------------------------------------------------------------------
# Fixed-point packing helpers
# ---------------------------------------------------------------------------

def pack(re, im) -> np.ndarray:
    re = np.asarray(re, dtype=np.int64)
    im = np.asarray(im, dtype=np.int64)
    return (((im & 0xFFFF) << 16) | (re & 0xFFFF)).astype(np.uint32)


def unpack(p) -> tuple[np.ndarray, np.ndarray]:
    p = np.asarray(p, dtype=np.uint32)
    re = (p & 0xFFFF).astype(np.uint16).view(np.int16).astype(np.int64)
    im = (p >> 16).astype(np.uint16).view(np.int16).astype(np.int64)
    return re, im


def q15(x: np.ndarray) -> np.ndarray:
    """Real -> Q1.15, round to nearest even then saturate."""
    v = np.rint(np.asarray(x, dtype=np.float64) * 32768.0)
    return np.clip(v, -32768, 32767).astype(np.int64)


# ---------------------------------------------------------------------------
# Coefficients and weights
# ---------------------------------------------------------------------------

def _window(name: str, n: int) -> np.ndarray:
    if n == 1:
        return np.ones(1)
    t = np.arange(n, dtype=np.float64) / float(n - 1)
    if name == "rect":
        return np.ones(n)
    if name == "hann":
        return 0.5 - 0.5 * np.cos(2 * np.pi * t)
    if name == "hamming":
        return 0.54 - 0.46 * np.cos(2 * np.pi * t)
    if name == "blackman":
        return 0.42 - 0.5 * np.cos(2 * np.pi * t) + 0.08 * np.cos(4 * np.pi * t)
    raise ValueError(name)


def coefficients(phases: int, taps: int, window: str = "hann", mix: float = 0.0,
                 l1_target: float = 0.98) -> np.ndarray:
    """Windowed-sinc channelizer prototype of length phases*taps (cutoff
    1/phases), split into phase branches h_p[k] = proto[k*phases + p], scaled
    so the largest branch L1 norm is l1_target (the output cannot clip),
    quantised to Q1.15. Returned phase-major, tap-minor, packed."""
    L = phases * taps
    n = np.arange(L, dtype=np.float64)
    fc = 1.0 / phases
    h = fc * np.sinc(fc * (n - (L - 1) / 2.0)) * _window(window, L)
    h = h.astype(np.complex128)
    if mix:
        h = h * np.exp(2j * np.pi * mix * n)
    br = h.reshape(taps, phases).T        # br[p, k] = h[k*phases + p]
    worst = np.max(np.sum(np.abs(br), axis=1))
    if worst > 0:
        br = br * (l1_target / worst)
    return pack(q15(br.real), q15(br.imag)).reshape(-1)


def identity_coefficients(phases: int, taps: int) -> np.ndarray:
    """Per-phase unit impulse at tap 0 (gain 0x7FFF): a pass-through bank."""
    re = np.zeros((phases, taps), dtype=np.int64)
    re[:, 0] = 32767
    return pack(re, np.zeros_like(re)).reshape(-1)


def steering_weights(n_chan: int, n_beams: int, gain: float = 0.9) -> np.ndarray:
    """DFT beams w[b][a] = gain/sqrt(C) * exp(-j 2 pi b a / B), beam-major."""
    b = np.arange(n_beams)[:, None]
    a = np.arange(n_chan)[None, :]
    w = gain / np.sqrt(n_chan) * np.exp(-2j * np.pi * b * a / max(n_beams, 1))
    return pack(q15(w.real), q15(w.imag)).reshape(-1)


# ---------------------------------------------------------------------------
# Integer ADC generator
# ---------------------------------------------------------------------------

def _mix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return x


@dataclass(frozen=True)
class Tone:
    amp: int        # peak amplitude in LSB
    freq: int       # phase increment per sample, u32 turns
    dphi: int       # phase step per antenna, u32 turns
    phi0: int       # initial phase, u32 turns
    chirp: int = 0  # phase-increment increment per sample (linear chirp)


def scene(p: Preset, seed: int | None = None) -> list[Tone]:
    """Seeded scene: n_tones plane waves (+ one chirp) with a total peak
    amplitude of 2047 - 4*sigma, sigma = 64."""
    rng = np.random.default_rng(p.seed if seed is None else seed)
    n_sig = p.n_tones + (1 if p.chirp else 0)
    budget = 2047 - 4 * 64
    amps = rng.uniform(0.4, 1.0, size=n_sig)
    amps = np.floor(amps / amps.sum() * budget).astype(int)
    tones = []
    for i in range(n_sig):
        # a frequency at a channel centre plus a seeded offset inside it
        k = int(rng.integers(0, p.n_fft))
        frac = float(rng.uniform(-0.3, 0.3))
        f = ((k + frac) / p.n_fft) % 1.0
        # arrival angle -> per-antenna phase step, aligned to a beam for half
        beam = int(rng.integers(0, max(p.n_beams, 1)))
        ds = (beam / max(p.n_beams, 1)) + (0.0 if i % 2 == 0 else float(rng.uniform(-0.2, 0.2)) / max(p.n_beams, 1))
        chirp = 0
        if p.chirp and i == n_sig - 1:
            # sweeps a quarter of the band over one CPI
            chirp = int(round(0.25 / p.cpi_samples * 2**32 / max(p.cpi_samples, 1)))
        tones.append(Tone(int(amps[i]), int(round(f * 2**32)) & 0xFFFFFFFF,
                          int(round((-ds % 1.0) * 2**32)) & 0xFFFFFFFF,
                          int(rng.integers(0, 2**32)), chirp))
    return tones


TW_RE, TW_IM = unpack(np.array(TWIDDLES, dtype=np.uint32))


def _adc_row(tones, s: int, a: int, idx: np.ndarray, out_row: np.ndarray) -> None:
    """Channel a of the ADC samples at time indices idx, into out_row."""
    n = idx.size
    re = np.zeros(n, dtype=np.int64)
    im = np.zeros(n, dtype=np.int64)
    for t in tones:
        with np.errstate(over="ignore"):
            ph = (np.uint64(t.phi0) + np.uint64(t.dphi) * np.uint64(a)
                  + np.uint64(t.freq) * idx)
            if t.chirp:
                ph = ph + np.uint64(t.chirp) * ((idx * (idx - np.uint64(1))) >> np.uint64(1))
        e = ((ph & np.uint64(0xFFFFFFFF)) >> np.uint64(22)).astype(np.int64)
        # exp(+j phase) = conj(W^e)
        re += (t.amp * TW_RE[e] + (1 << 14)) >> 15
        im += (-t.amp * TW_IM[e] + (1 << 14)) >> 15
    key = (np.uint64(s & 0xFFFFFFFF) << np.uint64(32)) ^ (np.uint64(a) << np.uint64(40))
    h1 = _mix64(key ^ (idx * np.uint64(2)))
    h2 = _mix64(key ^ (idx * np.uint64(2) + np.uint64(1)))
    for h, acc in ((h1, re), (h2, im)):
        u = sum(((h >> np.uint64(16 * k)) & np.uint64(0xFFFF)).astype(np.int64) for k in range(4))
        acc += ((u - 2 * 65535) * 111) >> 16     # sigma ~ 64
    np.clip(re, -2047, 2047, out=re)
    np.clip(im, -2047, 2047, out=im)
    out_row[:] = pack(re, im)


def adc(p: Preset, n: int, start: int = 0, seed: int | None = None,
        chans: slice | None = None, threads: int | None = None) -> np.ndarray:
    """ADC samples [n_chan][n] (packed complex int16) for sample indices
    start .. start+n-1 of the stream. Integer-only, deterministic. Large
    requests spread the channels over host threads (the values do not depend
    on it)."""
    import os
    s = p.seed if seed is None else seed
    tones = scene(p, s)
    ch = range(p.n_chan)[chans] if chans is not None else range(p.n_chan)
    out = np.empty((len(ch), n), dtype=np.uint32)
    # rows in pieces of at most 2^20 samples keep the temporaries small
    piece = 1 << 20
    jobs = [(row, a, lo) for row, a in enumerate(ch) for lo in range(0, n, piece)]

    def run(job):
        row, a, lo = job
        hi = min(n, lo + piece)
        idx = np.arange(start + lo, start + hi, dtype=np.uint64)
        _adc_row(tones, s, a, idx, out[row, lo:hi])

    if threads is None:
        threads = min(os.cpu_count() or 1, 16) if len(ch) * n >= (1 << 22) else 1
    if threads > 1 and len(jobs) > 1:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(run, jobs))
    else:
        for j in jobs:
            run(j)
    return out


# ---------------------------------------------------------------------------
# The batching workload: independent scenarios of uneven geometry
# ---------------------------------------------------------------------------

def batch_scenarios(n: int, seed_index: int = 3, log2_min: int = 12,
                    log2_max: int = 18) -> list[Preset]:
    """`n` scenarios drawn from a seed: channels in {4, 16, 32, 64}, PFB/FFT
    size in {16, 64, 256, 1024}, taps in {4, 8, 16}, CPI length log-uniform
    in 2^log2_min .. 2^log2_max samples per channel (rounded to a multiple of
    the FFT size), beams = channels, channel covariance over 256-frame
    windows, CA-CFAR with reference/guard cells scaled to the frame, tones
    plus noise."""
    rng = np.random.default_rng(BASE_SEED + seed_index)
    out = []
    for i in range(n):
        C = int(rng.choice([4, 16, 32, 64]))
        N = int(rng.choice([16, 64, 256, 1024]))
        T = int(rng.choice([4, 8, 16]))
        cpi = int(round(2.0 ** rng.uniform(log2_min, log2_max)))
        cpi = max(N, (cpi // N) * N)
        ref = max(2, min(16, N // 8))
        guard = max(1, min(4, N // 64))
        out.append(Preset(f"batch{i}", C, N, T, 2, 8, C, (guard, guard), (ref, ref), guard, ref,
                          0x0800, abi.RD_COV_CHANNEL, 256, 64, 128, cpi, 1, 3, False,
                          1000 + i))
    return out
