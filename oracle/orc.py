"""Python bindings of the CPU oracles (TEST INFRASTRUCTURE ONLY).

``Oracle("port")`` loads oracle/_build/liborc.so, the plain-C restatement of
the reference model's chain; ``Oracle("ref")`` loads oracle/_ref/liborc_ref.so,
the composition driver over the reference's own model/cpp headers (present
only where the reference sources were available to build it). Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
and only to check or time the CUDA product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
REPO = ROOT.parent
sys.path.insert(0, str(REPO / "agilex-7-radar-detect_gb300"))

from rdgb import abi  # noqa: E402

LIBS = {"port": ROOT / "_build" / "liborc.so", "ref": ROOT / "_ref" / "liborc_ref.so",
        "san": ROOT / "_build" / "liborc_san.so"}
# the reference checkout: $RD_REFERENCE, else a directory named `reference`
# beside the repository
REF_SOURCES = Path(os.environ.get("RD_REFERENCE", str(REPO.parent / "reference")))


def build(which: str = "port") -> Path:
    """Builds an oracle library with oracle/Makefile (gcc/g++ only)."""
    subprocess.run(["make", "-s", "-C", str(ROOT), which, f"REF={REF_SOURCES}"], check=True)
    return LIBS[which]


def available(which: str) -> bool:
    return LIBS[which].exists()


VP, U32, U64, I32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int


class Oracle:
    def __init__(self, which: str = "port"):
        path = LIBS[which]
        if not path.exists():
            raise RuntimeError(f"oracle library {path} not built")
        self.which = which
        L = self.lib = C.CDLL(str(path))
        P = C.POINTER
        for name, res, args in [
            ("orc_chain_create", I32, [P(abi.RdConfig), VP, VP, VP, VP, U32, P(VP)]),
            ("orc_chain_destroy", None, [VP]),
            ("orc_chain_set_coeff", I32, [VP, VP]),
            ("orc_chain_set_weights", I32, [VP, VP]),
            ("orc_chain_process", I32, [VP, VP, U64, U64, P(abi.RdOutput), I32]),
            ("orc_chain_flush_cov", I32, [VP, P(abi.RdOutput)]),
            ("orc_chain_stats", I32, [VP, P(abi.RdStats)]),
            ("orc_chain_read_history", I32, [VP, U32, U32, VP, P(U32), P(U32)]),
            ("orc_chain_set_history_depth", I32, [VP, U32]),
            ("orc_pfb_run", I32, [U32, U32, VP, VP, VP, U32, VP, VP]),
            ("orc_fft_run", I32, [U32, U32, U32, I32, VP, U32, VP, VP, VP]),
            ("orc_bf_run", I32, [U32, U32, VP, VP, U64, VP, VP, VP]),
            ("orc_power_run", I32, [VP, U64, VP]),
            ("orc_cross_power_run", I32, [VP, VP, U64, VP]),
            ("orc_cfar_run", I32, [VP, U32, U32, P(abi.RdConfig), VP, VP, U64, P(U64)]),
            ("orc_packetize", I32, [VP, U64, U32, U32, U32, U32, U32, VP]),
            ("orc_fxp_apply", I32, [VP, VP, VP, VP, VP, U64, VP, VP]),
            ("orc_twiddles", None, [VP]),
            ("orc_name", C.c_char_p, []),
        ]:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        if hasattr(L, "orc_ref_scoreboard"):  # the reference leg only
            L.orc_ref_scoreboard.restype = I32
            L.orc_ref_scoreboard.argtypes = [U32, U32, U32, VP, U64, VP, VP, U64, VP, VP, U64]

    # ---- per block --------------------------------------------------------
    def twiddles(self) -> np.ndarray:
        a = np.zeros(1024, np.uint32)
        self.lib.orc_twiddles(abi.ptr(a))
        return a

    def pfb(self, phases, taps, coeff, state, x):
        x = np.ascontiguousarray(x, np.uint32)
        beats = x.size // phases
        st = np.ascontiguousarray(state, np.uint32).copy()
        y = np.zeros(beats * phases, np.uint32)
        fl = np.zeros(beats * phases, np.uint8)
        assert self.lib.orc_pfb_run(phases, taps, abi.ptr(np.ascontiguousarray(coeff, np.uint32)),
                                    abi.ptr(st), abi.ptr(x), beats, abi.ptr(y), abi.ptr(fl)) == 0
        return y, fl, st

    def fft(self, n, spc, sched, reorder, x):
        x = np.ascontiguousarray(x, np.uint32)
        frames = x.size // n
        out = np.zeros(frames * n, np.uint32)
        bins = np.zeros(frames * n, np.uint32)
        st = int(np.log2(n))
        sf = np.zeros(frames * st, np.uint8)
        r = self.lib.orc_fft_run(n, spc, sched, int(reorder), abi.ptr(x), frames,
                                 abi.ptr(out), abi.ptr(bins), abi.ptr(sf))
        assert r == 0, r
        return out, bins, sf

    def bf(self, n_ant, n_beams, w, x):
        x = np.ascontiguousarray(x, np.uint32)
        nv = x.size // n_ant
        y = np.zeros(nv * n_beams, np.uint32)
        acc = np.zeros(nv * n_beams * 2, np.int64)
        fl = np.zeros(nv * n_beams, np.uint8)
        assert self.lib.orc_bf_run(n_ant, n_beams, abi.ptr(np.ascontiguousarray(w, np.uint32)),
                                   abi.ptr(x), nv, abi.ptr(y), abi.ptr(acc), abi.ptr(fl)) == 0
        return y, acc, fl

    def power(self, x):
        x = np.ascontiguousarray(x, np.uint32)
        p = np.zeros(x.size, np.int64)
        assert self.lib.orc_power_run(abi.ptr(x), x.size, abi.ptr(p)) == 0
        return p

    def cross_power(self, x, y):
        x = np.ascontiguousarray(x, np.uint32)
        y = np.ascontiguousarray(y, np.uint32)
        c = np.zeros(2 * x.size, np.int64)
        assert self.lib.orc_cross_power_run(abi.ptr(x), abi.ptr(y), x.size, abi.ptr(c)) == 0
        return c

    def cfar(self, cells, n, cfg, frame_ids):
        cells = np.ascontiguousarray(cells, np.int64)
        frames = cells.size // n
        fid = np.ascontiguousarray(frame_ids, np.uint32)
        cap = frames * (n + 1)
        ev = np.zeros(cap, abi.EVENT_DTYPE)
        ne = C.c_uint64(0)
        r = self.lib.orc_cfar_run(abi.ptr(cells), n, frames, C.byref(cfg), abi.ptr(fid),
                                  abi.ptr(ev), cap, C.byref(ne))
        assert r == 0, r
        return ev[: ne.value]

    def packetize(self, ev, packet_w, src=0, dest=0, vc=0, seq0=0):
        ev = np.ascontiguousarray(ev, abi.EVENT_DTYPE)
        words = (packet_w + 5 + 31) // 32
        nfl = 1 + (176 + packet_w - 1) // packet_w
        fl = np.zeros(len(ev) * nfl * words, np.uint32)
        assert self.lib.orc_packetize(abi.ptr(ev), len(ev), packet_w, src, dest, vc, seq0,
                                      abi.ptr(fl)) == 0
        return fl.reshape(len(ev) * nfl, words)

    def scoreboard(self, packet_w, radix, stages, injected, ports, observed):
        """The reference's packet_model::Scoreboard (liborc_ref.so only):
        whole packets injected as flit rows, then (port, flit row) observed;
        returns the counts and the delivery log."""
        from scoreboard import COUNT_KEYS
        inj = np.ascontiguousarray(injected, np.uint32)
        obs = np.ascontiguousarray(observed, np.uint32)
        words = (packet_w + 5 + 31) // 32
        pt = np.ascontiguousarray(ports, np.uint32)
        counts = np.zeros(9, np.uint64)
        cap = 64 + 32 * (obs.size // words + 1)
        log = C.create_string_buffer(cap)
        r = self.lib.orc_ref_scoreboard(packet_w, radix, stages, abi.ptr(inj), inj.size // words,
                                        abi.ptr(pt), abi.ptr(obs), obs.size // words,
                                        abi.ptr(counts), log, cap)
        assert r == 0, r
        return dict(zip(COUNT_KEYS, map(int, counts))), log.value.decode().split()

    def fxp(self, op, a, b, sh, w):
        n = len(op)
        y = np.zeros(n, np.int64)
        fl = np.zeros(n, np.uint8)
        args = [np.ascontiguousarray(op, np.uint32), np.ascontiguousarray(a, np.int64),
                np.ascontiguousarray(b, np.int64), np.ascontiguousarray(sh, np.uint32),
                np.ascontiguousarray(w, np.uint32)]
        assert self.lib.orc_fxp_apply(*[abi.ptr(v) for v in args], n, abi.ptr(y), abi.ptr(fl)) == 0
        return y, fl

    # ---- chain -------------------------------------------------------------
    def chain(self, cfg, coeff, weights, px, py):
        return OracleChain(self, cfg, coeff, weights, px, py)


class Outputs:
    """Host buffers for one process call, shared by the oracle and the CUDA
    library so their results compare array for array."""

    def __init__(self, cfg, frames: int, n_pairs: int, taps: bool = True,
                 cap_events: int | None = None):
        N, C_, B = cfg.n_fft, cfg.n_chan, cfg.n_beams
        cap_events = cap_events if cap_events is not None else frames * B * (N + 1)
        words = (cfg.packet_w + 5 + 31) // 32
        nfl = 1 + (176 + cfg.packet_w - 1) // cfg.packet_w
        wl = max(cfg.cov_window, 1)
        cap_w = frames // wl + 2 if cfg.cov_source else 0
        self.events = np.zeros(max(cap_events, 1), abi.EVENT_DTYPE)
        self.flits = np.zeros((max(cap_events, 1) * nfl, words), np.uint32)
        self.cov_windows = np.zeros(max(cap_w, 1), abi.COVWIN_DTYPE)
        self.cov_acc = np.zeros((max(cap_w, 1), N, max(n_pairs, 1), 2), np.int64)
        self.taps = taps
        if taps:
            self.tap_pfb = np.zeros((frames, C_, N), np.uint32)
            self.tap_spectrum = np.zeros((frames, N, C_), np.uint32)
            self.tap_beams = np.zeros((frames, B, N), np.uint32)
            self.tap_power = np.zeros((frames, B, N), np.uint32)
        o = self.c = abi.RdOutput()
        o.events, o.cap_events = abi.ptr(self.events), cap_events
        o.flits, o.cap_flits = abi.ptr(self.flits), cap_events * nfl
        o.cov_windows, o.cap_cov_windows = abi.ptr(self.cov_windows), cap_w
        o.cov_acc = abi.ptr(self.cov_acc)
        if taps:
            o.tap_pfb = abi.ptr(self.tap_pfb)
            o.tap_spectrum = abi.ptr(self.tap_spectrum)
            o.tap_beams = abi.ptr(self.tap_beams)
            o.tap_power = abi.ptr(self.tap_power)

    def result(self) -> dict:
        o = self.c
        r = {
            "n_frames": int(o.n_frames),
            "events": self.events[: o.n_events].copy(),
            "flits": self.flits[: o.n_flits].copy(),
            "cov_windows": self.cov_windows[: o.n_cov_windows].copy(),
            "cov_acc": self.cov_acc[: o.n_cov_windows].copy(),
        }
        if self.taps:
            r.update(tap_pfb=self.tap_pfb.copy(), tap_spectrum=self.tap_spectrum.copy(),
                     tap_beams=self.tap_beams.copy(), tap_power=self.tap_power.copy())
        return r


class OracleChain:
    def __init__(self, orc: Oracle, cfg, coeff, weights, px, py):
        self.orc, self.cfg = orc, cfg
        self.n_pairs = len(px)
        h = C.c_void_p()
        args = [np.ascontiguousarray(coeff, np.uint32), np.ascontiguousarray(weights, np.uint32),
                np.ascontiguousarray(px, np.uint32), np.ascontiguousarray(py, np.uint32)]
        self._keep = args
        r = orc.lib.orc_chain_create(C.byref(cfg), *[abi.ptr(a) for a in args], len(px),
                                     C.byref(h))
        if r != 0:
            raise ValueError(f"orc_chain_create: {r}")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.orc.lib.orc_chain_destroy(self.h)
            self.h = None

    def process(self, adc: np.ndarray, taps: bool = True, threads: int = 1,
                cap_events: int | None = None) -> dict:
        adc = np.ascontiguousarray(adc, np.uint32)
        n = adc.shape[1]
        frames = n // self.cfg.n_fft
        out = Outputs(self.cfg, frames, self.n_pairs, taps, cap_events)
        r = self.orc.lib.orc_chain_process(self.h, abi.ptr(adc), n, n, C.byref(out.c), threads)
        if r != 0:
            raise RuntimeError(f"orc_chain_process: {r}")
        return out.result()

    def set_coeff(self, coeff):
        c = np.ascontiguousarray(coeff, np.uint32)
        assert self.orc.lib.orc_chain_set_coeff(self.h, abi.ptr(c)) == 0

    def set_weights(self, w):
        c = np.ascontiguousarray(w, np.uint32)
        assert self.orc.lib.orc_chain_set_weights(self.h, abi.ptr(c)) == 0

    def flush_cov(self) -> dict:
        out = Outputs(self.cfg, 0, self.n_pairs, taps=False)
        out.c.cap_cov_windows = 1
        assert self.orc.lib.orc_chain_flush_cov(self.h, C.byref(out.c)) == 0
        return out.result()

    def stats(self) -> dict:
        s = abi.RdStats()
        self.orc.lib.orc_chain_stats(self.h, C.byref(s))
        return s.as_dict()

    def set_history_depth(self, frames: int) -> None:
        assert self.orc.lib.orc_chain_set_history_depth(self.h, frames) == 0

    def read_history(self, bin_, frame_off):
        vec = np.zeros(self.cfg.n_chan, np.uint32)
        fid, fl = C.c_uint32(0), C.c_uint32(0)
        self.orc.lib.orc_chain_read_history(self.h, bin_, frame_off, abi.ptr(vec),
                                            C.byref(fid), C.byref(fl))
        return vec, fid.value, fl.value
