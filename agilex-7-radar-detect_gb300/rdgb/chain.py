"""Python host side of the GB300 radar chain, over the C ABI (librdgb.so).

``Chain`` mirrors the chain the reference composes from its model/cpp blocks
(see include/rd_chain.h); the module-level functions mirror the per-block
call surface (pfb::PfbModel::step, fft::transform, bf::dot, covar::power /
cross_power, cfar::run_frame, packet flits, the fxp op table). Every call
runs CUDA kernels; when the library or the device is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import ptr


def lib():
    return abi.load()


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


class Outputs:
    """Host result buffers for one process call (layout of rd_output)."""

    def __init__(self, cfg: abi.RdConfig, frames: int, n_pairs: int, taps: bool = False,
                 cap_events: int | None = None, alloc=np.zeros):
        """`alloc(shape, dtype)` makes the result arrays (np.zeros; a caller
        may pass pinned host memory so the device writes them by DMA)."""
        N, Cn, B = cfg.n_fft, cfg.n_chan, cfg.n_beams
        if cap_events is None:
            cap_events = frames * B * (2 + N // 16)
        words = (cfg.packet_w + 5 + 31) // 32
        nfl = 1 + (176 + cfg.packet_w - 1) // cfg.packet_w
        wl = max(cfg.cov_window, 1)
        cap_w = frames // wl + 2 if cfg.cov_source else 0
        self.events = alloc(max(cap_events, 1), abi.EVENT_DTYPE)
        self.flits = alloc((max(cap_events, 1) * nfl, words), np.uint32)
        self.cov_windows = alloc(max(cap_w, 1), abi.COVWIN_DTYPE)
        self.cov_acc = alloc((max(cap_w, 1), N, max(n_pairs, 1), 2), np.int64)
        self.taps = taps
        o = self.c = abi.RdOutput()
        o.events, o.cap_events = ptr(self.events), cap_events
        o.flits, o.cap_flits = ptr(self.flits), cap_events * nfl
        o.cov_windows, o.cap_cov_windows = ptr(self.cov_windows), cap_w
        o.cov_acc = ptr(self.cov_acc)
        if taps:
            self.tap_pfb = np.zeros((frames, Cn, N), np.uint32)
            self.tap_spectrum = np.zeros((frames, N, Cn), np.uint32)
            self.tap_beams = np.zeros((frames, B, N), np.uint32)
            self.tap_power = np.zeros((frames, B, N), np.uint32)
            o.tap_pfb = ptr(self.tap_pfb)
            o.tap_spectrum = ptr(self.tap_spectrum)
            o.tap_beams = ptr(self.tap_beams)
            o.tap_power = ptr(self.tap_power)

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
            r.update(tap_pfb=self.tap_pfb, tap_spectrum=self.tap_spectrum,
                     tap_beams=self.tap_beams, tap_power=self.tap_power)
        return r


class Chain:
    """One stream of the chain on the GPU (rd_chain_create ... destroy)."""

    def __init__(self, cfg: abi.RdConfig, coeff, weights, pairs=None):
        self.L = lib()
        self.cfg = cfg
        h = C.c_void_p()
        abi.check(self.L, self.L.rd_chain_create(C.byref(cfg), C.byref(h)), "rd_chain_create")
        self.h = h
        self.set_coeff(coeff)
        self.set_weights(weights)
        if pairs is not None and cfg.cov_source:
            x, y = _u32(pairs[0]), _u32(pairs[1])
            abi.check(self.L, self.L.rd_chain_set_pairs(self.h, ptr(x), ptr(y), len(x)),
                      "rd_chain_set_pairs")
        self.n_pairs = self.L.rd_cov_pairs(C.byref(cfg)) if pairs is None else len(pairs[0])

    def close(self):
        if getattr(self, "h", None):
            self.L.rd_chain_destroy(self.h)
            self.h = None

    __del__ = close

    def set_coeff(self, coeff):
        c = _u32(coeff)
        abi.check(self.L, self.L.rd_chain_set_coeff(self.h, ptr(c)), "rd_chain_set_coeff")

    def set_weights(self, w):
        c = _u32(w)
        abi.check(self.L, self.L.rd_chain_set_weights(self.h, ptr(c)), "rd_chain_set_weights")

    def process(self, adc: np.ndarray, taps: bool = False, cap_events: int | None = None,
                alloc=np.zeros) -> dict:
        """Runs n samples per channel of host ADC data [n_chan][n]; `alloc`
        makes the result buffers (page-locked ones fill while later chunks
        compute)."""
        adc = _u32(adc)
        n = adc.shape[1]
        frames = n // self.cfg.n_fft
        out = Outputs(self.cfg, frames, self.n_pairs, taps, cap_events, alloc=alloc)
        abi.check(self.L, self.L.rd_chain_process(self.h, ptr(adc), n, n, C.byref(out.c)),
                  "rd_chain_process")
        return out.result()

    def process_device(self, adc_dev_ptr: int, n: int, ld: int, stream: int = 0) -> None:
        abi.check(self.L, self.L.rd_chain_process_device(self.h, C.c_void_p(adc_dev_ptr), n, ld,
                                                         C.c_void_p(stream)),
                  "rd_chain_process_device")

    def fetch(self, frames: int, cap_events: int | None = None) -> dict:
        out = Outputs(self.cfg, frames, self.n_pairs, False, cap_events)
        abi.check(self.L, self.L.rd_chain_fetch(self.h, C.byref(out.c)), "rd_chain_fetch")
        return out.result()

    def save_state(self) -> bytes:
        """rd_chain_save_state: the stream's state as bytes (checkpoint)."""
        n = int(self.L.rd_chain_state_size(self.h))
        buf = C.create_string_buffer(n)
        abi.check(self.L, self.L.rd_chain_save_state(self.h, buf, n), "rd_chain_save_state")
        return buf.raw

    def load_state(self, blob: bytes) -> None:
        """rd_chain_load_state: continue the stream a save_state captured."""
        buf = C.create_string_buffer(blob, len(blob))
        abi.check(self.L, self.L.rd_chain_load_state(self.h, buf, len(blob)),
                  "rd_chain_load_state")

    def last_launches(self) -> int:
        return int(self.L.rd_chain_last_launches(self.h))

    def flush_cov(self) -> dict:
        out = Outputs(self.cfg, 0, self.n_pairs, False, 1)
        out.c.cap_cov_windows = 1
        abi.check(self.L, self.L.rd_chain_flush_cov(self.h, C.byref(out.c)), "rd_chain_flush_cov")
        return out.result()

    def stats(self) -> dict:
        s = abi.RdStats()
        abi.check(self.L, self.L.rd_chain_stats(self.h, C.byref(s)), "rd_chain_stats")
        return s.as_dict()

    def doppler(self, n_frames: int, scale_sched: int = 0xFFFFFFFF):
        """(map, stage_flags): map [n_chan][n_fft][n_frames] packed Q1.15, the
        slow-time transform of every (channel, bin) over the newest n_frames
        frames (rd_chain_doppler)."""
        C, N = self.cfg.n_chan, self.cfg.n_fft
        out = np.zeros((C, N, n_frames), np.uint32)
        st = int(np.log2(n_frames))
        fl = np.zeros((C * N, st), np.uint8)
        abi.check(self.L, self.L.rd_chain_doppler(self.h, n_frames, scale_sched, ptr(out),
                                                  ptr(fl)), "rd_chain_doppler")
        return out, fl

    def set_history_depth(self, frames: int) -> None:
        abi.check(self.L, self.L.rd_chain_set_history_depth(self.h, frames),
                  "rd_chain_set_history_depth")

    def read_history(self, bin_: int, frame_off: int):
        vec = np.zeros(self.cfg.n_chan, np.uint32)
        fid, fl = C.c_uint32(0), C.c_uint32(0)
        abi.check(self.L, self.L.rd_chain_read_history(self.h, bin_, frame_off, ptr(vec),
                                                       C.byref(fid), C.byref(fl)),
                  "rd_chain_read_history")
        return vec, fid.value, fl.value


# ---- per-block entry points -------------------------------------------------

def pfb(phases, taps, coeff, state, x):
    x = _u32(x)
    beats = x.size // phases
    st = _u32(state).copy()
    y = np.zeros(beats * phases, np.uint32)
    fl = np.zeros(beats * phases, np.uint8)
    L = lib()
    abi.check(L, L.rd_pfb_run(phases, taps, ptr(_u32(coeff)), ptr(st), ptr(x), beats, ptr(y),
                              ptr(fl)), "rd_pfb_run")
    return y, fl, st


def fft(n, spc, sched, reorder, x):
    x = _u32(x)
    frames = x.size // n
    out = np.zeros(frames * n, np.uint32)
    bins = np.zeros(frames * n, np.uint32)
    st = int(np.log2(n))
    sf = np.zeros(frames * st, np.uint8)
    L = lib()
    abi.check(L, L.rd_fft_run(n, spc, sched, int(reorder), ptr(x), frames, ptr(out), ptr(bins),
                              ptr(sf)), "rd_fft_run")
    return out, bins, sf


def bf(n_ant, n_beams, w, x, form=abi.RD_FORM_CUDA_CORE):
    x = _u32(x)
    nv = x.size // n_ant
    y = np.zeros(nv * n_beams, np.uint32)
    acc = np.zeros(nv * n_beams * 2, np.int64)
    fl = np.zeros(nv * n_beams, np.uint8)
    L = lib()
    abi.check(L, L.rd_bf_run(n_ant, n_beams, ptr(_u32(w)), ptr(x), nv, ptr(y), ptr(acc), ptr(fl),
                             form), "rd_bf_run")
    return y, acc, fl


def power(x):
    x = _u32(x)
    p = np.zeros(x.size, np.int64)
    L = lib()
    abi.check(L, L.rd_power_run(ptr(x), x.size, ptr(p)), "rd_power_run")
    return p


def cross_power(x, y):
    x, y = _u32(x), _u32(y)
    c = np.zeros(2 * x.size, np.int64)
    L = lib()
    abi.check(L, L.rd_cross_power_run(ptr(x), ptr(y), x.size, ptr(c)), "rd_cross_power_run")
    return c


def cfar(cells, n, cfg, frame_ids):
    cells = np.ascontiguousarray(cells, np.int64)
    frames = cells.size // n
    fid = _u32(frame_ids)
    cap = frames * (n + 1)
    ev = np.zeros(max(cap, 1), abi.EVENT_DTYPE)
    ne = C.c_uint64(0)
    L = lib()
    abi.check(L, L.rd_cfar_run(ptr(cells), n, frames, C.byref(cfg), ptr(fid), ptr(ev), cap,
                               C.byref(ne)), "rd_cfar_run")
    return ev[: ne.value]


def packetize(ev, packet_w, src=0, dest=0, vc=0, seq0=0):
    ev = np.ascontiguousarray(ev, abi.EVENT_DTYPE)
    words = (packet_w + 5 + 31) // 32
    nfl = 1 + (176 + packet_w - 1) // packet_w
    fl = np.zeros(max(len(ev) * nfl * words, 1), np.uint32)
    L = lib()
    abi.check(L, L.rd_packetize(ptr(ev), len(ev), packet_w, src, dest, vc, seq0, ptr(fl)),
              "rd_packetize")
    return fl[: len(ev) * nfl * words].reshape(len(ev) * nfl, words)


def fxp(op, a, b, sh, w):
    n = len(op)
    y = np.zeros(n, np.int64)
    fl = np.zeros(n, np.uint8)
    args = [_u32(op), np.ascontiguousarray(a, np.int64), np.ascontiguousarray(b, np.int64),
            _u32(sh), _u32(w)]
    L = lib()
    abi.check(L, L.rd_fxp_apply(*[ptr(v) for v in args], n, ptr(y), ptr(fl)), "rd_fxp_apply")
    return y, fl
