"""A request loop over many resident streams: the ctypes wrapper of
rd_server_* / rd_stream_* (include/rd_chain.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .chain import Outputs


class Server:
    def __init__(self, hbm_budget: int, max_inflight: int = 8, queue_cap: int = 64,
                 max_chan: int = 64, max_request_samples: int = 4096):
        self.L = abi.load()
        self.cfg = abi.RdServerConfig(hbm_budget, max_inflight, queue_cap, max_chan,
                                      max_request_samples)
        self.h = C.c_void_p()
        abi.check(self.L, self.L.rd_server_create(C.byref(self.cfg), C.byref(self.h)),
                  "rd_server_create")
        self.streams: dict[int, tuple] = {}   # id -> (cfg, n_pairs)
        self._keep = []

    def open(self, cfg: abi.RdConfig, coeff, weights, pairs=None) -> tuple[int, int]:
        """(status, stream id); the id is valid when status is RD_OK. `pairs`
        (x, y): the covariance pair table, else the default one."""
        co = np.ascontiguousarray(coeff, np.uint32)
        w = np.ascontiguousarray(weights, np.uint32)
        sid = C.c_uint32()
        st = self.L.rd_stream_open(self.h, C.byref(cfg), co.ctypes.data, w.ctypes.data,
                                   C.byref(sid))
        if st == abi.RD_OK and pairs is not None and cfg.cov_source:
            x = np.ascontiguousarray(pairs[0], np.uint32)
            y = np.ascontiguousarray(pairs[1], np.uint32)
            st = self.L.rd_stream_set_pairs(self.h, sid.value, x.ctypes.data, y.ctypes.data,
                                            len(x))
            if st != abi.RD_OK:
                self.L.rd_stream_close(self.h, sid.value)
        if st == abi.RD_OK:
            self.streams[sid.value] = (cfg, self.L.rd_cov_pairs(C.byref(cfg)))
        return st, sid.value

    def close_stream(self, sid: int) -> int:
        st = self.L.rd_stream_close(self.h, sid)
        if st == abi.RD_OK:
            self.streams.pop(sid, None)
        return st

    def submit(self, sid: int, adc: np.ndarray) -> tuple[int, int]:
        """(status, request id); RD_EAGAIN when the queue is full."""
        x = np.ascontiguousarray(adc, np.uint32)
        rid = C.c_uint64()
        st = self.L.rd_server_submit(self.h, sid, x.ctypes.data, x.shape[1], x.shape[1],
                                     C.byref(rid))
        return st, rid.value

    def poll(self, cap: int = 64) -> list[dict]:
        arr = (abi.RdCompletion * cap)()
        n = C.c_uint32()
        abi.check(self.L, self.L.rd_server_poll(self.h, arr, cap, C.byref(n)), "rd_server_poll")
        return [{f: getattr(arr[i], f) for f, _ in abi.RdCompletion._fields_}
                for i in range(n.value)]

    def take(self, rid: int, sid: int, frames: int) -> dict:
        cfg, n_pairs = self.streams[sid]
        out = Outputs(cfg, frames, n_pairs, False, None)
        abi.check(self.L, self.L.rd_server_take(self.h, rid, C.byref(out.c)), "rd_server_take")
        return out.result()

    def info(self) -> dict:
        i = abi.RdServerInfo()
        abi.check(self.L, self.L.rd_server_info_get(self.h, C.byref(i)), "rd_server_info_get")
        return {f: getattr(i, f) for f, _ in abi.RdServerInfo._fields_}

    def run_trace(self, stream_ids, arrival_us, adcs) -> tuple[np.ndarray, float]:
        n = len(stream_ids)
        sids = np.ascontiguousarray(stream_ids, np.uint32)
        arr = np.ascontiguousarray(arrival_us, np.float64)
        xs = [np.ascontiguousarray(a, np.uint32) for a in adcs]
        ptrs = (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        ns = np.array([x.shape[1] for x in xs], np.uint64)
        lat = np.zeros(n, np.float64)
        mk = C.c_double()
        abi.check(self.L, self.L.rd_server_run_trace(self.h, n, sids.ctypes.data, arr.ctypes.data,
                                                     ptrs, ns.ctypes.data, lat.ctypes.data,
                                                     C.byref(mk)), "rd_server_run_trace")
        return lat, mk.value

    def close(self) -> None:
        if self.h:
            self.L.rd_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
