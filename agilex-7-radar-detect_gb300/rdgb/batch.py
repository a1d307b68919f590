"""Many independent scenarios of uneven geometry in one CUDA graph: the
ctypes wrapper of rd_batch_* (include/rd_chain.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .chain import Outputs


class Batch:
    def __init__(self, cfgs: list, coeffs: list, weights: list, n_streams: int = 16,
                 launch_frames: int = 0, use_graph: bool = True):
        self.L = abi.load()
        n = len(cfgs)
        self.cfgs = cfgs
        arr = (abi.RdConfig * n)(*cfgs)
        self._coeff = [np.ascontiguousarray(c, np.uint32) for c in coeffs]
        self._w = [np.ascontiguousarray(w, np.uint32) for w in weights]
        cp = (C.c_void_p * n)(*[c.ctypes.data for c in self._coeff])
        wp = (C.c_void_p * n)(*[w.ctypes.data for w in self._w])
        self.opt = abi.RdBatchOptions(n_streams, launch_frames, 1 if use_graph else 0)
        self._outs = None
        self.h = C.c_void_p()
        abi.check(self.L, self.L.rd_batch_create(n, arr, cp, wp, C.byref(self.opt),
                                                 C.byref(self.h)), "rd_batch_create")

    def _args(self, ptrs, ns):
        n = len(self.cfgs)
        return (C.c_void_p * n)(*ptrs), (C.c_uint64 * n)(*ns)

    def run(self, ptrs, ns, stream: int = 0, sequential: bool = False) -> None:
        p, q = self._args(ptrs, ns)
        fn = self.L.rd_batch_run_sequential if sequential else self.L.rd_batch_run
        abi.check(self.L, fn(self.h, p, q, C.c_void_p(stream)), "rd_batch_run")

    def tune(self, ptrs, ns, reps: int = 3, cache: str | None = None):
        """Autotune (rd_batch_tune): the chosen options and their time. With
        `cache` (a file path), rd_batch_tune_cached: a choice recorded there
        for these scenarios on this device is applied without tuning, else the
        tuning's choice is appended; the result then also says whether the
        cache answered (`hit`)."""
        p, q = self._args(ptrs, ns)
        o = abi.RdBatchOptions()
        ms = C.c_double()
        if cache is None:
            abi.check(self.L, self.L.rd_batch_tune(self.h, p, q, reps, C.byref(o), C.byref(ms)),
                      "rd_batch_tune")
            return {"n_streams": o.n_streams, "launch_frames": o.launch_frames}, ms.value
        hit = C.c_int(0)
        abi.check(self.L, self.L.rd_batch_tune_cached(self.h, p, q, reps, str(cache).encode(),
                                                      C.byref(o), C.byref(ms), C.byref(hit)),
                  "rd_batch_tune_cached")
        return ({"n_streams": o.n_streams, "launch_frames": o.launch_frames, "hit": bool(hit.value)},
                ms.value)

    def fetch(self, i: int, frames: int, n_pairs: int) -> dict:
        out = Outputs(self.cfgs[i], frames, n_pairs, False, None)
        abi.check(self.L, self.L.rd_batch_fetch(self.h, i, C.byref(out.c)), "rd_batch_fetch")
        return out.result()

    def set_outputs(self, outs: list | None) -> None:
        """rd_batch_set_outputs: every run writes scenario i's results into
        outs[i] (an Outputs over page-locked host arrays); None stops it."""
        if outs is None:
            abi.check(self.L, self.L.rd_batch_set_outputs(self.h, None), "rd_batch_set_outputs")
            self._outs = None
            return
        arr = (abi.RdOutput * len(outs))(*[o.c for o in outs])
        abi.check(self.L, self.L.rd_batch_set_outputs(self.h, arr), "rd_batch_set_outputs")
        self._outs = list(outs)  # the arrays stay alive while registered

    def results(self, i: int, check: bool = True) -> dict:
        """rd_batch_results: scenario i's results of the last run, from its
        registered Outputs (no device read)."""
        out = self._outs[i]
        st = self.L.rd_batch_results(self.h, i, C.byref(out.c))
        if check:
            abi.check(self.L, st, "rd_batch_results")
        return out.result()

    def egress(self, n_ports: int, ring: int, cap_per_port: int, port_count: int,
               src_of: int = 0, stream: int = 0) -> None:
        """rd_batch_egress: the last run's packets, scenario i a source of
        port cfgs[i].dest, merged into device rings on `stream`."""
        abi.check(self.L, self.L.rd_batch_egress(self.h, n_ports, C.c_void_p(ring), cap_per_port,
                                                 C.c_void_p(src_of or None),
                                                 C.c_void_p(port_count), C.c_void_p(stream)),
                  "rd_batch_egress")

    def close(self) -> None:
        if self.h:
            self.L.rd_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
