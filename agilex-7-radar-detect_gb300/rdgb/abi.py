"""ctypes mirror of include/rd_chain.h and the loader of the CUDA library.

The structures here are the C ABI's, field for field; the library itself is
built in-tree by :mod:`rdgb.build` into ``agilex-7-radar-detect_gb300/_build``.
Loading fails loudly when the library is missing: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_ROOT = Path(__file__).resolve().parent.parent
BUILD_DIR = PKG_ROOT / "_build"
LIB_PATH = BUILD_DIR / "librdgb.so"

RD_OK, RD_EINVAL, RD_ENOMEM, RD_ETIMEOUT, RD_EDEVICE, RD_ETRUNC, RD_EAGAIN = range(7)
STATUS_NAMES = {0: "RD_OK", 1: "RD_EINVAL", 2: "RD_ENOMEM", 3: "RD_ETIMEOUT",
                4: "RD_EDEVICE", 5: "RD_ETRUNC", 6: "RD_EAGAIN"}

RD_CFAR_CA, RD_CFAR_GO = 0, 1
RD_CFAR_EVENTS, RD_CFAR_DENSE = 0, 1
RD_EV_DETECT, RD_EV_BIN, RD_EV_SUPPRESSED, RD_EV_SUMMARY = 0, 1, 2, 3
RD_COV_OFF, RD_COV_CHANNEL, RD_COV_BEAM = 0, 1, 2
RD_COV_BLOCK, RD_COV_EXP = 0, 1
RD_FORM_CUDA_CORE, RD_FORM_TENSOR, RD_FORM_TENSOR_WARP = 0, 1, 2
RD_TC_MAX_CHAN = 128
RD_STATIC_CFAR_MAX_FRAMES, RD_STATIC_CFAR_MAX_CELLS = 4096, 1024

OPS = ["sat", "trunc", "round_even", "round_half_up", "round", "round_sat",
       "add_sat", "sub_sat", "neg_sat", "mul_q15", "mul_q15_rs", "cmul_re",
       "cmul_im", "acc_w", "growth_bits"]
OP_CODE = {name: i for i, name in enumerate(OPS)}


class RdConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "n_chan", "n_fft", "taps", "spc", "scale_sched", "hist_frames", "n_beams",
        "cfar_enable", "cfar_mode", "cfar_out_mode", "guard_lead", "guard_lag",
        "ref_lead", "ref_lag", "alpha", "max_guard", "max_ref",
        "cov_source", "cov_mode", "cov_exp_k", "cov_window", "cov_acc_w",
        "cov_n_pairs", "packet_w", "src_id", "dest", "vc", "max_frames", "form",
        "engine_pairs")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


class RdEvent(C.Structure):
    _fields_ = [("w", C.c_uint64 * 3), ("frame", C.c_uint32), ("beam", C.c_uint16),
                ("kind", C.c_uint8), ("framing", C.c_uint8)]


EVENT_DTYPE = np.dtype([("w", "<u8", (3,)), ("frame", "<u4"), ("beam", "<u2"),
                        ("kind", "u1"), ("framing", "u1")])
assert EVENT_DTYPE.itemsize == C.sizeof(RdEvent) == 32


class RdCovWindow(C.Structure):
    _fields_ = [("window_id", C.c_uint32), ("sample_count", C.c_uint32),
                ("end_frame", C.c_uint32), ("flushed", C.c_uint8),
                ("truncated", C.c_uint8), ("sat_flags", C.c_uint8), ("pad", C.c_uint8)]


COVWIN_DTYPE = np.dtype([("window_id", "<u4"), ("sample_count", "<u4"),
                         ("end_frame", "<u4"), ("flushed", "u1"), ("truncated", "u1"),
                         ("sat_flags", "u1"), ("pad", "u1")])
assert COVWIN_DTYPE.itemsize == C.sizeof(RdCovWindow) == 16


class RdOutput(C.Structure):
    _fields_ = [
        ("events", C.c_void_p), ("cap_events", C.c_uint64), ("n_events", C.c_uint64),
        ("flits", C.c_void_p), ("cap_flits", C.c_uint64), ("n_flits", C.c_uint64),
        ("flit_words", C.c_uint32),
        ("cov_windows", C.c_void_p), ("cap_cov_windows", C.c_uint32),
        ("n_cov_windows", C.c_uint32),
        ("cov_acc", C.c_void_p),
        ("tap_pfb", C.c_void_p), ("tap_spectrum", C.c_void_p),
        ("tap_beams", C.c_void_p), ("tap_power", C.c_void_p),
        ("n_frames", C.c_uint64),
    ]


class RdKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("total_ms", C.c_double)]


class RdStats(C.Structure):
    _fields_ = [
        ("frames", C.c_uint64), ("pfb_flags", C.c_uint32), ("pfb_sat_samples", C.c_uint64),
        ("fft_stage_flags", C.c_uint32 * 11), ("bf_flags", C.c_uint32),
        ("bf_sat_samples", C.c_uint64), ("cov_flags", C.c_uint32),
        ("cov_sat_steps", C.c_uint64),
        ("hist_frames_done", C.c_uint32), ("hist_write_beats", C.c_uint32),
        ("hist_reads", C.c_uint32), ("hist_collisions", C.c_uint32),
        ("hist_errors", C.c_uint32), ("hist_overwrites", C.c_uint32),
        ("hist_skew", C.c_uint32),
        ("align_beats", C.c_uint32), ("align_missing", C.c_uint32),
        ("align_dup", C.c_uint32), ("align_orphan", C.c_uint32),
        ("align_timeout", C.c_uint32), ("align_fault", C.c_uint32),
        ("cfar_det", C.c_uint64), ("cfar_sup", C.c_uint64), ("cfar_frames", C.c_uint64),
        ("packets", C.c_uint64), ("flits", C.c_uint64), ("next_seq", C.c_uint32),
        ("hist_depth", C.c_uint32), ("hist_epoch", C.c_uint32),
        ("engine_window", C.c_uint32), ("engine_samples", C.c_uint32),
        ("engine_sat", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        d = {}
        for n, _ in self._fields_:
            v = getattr(self, n)
            d[n] = list(v) if n == "fft_stage_flags" else int(v)
        return d


def ptr(a) -> C.c_void_p | None:
    """Address of a numpy array's data (None for None)."""
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)


# C prototypes shared by the product library and the oracles' per-block calls.
class RdBatchOptions(C.Structure):
    _fields_ = [("n_streams", C.c_uint32), ("launch_frames", C.c_uint32), ("use_graph", C.c_int)]


class RdServerConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_inflight", C.c_uint32),
                ("queue_cap", C.c_uint32), ("max_chan", C.c_uint32),
                ("max_request_samples", C.c_uint64)]


class RdCompletion(C.Structure):
    _fields_ = [("req_id", C.c_uint64), ("stream_id", C.c_uint32), ("status", C.c_int32),
                ("n_events", C.c_uint64), ("n_cov_windows", C.c_uint32),
                ("t_submit_us", C.c_double), ("t_start_us", C.c_double),
                ("t_done_us", C.c_double)]


class RdServerInfo(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("hbm_used", C.c_uint64), ("streams", C.c_uint32),
                ("inflight", C.c_uint32), ("queued", C.c_uint32)]


class RdEgressSource(C.Structure):
    _fields_ = [("flits", C.c_void_p), ("count_dev", C.c_void_p), ("n_packets", C.c_uint64),
                ("dest", C.c_uint32), ("reserved", C.c_uint32)]


RD_EGRESS_MAX_SRC = 512


def _proto(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


VP, U32, U64, I32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int


def declare_rd(lib) -> None:
    """Declares the product's exported functions on a loaded CDLL."""
    P = C.POINTER
    _proto(lib, "rd_config_default", None, [P(RdConfig)])
    _proto(lib, "rd_config_validate", I32, [P(RdConfig)])
    _proto(lib, "rd_flit_words", U32, [U32])
    _proto(lib, "rd_detection_flits", U32, [U32])
    _proto(lib, "rd_cov_pairs", U32, [P(RdConfig)])
    _proto(lib, "rd_chain_create", I32, [P(RdConfig), P(VP)])
    _proto(lib, "rd_chain_destroy", None, [VP])
    _proto(lib, "rd_chain_set_coeff", I32, [VP, VP])
    _proto(lib, "rd_chain_set_weights", I32, [VP, VP])
    _proto(lib, "rd_chain_set_pairs", I32, [VP, VP, VP, U32])
    _proto(lib, "rd_chain_process", I32, [VP, VP, U64, U64, P(RdOutput)])
    _proto(lib, "rd_chain_process_device", I32, [VP, VP, U64, U64, VP])
    _proto(lib, "rd_chain_fetch", I32, [VP, P(RdOutput)])
    _proto(lib, "rd_chain_last_launches", U64, [VP])
    _proto(lib, "rd_chain_flush_cov", I32, [VP, P(RdOutput)])
    _proto(lib, "rd_chain_set_profiling", I32, [VP, I32])
    _proto(lib, "rd_chain_kernel_times", I32, [VP, P(RdKernelTime), U32, P(U32)])
    _proto(lib, "rd_chain_stats", I32, [VP, P(RdStats)])
    _proto(lib, "rd_chain_read_history", I32, [VP, U32, U32, VP, P(U32), P(U32)])
    _proto(lib, "rd_chain_reset", I32, [VP, VP])
    _proto(lib, "rd_chain_set_history_depth", I32, [VP, U32])
    _proto(lib, "rd_chain_state_size", U64, [VP])
    _proto(lib, "rd_chain_save_state", I32, [VP, VP, U64])
    _proto(lib, "rd_chain_load_state", I32, [VP, VP, U64])
    _proto(lib, "rd_egress_merge", I32, [P(RdEgressSource), U32, U32, U32, VP, U64, VP, VP, VP])
    _proto(lib, "rd_batch_egress", I32, [VP, U32, VP, U64, VP, VP, VP])
    _proto(lib, "rd_route_path", I32, [U32, U32, U32, U32, VP])
    _proto(lib, "rd_chain_doppler", I32, [VP, U32, U32, VP, VP])
    _proto(lib, "rd_chain_set_launch_frames", I32, [VP, U32])
    _proto(lib, "rd_chain_footprint", U64, [P(RdConfig), U64])
    _proto(lib, "rd_batch_create", I32, [U32, P(RdConfig), VP, VP, P(RdBatchOptions), P(VP)])
    _proto(lib, "rd_batch_destroy", None, [VP])
    _proto(lib, "rd_batch_run", I32, [VP, VP, VP, VP])
    _proto(lib, "rd_batch_run_sequential", I32, [VP, VP, VP, VP])
    _proto(lib, "rd_batch_fetch", I32, [VP, U32, P(RdOutput)])
    _proto(lib, "rd_batch_set_outputs", I32, [VP, P(RdOutput)])
    _proto(lib, "rd_batch_results", I32, [VP, U32, P(RdOutput)])
    _proto(lib, "rd_batch_tune", I32, [VP, VP, VP, U32, P(RdBatchOptions), P(C.c_double)])
    _proto(lib, "rd_batch_tune_cached", I32, [VP, VP, VP, U32, C.c_char_p, P(RdBatchOptions),
                                              P(C.c_double), P(C.c_int)])
    _proto(lib, "rd_server_create", I32, [P(RdServerConfig), P(VP)])
    _proto(lib, "rd_server_destroy", None, [VP])
    _proto(lib, "rd_stream_open", I32, [VP, P(RdConfig), VP, VP, P(U32)])
    _proto(lib, "rd_stream_close", I32, [VP, U32])
    _proto(lib, "rd_stream_set_pairs", I32, [VP, U32, VP, VP, U32])
    _proto(lib, "rd_server_submit", I32, [VP, U32, VP, U64, U64, P(U64)])
    _proto(lib, "rd_server_poll", I32, [VP, P(RdCompletion), U32, P(U32)])
    _proto(lib, "rd_server_take", I32, [VP, U64, P(RdOutput)])
    _proto(lib, "rd_server_info_get", I32, [VP, P(RdServerInfo)])
    _proto(lib, "rd_server_run_trace", I32, [VP, U64, VP, VP, VP, VP, VP, P(C.c_double)])
    _proto(lib, "rd_pfb_run", I32, [U32, U32, VP, VP, VP, U32, VP, VP])
    _proto(lib, "rd_fft_run", I32, [U32, U32, U32, I32, VP, U32, VP, VP, VP])
    _proto(lib, "rd_bf_run", I32, [U32, U32, VP, VP, U64, VP, VP, VP, U32])
    _proto(lib, "rd_power_run", I32, [VP, U64, VP])
    _proto(lib, "rd_cross_power_run", I32, [VP, VP, U64, VP])
    _proto(lib, "rd_cfar_run", I32, [VP, U32, U32, P(RdConfig), VP, VP, U64, P(U64)])
    _proto(lib, "rd_cfar_run_static", I32, [VP, U32, U32, P(RdConfig), VP, VP, U64, VP, VP])
    _proto(lib, "rd_packetize", I32, [VP, U64, U32, U32, U32, U32, U32, VP])
    _proto(lib, "rd_fxp_apply", I32, [VP, VP, VP, VP, VP, U64, VP, VP])
    _proto(lib, "rd_last_error", C.c_char_p, [])
    _proto(lib, "rd_device_ok", I32, [])
    _proto(lib, "rd_version", C.c_char_p, [])


# Every function include/rd_chain.h declares (checked by the CPU tests).
EXPORTED = [
    "rd_config_default", "rd_config_validate", "rd_flit_words", "rd_detection_flits",
    "rd_cov_pairs", "rd_chain_create", "rd_chain_destroy", "rd_chain_set_coeff",
    "rd_chain_set_weights", "rd_chain_set_pairs", "rd_chain_process",
    "rd_chain_process_device", "rd_chain_fetch", "rd_chain_last_launches",
    "rd_chain_flush_cov", "rd_chain_set_profiling", "rd_chain_kernel_times", "rd_chain_stats",
    "rd_chain_reset", "rd_chain_set_history_depth", "rd_chain_state_size", "rd_chain_save_state", "rd_chain_load_state",
    "rd_chain_set_launch_frames", "rd_chain_footprint", "rd_chain_doppler",
    "rd_egress_merge", "rd_route_path",
    "rd_batch_create", "rd_batch_destroy", "rd_batch_run", "rd_batch_run_sequential",
    "rd_batch_fetch", "rd_batch_set_outputs", "rd_batch_results", "rd_batch_tune", "rd_batch_tune_cached", "rd_batch_egress", "rd_server_create",
    "rd_server_destroy", "rd_stream_open",
    "rd_stream_close", "rd_stream_set_pairs", "rd_server_submit", "rd_server_poll", "rd_server_take",
    "rd_server_info_get", "rd_server_run_trace", "rd_chain_read_history", "rd_pfb_run",
    "rd_fft_run", "rd_bf_run", "rd_power_run", "rd_cross_power_run", "rd_cfar_run", "rd_cfar_run_static",
    "rd_packetize", "rd_fxp_apply", "rd_last_error", "rd_device_ok", "rd_version",
]

_LIB = None


def load(path: str | os.PathLike | None = None):
    """Loads the CUDA library. Raises when it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    declare_rd(lib)
    if path is None:
        _LIB = lib
    return lib


def check(lib, status: int, what: str = "") -> None:
    if status != RD_OK:
        msg = lib.rd_last_error()
        raise RuntimeError(f"{what}: {STATUS_NAMES.get(status, status)}: "
                           f"{msg.decode() if msg else ''}")
