"""rd_cfar_run_static: the CFAR entry point for callers that may not allocate
device memory (they are handed buffers by another framework's pool, or run in
a loop where cudaMalloc would stall the device). It keeps its scratch in a
static device array; this test checks, through the C ABI, that its events
equal those of the allocating entry point rd_cfar_run on two calls in a row
(the second with different data and sizes, so stale scratch would show), and
that sizes beyond the static scratch are refused.

The test allocates its own input and output buffers with torch - it stands in
for the caller's framework - and the entry point under test only receives
them. This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu


def _cfg(mode, out_mode, gl, gg, rl, rg, alpha, mg=4, mr=16):
    c = sc.make_config(sc.preset("tiny"))
    c.cfar_mode, c.cfar_out_mode = mode, out_mode
    c.guard_lead, c.guard_lag, c.ref_lead, c.ref_lag = gl, gg, rl, rg
    c.alpha, c.max_guard, c.max_ref = alpha, mg, mr
    return c


def _run_static(lib, torch, cells, n, cfg, fid, cap):
    frames = cells.size // n
    d_cells = torch.from_numpy(np.ascontiguousarray(cells, np.int64)).cuda()
    d_fid = torch.from_numpy(np.ascontiguousarray(fid, np.uint32).view(np.int32)).cuda()
    d_ev = torch.zeros(max(cap, 1) * 32, dtype=torch.uint8, device="cuda")
    d_n = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    st = lib.rd_cfar_run_static(C.c_void_p(d_cells.data_ptr()), n, frames, C.byref(cfg),
                                C.c_void_p(d_fid.data_ptr()), C.c_void_p(d_ev.data_ptr()), cap,
                                C.c_void_p(d_n.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert st == abi.RD_OK, lib.rd_last_error()
    torch.cuda.synchronize()
    n_ev = int(d_n.item())
    ev = d_ev.cpu().numpy().view(abi.EVENT_DTYPE)[: min(n_ev, cap)]
    return n_ev, ev


def test_static_cfar_matches_allocating_entry_point(gpulib):
    torch = pytest.importorskip("torch")
    lib = gpulib
    rng = np.random.default_rng(2026)
    cases = [
        (256, 64, _cfg(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS, 2, 2, 8, 8, 2000)),
        (1024, 37, _cfg(abi.RD_CFAR_GO, abi.RD_CFAR_DENSE, 4, 1, 16, 5, 3000)),
        # short frames (several a warp) up to the scratch's frame limit
        (16, abi.RD_STATIC_CFAR_MAX_FRAMES, _cfg(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS, 1, 1, 4, 4, 2600)),
        (47, 301, _cfg(abi.RD_CFAR_GO, abi.RD_CFAR_DENSE, 1, 2, 6, 3, 1900)),
    ]
    for n, frames, cfg in cases:  # two calls in a row on the shared scratch
        cells = rng.exponential(1000.0, frames * n).astype(np.int64)
        cells[rng.integers(0, cells.size, 25)] *= 50
        cells[:2] = [-7, 2**31]
        fid = rng.integers(0, 2**16, frames).astype(np.uint32)
        want = gc.cfar(cells, n, cfg, fid)
        cap = frames * (n + 1)
        n_ev, got = _run_static(lib, torch, cells, n, cfg, fid, cap)
        assert n_ev == len(want)
        assert np.array_equal(got, want)


def test_static_cfar_rejects_oversize(gpulib):
    lib = gpulib
    cfg = _cfg(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS, 2, 2, 8, 8, 2000)
    dummy = C.c_void_p(8)  # never dereferenced: the sizes are refused first
    st = lib.rd_cfar_run_static(dummy, abi.RD_STATIC_CFAR_MAX_CELLS + 1, 1, C.byref(cfg), dummy,
                                dummy, 1, dummy, None)
    assert st == abi.RD_EINVAL and b"static scratch" in lib.rd_last_error()
    st = lib.rd_cfar_run_static(dummy, 64, abi.RD_STATIC_CFAR_MAX_FRAMES + 1, C.byref(cfg), dummy,
                                dummy, 1, dummy, None)
    assert st == abi.RD_EINVAL and b"static scratch" in lib.rd_last_error()
