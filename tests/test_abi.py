"""The C ABI library: it builds, loads and exports every function that
include/rd_chain.h declares; its host-only entry points behave without a GPU;
compute entry points fail loudly (no CPU fallback) when no device is usable."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from rdgb import abi, scenario as sc

ROOT = Path(__file__).resolve().parent.parent


def declared():
    txt = (ROOT / "include" / "rd_chain.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(rd_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert sorted(abi.EXPORTED) == declared()


@pytest.fixture(scope="module")
def lib():
    from rdgb import build
    build.build()
    return abi.load()


def test_library_exports_every_symbol(lib):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (rd_[a-z0-9_]+)$", out, flags=re.M))
    missing = [s for s in declared() if s not in exported]
    assert missing == []


def test_config_validation(lib):
    c = abi.RdConfig()
    lib.rd_config_default(C.byref(c))
    assert lib.rd_config_validate(C.byref(c)) == abi.RD_OK
    for name in ("tiny", "medium", "full", "ref_tiny"):
        cfg = sc.make_config(sc.preset(name))
        assert lib.rd_config_validate(C.byref(cfg)) == abi.RD_OK, name
    for field, bad in (("n_fft", 100), ("n_fft", 2048), ("spc", 3), ("hist_frames", 2),
                       ("taps", 0), ("packet_w", 48), ("cov_acc_w", 20), ("n_chan", 0)):
        cfg = sc.make_config(sc.preset("tiny"))
        setattr(cfg, field, bad)
        assert lib.rd_config_validate(C.byref(cfg)) == abi.RD_EINVAL, field
        assert lib.rd_last_error()


def test_tensor_form_channel_limit(lib):
    # the tensor form's exactness bound: at most RD_TC_MAX_CHAN channels
    assert abi.RD_TC_MAX_CHAN == 128
    cfg = sc.make_config(sc.preset("tiny"), form=abi.RD_FORM_TENSOR)
    assert lib.rd_config_validate(C.byref(cfg)) == abi.RD_OK
    cfg.n_chan = abi.RD_TC_MAX_CHAN + 1
    assert lib.rd_config_validate(C.byref(cfg)) == abi.RD_EINVAL
    n = abi.RD_TC_MAX_CHAN + 1
    w = np.zeros(n, np.uint32)
    y = np.zeros(1, np.uint32)
    st = lib.rd_bf_run(n, 1, w.ctypes.data, w.ctypes.data, 1, y.ctypes.data, None, None,
                       abi.RD_FORM_TENSOR)
    assert st == abi.RD_EINVAL and b"tensor form" in lib.rd_last_error()


def test_geometry_helpers(lib):
    # packet_model.hpp:118-127: 1 + ceil(176 / W) flits of W + 5 bits
    assert [lib.rd_detection_flits(w) for w in (64, 128, 512)] == [4, 3, 2]
    assert [lib.rd_flit_words(w) for w in (64, 128, 512)] == [3, 5, 17]
    for name, pairs in (("tiny", 10), ("medium", 136), ("full", 2080)):
        assert lib.rd_cov_pairs(C.byref(sc.make_config(sc.preset(name)))) == pairs


def test_no_cpu_fallback(lib):
    if lib.rd_device_ok():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    cfg = sc.make_config(sc.preset("tiny"))
    assert lib.rd_chain_create(C.byref(cfg), C.byref(h)) == abi.RD_EDEVICE
    assert b"device" in lib.rd_last_error()
    x = np.zeros(64, np.uint32)
    assert lib.rd_fft_run(64, 2, 0xFFFFFFFF, 1, abi.ptr(x), 1, abi.ptr(x), None, None) == abi.RD_EDEVICE


def test_footprint(lib):
    """rd_chain_footprint, the figure the server admits streams against: 0
    for an invalid configuration; linear in the launch size, by exactly the
    per-frame buffers of the data layout (spectrum ring, power cells, CFAR
    counts and emit mask, PFB pass outputs); more with covariance on and
    with the tensor form's operands; never below the resident buffers."""
    bad = sc.make_config(sc.preset("tiny"))
    bad.n_fft = 12
    assert lib.rd_chain_footprint(C.byref(bad), 16) == 0
    for name in ("tiny", "medium", "full"):
        p = sc.preset(name)
        N, Cn, B, D, H = p.n_fft, p.n_chan, p.n_beams, p.taps - 1, p.hist_frames

        def fp(frames, form=abi.RD_FORM_CUDA_CORE, cov=True, per_call=16):
            cfg = sc.make_config(p, max_frames=frames, form=form)
            if not cov:
                cfg.cov_source = abi.RD_COV_OFF
            return lib.rd_chain_footprint(C.byref(cfg), per_call)

        per_frame = N * Cn * 4 + B * N * 4 + B * 20 + B * ((N + 31) // 32) * 4 + Cn * N * 4
        assert fp(1024) - fp(256) == 768 * per_frame, name
        assert fp(4096) - fp(1024) == 3072 * per_frame, name
        for f in (256, 4096):
            resident = (f + H) * N * Cn * 4 + f * B * N * 4 + 2 * Cn * D * N * 4
            assert fp(f) > resident, (name, f)
            assert fp(f, form=abi.RD_FORM_TENSOR) > fp(f) > fp(f, cov=False), (name, f)
            assert fp(f, per_call=256) >= fp(f, per_call=16), (name, f)
