"""The bench's roofline inputs read from the committed ncu summaries: the
dominant kernel's DRAM bytes and warp instructions per launch parse, and
they are consistent with the launch they describe (traffic between a tenth
and twice the algorithmic bytes of the launch)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "agilex-7-radar-detect_gb300"))

import bench  # noqa: E402
from rdgb import scenario as sc  # noqa: E402


def test_profile_lines_parse():
    traffic = bench.profile_line("medium", "traffic", "k_front")
    inst = bench.profile_line("medium", "instructions", "k_front")
    assert traffic is not None and inst is not None
    assert bench.profile_line("medium", "traffic", "no_such_kernel") is None
    assert bench.profile_line("medium", "instructions", "no_such_kernel") is None
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=4096)
    alg = bench.kernel_bytes(cfg, "k_front", 4096)
    assert alg == 4096 * p.n_fft * p.n_chan * 8
    assert 0.1 * alg < traffic < 2 * alg
    # a few hundred warp instructions per sample group is the front end's range
    assert 1e7 < inst < 1e9


def _args(*argv):
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py", *argv]
        return bench.args_()
    finally:
        sys.argv = sys_argv


def test_bench_default_launch_matches_profile():
    # the medium summary describes launches of the bench's medium size
    text = (ROOT / "profiles" / "kernels_medium_ncu_full.md").read_text()
    a = _args("--workload", "medium")
    assert a.max_frames == 4096 and a.form == "cuda_core"
    assert f"{a.max_frames} frames" in text


def test_bench_defaults_full_scale():
    # no flags: the full-scale workload in the tensor form, 1024-frame launches
    a = _args()
    assert (a.workload, a.form, a.max_frames, a.gpus) == ("full", "tensor", 1024, 1)
    p = sc.preset("full")
    cfg = sc.make_config(p, max_frames=1024, form=1)
    # the tcgen05 beamformer's four limb GEMMs of one launch: 1024 x 1024 rows
    # x 128 columns (64 beams, re and im) x 128 deep (64 channels, re and im)
    assert bench.kernel_tensor_flops(cfg, "k_beam", 1024, 2080) == 2.0 * 1024 * 1024 * 4 * 128 * 128
    # the tcgen05 covariance: per bin and frame, four 128 x 64 GEMMs of depth 2
    assert bench.kernel_tensor_flops(cfg, "k_cov", 1024, 2080) == \
        2.0 * 1024 * 1024 * 4 * 128 * 64 * 2
    # the warp-level covariance's Gram tiles: 10 of the 16 16x16 channel tiles
    cfg_w = sc.make_config(p, max_frames=1024, form=2)
    assert bench.kernel_tensor_flops(cfg_w, "k_cov", 1024, 2080) == \
        2.0 * 1024 * 1024 * 4 * 10 * 16 * 16 * 6


def test_full_profile_lines():
    # the full-scale summary: the front stage's launch of 1024 frames x 64
    # channels x 1024 phases (the PFB pass and the FFT kernel), its DRAM bytes
    # the algorithmic 8 B a sample plus the PFB outputs written and read back
    # (within a tenth of 16 B a sample), and a few hundred thread
    # instructions a sample
    p = sc.preset("full")
    cfg = sc.make_config(p, max_frames=1024)
    alg = bench.kernel_bytes(cfg, "k_front", 1024)
    traffic = bench.profile_line("full", "traffic", "k_front")
    inst = bench.profile_line("full", "instructions", "k_front")
    assert 1.8 * alg < traffic < 2.2 * alg
    assert 100 < inst * 32 / (1024 * 1024 * 64) < 1000
    assert "1024 frames" in (ROOT / "profiles" / "chain_full_ncu.md").read_text()
