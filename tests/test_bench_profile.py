"""The bench's roofline inputs read from the committed ncu summary: the
dominant kernel's DRAM bytes and warp instructions per launch parse, and
they are consistent with the launch they describe (traffic between a tenth
and twice the algorithmic bytes of a 4096-frame medium launch)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "agilex-7-radar-detect_gb300"))

import bench  # noqa: E402
from rdgb import scenario as sc  # noqa: E402


def test_profile_lines_parse():
    traffic = bench.profile_traffic("k_front")
    inst = bench.profile_instructions("k_front")
    assert traffic is not None and inst is not None
    assert bench.profile_traffic("no_such_kernel") is None
    assert bench.profile_instructions("no_such_kernel") is None
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=4096)
    alg = bench.kernel_bytes(cfg, "k_front", 4096)
    assert alg == 4096 * p.n_fft * p.n_chan * 8
    assert 0.1 * alg < traffic < 2 * alg
    # a few hundred warp instructions per sample group is the front end's range
    assert 1e7 < inst < 1e9


def test_bench_default_launch_matches_profile():
    # the summary describes launches of the bench's default size
    text = (ROOT / "profiles" / "kernels_medium_ncu_full.md").read_text()
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        a = bench.args_()
    finally:
        sys.argv = sys_argv
    assert f"{a.max_frames} frames" in text
