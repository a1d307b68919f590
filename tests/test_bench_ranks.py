"""The bench's multi-process contract on CPU: under torchrun with two ranks
the reference arm runs on rank 0 alone, which prints one JSON line; the
other rank exits 0 without work (the GPU arm's ranks are independent
replicas, so there is no data-path collective to test)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks():
    pytest.importorskip("torch")
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--workload", "tiny",
           "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


def test_gpu_arm_rank_logic_two_ranks(tmp_path):
    # the GPU arm's host-side multi-rank logic on two gloo ranks
    # (tests/rank_child.py): each rank's inputs come from its own seed, and
    # the time every rank reports is the slowest rank's (bench.max_over_ranks
    # after the barrier, as bench.run_gpu does)
    pytest.importorskip("torch")
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    env["RANK_OUT_DIR"] = str(tmp_path)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "tests" / "rank_child.py")]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in range(2)]
    assert [g["rank"] for g in got] == [0, 1]
    assert got[0]["digest"] != got[1]["digest"]          # a stream per replica
    assert got[0]["t"] == got[1]["t"] == 17.5            # the slowest rank's time
