"""One rank of tests/test_bench_ranks.py::test_gpu_arm_rank_logic_two_ranks
(launched by torch.distributed.run; not a test module): the GPU arm's
host-side multi-rank steps on gloo, written as JSON to
$RANK_OUT_DIR/rank<r>.json (the ranks' stdout would interleave)."""
import json
import os
import sys
from pathlib import Path

import numpy as np
import torch
import torch.distributed as dist

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "agilex-7-radar-detect_gb300"))

import bench  # noqa: E402
from rdgb import scenario as sc  # noqa: E402

rank = int(os.environ["RANK"])
dist.init_process_group("gloo")
p = sc.preset("tiny")
_, x = bench.workload_input(torch, p, 1, 1, seed=p.seed + rank)  # as run_gpu seeds it
digest = int(np.bitwise_xor.reduce(x.reshape(-1).astype(np.uint64) * np.uint64(2654435761)))
dist.barrier()
t = bench.max_over_ranks(torch, dist, 10.0 + 7.5 * rank)
(Path(os.environ["RANK_OUT_DIR"]) / f"rank{rank}.json").write_text(
    json.dumps({"rank": rank, "digest": digest, "t": t}))
dist.destroy_process_group()
