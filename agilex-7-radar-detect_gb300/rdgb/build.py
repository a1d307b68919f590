"""Builds the CUDA library librdgb.so in-tree for sm_103a with nvcc.

Translation units compile in parallel, then link into one shared object with
the CUDA runtime linked statically. No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

from . import abi

CSRC = abi.PKG_ROOT / "csrc"
SOURCES = ["k_frontend.cu", "k_front_fast.cu", "k_front_fast_256.cu", "k_front_fast_1024.cu",
           "k_backend.cu", "k_beam_tc.cu", "k_beam_t5.cu", "k_cov_tc.cu", "k_cov_t5.cu", "k_pfb_rows.cu",
           "k_engine.cu",
           "cfar_static.cu", "batch.cu", "server.cu", "fabric.cu", "api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: Path, deps: list[Path]) -> bool:
    return target.exists() and all(target.stat().st_mtime >= d.stat().st_mtime for d in deps)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> Path:
    out = abi.LIB_PATH
    out.parent.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(CSRC.glob("*.inc")) + \
        [abi.PKG_ROOT.parent / "include" / "rd_chain.h"]
    cc = nvcc()
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = out.parent / (s.stem + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(subprocess.run, cmd, capture_output=True, text=True) for cmd in jobs]
        for cmd, f in zip(jobs, futs):
            r = f.result()
            if verbose or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    if force or jobs or not _newer(out, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return out


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
