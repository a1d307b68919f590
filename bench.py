#!/usr/bin/env python
"""Throughput of the bit-exact radar chain on GB300.

One step = one pass of the whole chain (PFB -> FFT -> history/corner turn ->
align -> beamform -> power + covariance -> CFAR -> events -> packet flits) over
the medium workload: 16 channels x 64 CPIs x 65536 complex int16 samples per
channel (seeded synthetic ADC data), one stream. The input (268 MB, larger
than L2) is resident in HBM before the timed region; every step processes all
of it. `e2e` times the same work through the C ABI from pinned host buffers,
with the host->device copies and the result reads inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Under torchrun with N > 1 every rank runs an independent replica of the
workload (streams shard across GPUs; there is no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "agilex-7-radar-detect_gb300"))

import numpy as np  # noqa: E402

METRIC = "bit-exact chain Msamples/s on 1 GB300 (TC vs plain int), %HBM roofline; p99 latency"
UNIT = "Msamples/s"


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", default="medium")
    ap.add_argument("--cpis", type=int, default=None, help="CPIs per step (default: the workload's)")
    ap.add_argument("--max-frames", type=int, default=1024)
    ap.add_argument("--form", choices=["cuda_core", "tensor"], default="cuda_core")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def peaks() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the run."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def kernel_bytes(cfg, name: str, frames: int) -> float:
    """Algorithmic HBM bytes of one launch over `frames` frames."""
    N, C, B = cfg.n_fft, cfg.n_chan, cfg.n_beams
    if name == "k_front":      # ADC read + spectrum (history ring) write
        return frames * N * C * 8.0
    if name == "k_beam":       # spectrum read + power cells write
        return frames * N * (C + B) * 4.0
    if name == "k_cov":        # spectrum read (windows amortise to ~0)
        return frames * N * C * 4.0
    if name == "k_cfar_decide":  # power cells read
        return frames * N * B * 4.0
    return 0.0


def profile_traffic(kernel: str) -> float | None:
    """dram read+write bytes per launch of `kernel` at the bench's launch size,
    from the committed ncu summary of the medium chain (a line
    `traffic <kernel> dram_bytes_per_launch=<bytes>`), or None."""
    import re
    f = ROOT / "profiles" / "kernels_medium_ncu_full.md"
    if f.exists():
        m = re.search(rf"^traffic {re.escape(kernel)} dram_bytes_per_launch=(\d+)$",
                      f.read_text(), re.M)
        if m:
            return float(m.group(1))
    return None


def cpu_baseline(p, cfg, coeff, w, pairs, x, cpis: int) -> dict:
    sys.path.insert(0, str(ROOT / "oracle"))
    import orc

    if not orc.available("port"):
        orc.build("port")
    o = orc.Oracle("port")
    threads = os.cpu_count() or 1
    n = cpis * p.cpi_samples
    ch = o.chain(cfg, coeff, w, pairs[0], pairs[1])
    t = time.perf_counter()
    ch.process(x[:, :n], taps=False, threads=threads)
    dt = time.perf_counter() - t
    n1 = p.cpi_samples // 4
    ch1 = o.chain(cfg, coeff, w, pairs[0], pairs[1])
    t = time.perf_counter()
    ch1.process(x[:, :n1], taps=False, threads=1)
    dt1 = time.perf_counter() - t
    return {"value": round(p.n_chan * n / dt / 1e6, 3), "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{cpis} CPIs x {p.n_chan} ch x {p.cpi_samples} samples of the same "
                      f"workload through oracle/orc_port.c with {threads} threads",
            "single_thread_value": round(p.n_chan * n1 / dt1 / 1e6, 3)}


def run_reference(a, rank: int, world: int) -> None:
    """The reference arm: the reference's chain on host cores. The reference
    model (C++ headers) cannot be built on the GPU host (no reference
    checkout there and no cross toolchain here), so its plain-C restatement,
    pinned against the reference's own outputs, stands in."""
    if rank != 0:
        return
    from rdgb import scenario as sc

    sys.path.insert(0, str(ROOT / "oracle"))
    import orc

    if not orc.available("port"):
        orc.build("port")
    p = sc.preset(a.workload)
    cfg = sc.make_config(p, max_frames=a.max_frames)
    pairs = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    cpis = 4 if a.workload == "medium" else 1
    n = cpis * p.cpi_samples
    x = sc.adc(p, n)
    o = orc.Oracle("port")
    threads = os.cpu_count() or 1
    times = []
    for i in range(a.warmup + a.steps):
        ch = o.chain(cfg, coeff, w, pairs[0], pairs[1])
        t = time.perf_counter()
        ch.process(x, taps=False, threads=threads)
        if i >= a.warmup:
            times.append(time.perf_counter() - t)
    ms = 1e3 * sum(times) / len(times)
    v = p.n_chan * n / (ms / 1e3) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT,
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (seeded tones + chirp + noise, complex int16 12-bit range)",
            "config": {"workload": f"{a.workload}: {p.n_chan} ch, {p.n_fft}-point PFB x {p.taps} taps, "
                                   f"{p.n_fft}-point FFT, {p.hist_frames}-frame history, {p.n_beams} beams, "
                                   f"{p.n_chan}x{p.n_chan} covariance, CA-CFAR; step = {cpis} CPIs "
                                   f"of {p.cpi_samples} samples/ch (bounded sample)"},
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{cpis} CPIs of the {a.workload} workload per step"},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(a, rank: int, world: int, local: int) -> None:
    import torch

    from rdgb import abi, chain as gc, scenario as sc

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    p = sc.preset(a.workload)
    cpis = a.cpis or p.n_cpi
    n = cpis * p.cpi_samples
    form = abi.RD_FORM_TENSOR if a.form == "tensor" else abi.RD_FORM_CUDA_CORE
    cfg = sc.make_config(p, max_frames=a.max_frames, form=form)
    pairs = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    x = sc.adc(p, n, seed=p.seed + rank)  # each replica its own stream
    host = torch.from_numpy(x.view(np.int32)).pin_memory()
    dev = host.cuda()
    samples = p.n_chan * n
    chain = gc.Chain(cfg, coeff, w, pairs)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream

    for _ in range(a.warmup):
        chain.process_device(dev.data_ptr(), n, n, sh)
    torch.cuda.synchronize()
    warm = chain.fetch(n // p.n_fft, cap_events=n // p.n_fft * p.n_beams * 8)
    n_events = len(warm["events"])

    # timed region: inputs larger than L2 (no flush needed)
    chain.L.rd_chain_set_profiling(chain.h, 1)
    kt = (abi.RdKernelTime * 16)()
    nk = abi.C.c_uint32(0)
    chain.L.rd_chain_kernel_times(chain.h, kt, 16, abi.C.byref(nk))  # reset
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps + 1)]
    evs[0].record(stream)
    launches = 0
    for i in range(a.steps):
        chain.process_device(dev.data_ptr(), n, n, sh)
        launches += chain.last_launches()
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    step_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(a.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    chain.L.rd_chain_kernel_times(chain.h, kt, 16, abi.C.byref(nk))
    kernels = {kt[i].name.decode(): {"launches": int(kt[i].launches),
                                     "avg_ms": kt[i].total_ms / max(kt[i].launches, 1),
                                     "total_ms": kt[i].total_ms} for i in range(nk.value)}
    chain.L.rd_chain_set_profiling(chain.h, 0)
    t_max = total_ms
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * samples * a.steps / (t_max / 1e3) / 1e6

    # roofline of the dominant kernel
    dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
    frames_total = n // p.n_fft
    per_launch_frames = frames_total / max(kernels[dom]["launches"] / a.steps, 1)
    alg = kernel_bytes(cfg, dom, per_launch_frames)
    peak, which = peaks()
    achieved = alg / (kernels[dom]["avg_ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"of {which}",
                "traffic": profile_traffic(dom),
                "algorithmic_bytes_per_launch": alg}

    # e2e through the C ABI from pinned host memory
    e2e = None
    if not a.no_e2e:
        cap = max(4 * n_events, 1024)
        out = gc.Outputs(cfg, n // p.n_fft, chain.n_pairs, False, cap)
        adc_ptr = abi.C.c_void_p(host.data_ptr())
        times = []
        for i in range(max(2, a.warmup) + a.steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            abi.check(chain.L, chain.L.rd_chain_process(chain.h, adc_ptr, n, n, abi.C.byref(out.c)),
                      "rd_chain_process")
            if i >= max(2, a.warmup):
                times.append(time.perf_counter() - t)
        ms = 1e3 * sum(times) / len(times)
        words = (cfg.packet_w + 5 + 31) // 32
        d2h = (out.c.n_events * 32 + out.c.n_flits * words * 4 +
               out.c.n_cov_windows * (16 + p.n_fft * chain.n_pairs * 16))
        e2e_ms = ms
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = {"value": round(world * samples / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": samples * 4, "d2h_bytes_per_step": int(d2h),
               "ms_per_step": round(e2e_ms, 3)}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if not a.no_cpu_baseline:
        cpu = cpu_baseline(p, cfg, coeff, w, pairs, x, cpis=min(16, cpis))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(t_max / a.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": "synthetic (seeded tones + chirp + noise, complex int16 12-bit range)",
        "config": {"workload": f"{a.workload}: {p.n_chan} ch, {p.n_fft}-point PFB x {p.taps} taps, "
                               f"{p.n_fft}-point FFT (spc {p.spc}), {p.hist_frames}-frame history, "
                               f"{p.n_beams} beams, {p.n_chan}x{p.n_chan} covariance over "
                               f"{p.cov_window} frames, CA-CFAR ref {p.ref[0]}/guard {p.guard[0]} per side; "
                               f"{cpis} CPIs x {p.cpi_samples} samples/ch per step",
                   "form": a.form, "frames_per_launch": a.max_frames,
                   "input_bytes": samples * 4, "l2": "inputs larger than L2 (no flush)"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": launches,
        "kernels": {k: {"launches": v["launches"], "avg_us": round(1e3 * v["avg_ms"], 2),
                        "share": round(v["total_ms"] / sum(x["total_ms"] for x in kernels.values()), 4)}
                    for k, v in kernels.items()},
        "step_ms": [round(s, 4) for s in step_ms],
        "events_per_step": n_events,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    a = args_()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(a.gpus if a.gpus == 1 else 1)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if a.impl == "reference":
        run_reference(a, rank, world)
    else:
        run_gpu(a, rank, world, local)


if __name__ == "__main__":
    main()
