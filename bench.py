#!/usr/bin/env python
"""Throughput of the bit-exact radar chain on GB300.

One step = one pass of the whole chain (PFB -> FFT -> history/corner turn ->
align -> beamform -> power + covariance -> CFAR -> events -> packet flits) over
the full-scale workload: 64 channels x 16 CPIs x 2^20 complex int16 samples
per channel (seeded synthetic ADC data, 4.3 GB), one stream, 1024-point PFB x
16 taps, 1024-point FFT, 64 beams, 64x64 Hermitian covariance (2080 pairs)
over 256-frame windows, CA-CFAR, 512-bit packets; beamforming and covariance
in the limb-split tensor-core form. The input (larger than L2) is resident in
HBM before the timed region; every step processes all of it. `e2e` times the
same work through the C ABI from pinned host buffers, with the host->device
copies and the result reads (events, packets, every closed covariance window)
inside the timed region. `--workload medium` measures the medium workload
(16 channels, 64 CPIs of 65536 samples) instead.

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
# 32 hardware work queues instead of the default 8, set before the CUDA
# context exists: the batch's 32 streams and the server's streams otherwise
# share 8 queues and wait on one another's launches (batched 17.2 -> 14.4 ms)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

METRIC = "bit-exact chain Msamples/s on 1 GB300 (TC vs plain int), %HBM roofline; p99 latency"
UNIT = "Msamples/s"
# frames per launch by workload: the full workload's 1024 frames (67 M samples
# a launch) fill every kernel; the medium one needs 4096 (16.8 M)
LAUNCH_FRAMES = {"full": 1024, "medium": 4096, "tiny": 1024}
# CPIs the timed input holds that are generated distinct (the rest repeats
# them, so that generating 4.3 GB stays within seconds)
DISTINCT_CPIS = {"full": 4, "medium": 64, "tiny": 1}


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=["full", "medium", "tiny"], default="full")
    ap.add_argument("--cpis", type=int, default=None, help="CPIs per step (default: the workload's)")
    ap.add_argument("--max-frames", type=int, default=None,
                    help="frames per launch (default: 1024 at full scale, 4096 at medium)")
    ap.add_argument("--form", choices=["cuda_core", "tensor", "tensor_warp"], default=None,
                    help="default: tensor at full scale, cuda_core at medium")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-patterns", action="store_true",
                    help="skip the form comparison, batching and serving measurements")
    a = ap.parse_args()
    if a.max_frames is None:
        a.max_frames = LAUNCH_FRAMES[a.workload]
    if a.form is None:
        a.form = "tensor" if a.workload == "full" else "cuda_core"
    return a


def peaks() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bf16_peak() -> tuple[float, str]:
    """Dense bf16 TFLOP/s for a kernel timed alone: the measured burst figure,
    else the recipe's fallback."""
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        v = json.loads(f.read_text()).get("bf16_tflops")
        if v:
            return float(v), "of measured"
    return 1900.0, "of fallback"


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
    if name == "k_cfar":       # power cells read (events and packets come on top)
        return frames * N * B * 4.0
    return 0.0


def kernel_tensor_flops(cfg, name: str, frames: int, n_pairs: int) -> float:
    """fp16 tensor-core flops of one launch of a limb-split contraction. The
    tcgen05 beamformer (up to 64 channels) runs four GEMMs per 128-row tile
    (high x high, low x low and the two cross terms) of (frame, bin) rows,
    2 columns per beam (re, im; beams padded to groups of up to 32) and 2
    parts per channel of depth (padded to 16); the warp-level one has 6
    class columns per beam and 4 limb parts per channel. The tcgen05
    covariance (up to 64 channels, windows of 64-256 frames) runs four
    128 x 64 GEMMs ([U; V] rows against U columns, 64 // Sp bins of Sp
    channels a tile, Sp the channel count rounded up to a power of two >= 16)
    of depth 2 per frame; the warp-level one has 6 class columns per channel
    and 4 parts per frame of depth over the 16-channel tiles that hold a
    requested pair (the whole triangle of tiles for the full table)."""
    N, C, B = cfg.n_fft, cfg.n_chan, cfg.n_beams
    rows = frames * N
    if name == "k_beam":
        if cfg.form == 1 and C <= 64:
            nb = min(32, -(-B // 8) * 8)
            cols = 2 * nb * -(-B // nb)
            depth = -(-2 * C // 16) * 16
            return 2.0 * rows * 4 * cols * depth
        return 2.0 * rows * (6 * B) * (4 * C)
    if name == "k_cov":
        S = B if cfg.cov_source == 2 else C
        if cfg.form == 1 and S <= 64 and 64 <= cfg.cov_window <= 256:
            sp = 16
            while sp < S:
                sp *= 2
            tiles = -(-N // (64 // sp))
            return 2.0 * tiles * frames * 4 * 128 * 64 * 2
        t = -(-S // 16)
        tiles = t * (t + 1) // 2 if n_pairs >= S * (S + 1) // 2 else t * t
        return 2.0 * N * frames * 4 * tiles * 16 * 16 * 6
    return 0.0


def profile_line(workload: str, key: str, kernel: str) -> float | None:
    """A figure of one launch of `kernel` at the bench's launch size from the
    committed ncu summary of the workload's chain: a line
    `<key> <kernel> <name>=<value>` (instructions: smsp__inst_executed.sum;
    traffic: dram__bytes_read.sum + dram__bytes_write.sum), or None."""
    import re
    f = ROOT / "profiles" / {"medium": "kernels_medium_ncu_full.md",
                             "full": "chain_full_ncu.md"}[workload]
    if f.exists():
        m = re.search(rf"^{key} {re.escape(kernel)} \w+=(\d+)$", f.read_text(), re.M)
        if m:
            return float(m.group(1))
    return None


def cpu_baseline(p, cfg, coeff, w, pairs, x) -> dict:
    """The oracle port on the machine's host cores over a bounded sample of the
    same workload: the first CPI's first 256 frames (one covariance window)
    with every host thread, and its first 32 frames on one thread."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import orc

    if not orc.available("port"):
        orc.build("port")
    o = orc.Oracle("port")
    threads = os.cpu_count() or 1
    frames = min(256, x.shape[1] // p.n_fft)
    cap = lambda f: f * p.n_beams * (2 + p.n_fft // 16)  # noqa: E731
    n = frames * p.n_fft
    ch = o.chain(cfg, coeff, w, pairs[0], pairs[1])
    t = time.perf_counter()
    ch.process(x[:, :n], taps=False, threads=threads, cap_events=cap(frames))
    dt = time.perf_counter() - t
    n1 = max(1, frames // 8) * p.n_fft
    ch1 = o.chain(cfg, coeff, w, pairs[0], pairs[1])
    t = time.perf_counter()
    ch1.process(x[:, :n1], taps=False, threads=1, cap_events=cap(n1 // p.n_fft))
    dt1 = time.perf_counter() - t
    return {"value": round(p.n_chan * n / dt / 1e6, 3), "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{frames} frames x {p.n_fft} samples x {p.n_chan} ch of the same workload "
                      f"(one covariance window) through oracle/orc_port.c with {threads} threads; "
                      f"single_thread_value: {n1 // p.n_fft} frames on one thread",
            "single_thread_value": round(p.n_chan * n1 / dt1 / 1e6, 3)}


def tiled_adc(p, n: int, block: int = 65536):
    """Seeded tones + noise for `n` samples per channel: one generated block
    of `block` samples repeated (the statistics are the same)."""
    from rdgb import scenario as sc

    b = sc.adc(p, min(n, block))
    reps = -(-n // b.shape[1])
    return np.ascontiguousarray(np.tile(b, (1, reps))[:, :n])


def workload_input(torch, p, cpis: int, distinct: int, seed: int):
    """[C][cpis x cpi_samples] ADC samples in page-locked host memory (plain
    memory without a GPU): the first `distinct` CPIs of one seeded stream,
    repeated up to `cpis`."""
    from rdgb import scenario as sc

    n = cpis * p.cpi_samples
    host = torch.empty((p.n_chan, n), dtype=torch.int32, pin_memory=torch.cuda.is_available())
    h = host.numpy().view(np.uint32)
    d = min(distinct, cpis)
    h[:, :d * p.cpi_samples] = sc.adc(p, d * p.cpi_samples, seed=seed)
    for k in range(d, cpis, d):
        m = min(d, cpis - k) * p.cpi_samples
        h[:, k * p.cpi_samples:k * p.cpi_samples + m] = h[:, :m]
    return host, h


def time_chain(torch, chain, dev, n: int, stream, steps: int, warmup: int):
    """(ms per step, {kernel: avg us}) of process_device over `n` samples/ch."""
    from rdgb import abi

    sh = stream.cuda_stream
    for _ in range(warmup):
        chain.process_device(dev.data_ptr(), n, n, sh)
    torch.cuda.synchronize()
    chain.L.rd_chain_set_profiling(chain.h, 1)
    kt = (abi.RdKernelTime * 16)()
    nk = abi.C.c_uint32(0)
    chain.L.rd_chain_kernel_times(chain.h, kt, 16, abi.C.byref(nk))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        chain.process_device(dev.data_ptr(), n, n, sh)
    e1.record(stream)
    torch.cuda.synchronize()
    chain.L.rd_chain_kernel_times(chain.h, kt, 16, abi.C.byref(nk))
    chain.L.rd_chain_set_profiling(chain.h, 0)
    ks = {kt[i].name.decode(): round(1e3 * kt[i].total_ms / max(kt[i].launches, 1), 2)
          for i in range(nk.value)}
    return e0.elapsed_time(e1) / steps, ks


def run_forms(torch, a, stream) -> dict:
    """The chain in the CUDA-core integer form and in the limb-split
    tensor-core form, on the medium workload (the bench's frames per launch)
    and on the full-scale one (1024 frames, 67 M samples, per launch)."""
    from rdgb import abi, chain as gc, scenario as sc

    out = {}
    medium_frames = LAUNCH_FRAMES["medium"]
    for wl, cpis, frames in (("medium", 64, medium_frames), ("full", 2, 1024)):
        p = sc.preset(wl)
        n = cpis * p.cpi_samples
        x = tiled_adc(p, n)
        dev = torch.from_numpy(x.view(np.int32)).cuda()
        coeff = sc.coefficients(p.n_fft, p.taps)
        w = sc.steering_weights(p.n_chan, p.n_beams)
        r = {"samples_per_step": p.n_chan * n, "frames_per_launch": frames}
        pairs = sc.pair_table(p)
        rows = frames * p.n_fft  # (frame, bin) rows of one launch
        # int MACs a launch (4 B C a bin-frame for the beams, 4 per pair for the
        # covariance) and the limb GEMM's fp16 flops (6 B columns, 4 C depth)
        beam_mac, cov_mac = 4 * p.n_beams * p.n_chan * rows, 4 * len(pairs[0]) * rows
        beam_tc_flop = 2 * rows * (6 * p.n_beams) * (4 * p.n_chan)
        for name, form in (("cuda_core", abi.RD_FORM_CUDA_CORE), ("tensor", abi.RD_FORM_TENSOR)):
            ch = gc.Chain(sc.make_config(p, max_frames=frames, form=form), coeff, w, pairs)
            ms, ks = time_chain(torch, ch, dev, n, stream, steps=3, warmup=3)
            r[name] = {"value": round(p.n_chan * n / (ms / 1e3) / 1e6, 3), "unit": UNIT,
                       "ms_per_step": round(ms, 3), "k_beam_us": ks.get("k_beam"),
                       "k_cov_us": ks.get("k_cov")}
            if ks.get("k_beam") and ks.get("k_cov"):
                r[name]["beam_int_gmac_s"] = round(beam_mac / ks["k_beam"] / 1e3, 1)
                r[name]["cov_int_gmac_s"] = round(cov_mac / ks["k_cov"] / 1e3, 1)
                if form == abi.RD_FORM_TENSOR:
                    tf = beam_tc_flop / ks["k_beam"] / 1e6
                    peak, src = bf16_peak()
                    r[name]["beam_fp16_tflop_s"] = round(tf, 1)
                    r[name]["beam_fp16_frac"] = round(tf / peak, 4)
                    r[name]["beam_fp16_peak"] = f"{peak} TFLOP/s dense bf16, {src}"
            ch.close()
        cc, tc = r["cuda_core"], r["tensor"]
        r["chain_speedup"] = round(tc["value"] / cc["value"], 3)
        r["beam_cov_speedup"] = round((cc["k_beam_us"] + cc["k_cov_us"]) /
                                      (tc["k_beam_us"] + tc["k_cov_us"]), 3)
        out[wl] = r
        del dev
    out["note"] = ("tensor form: int16 samples and weights split into 8-bit limbs held exactly "
                   "in fp16, products on the tensor cores with fp32 accumulation of exact "
                   "integers, int64 recombine (tcgen05 with TMEM accumulators up to 64 "
                   "channels, else warp-level mma); per-launch stage times from CUDA events; "
                   "inputs: one 65536-sample seeded block per channel repeated")
    return out


def pinned_alloc(torch):
    """An Outputs allocator of page-locked host arrays: the device writes
    the results by DMA."""
    def alloc(shape, dtype):
        dt = np.dtype(dtype)
        k = int(np.prod(shape)) * dt.itemsize
        return torch.empty(k, dtype=torch.uint8, pin_memory=True).numpy().view(dt).reshape(shape)
    return alloc


def run_batching(torch, n_scen: int = 256, runs: int = 5) -> dict:
    """256 independent scenarios of seeded uneven geometry: one autotuned
    graph replay against the scenarios one after another on one stream."""
    from rdgb import abi, chain as gc, scenario as sc
    from rdgb.batch import Batch

    ps = sc.batch_scenarios(n_scen)
    # the tensor form for every scenario (bit-identical to the CUDA-core one);
    # buffers for a whole CPI, the launch size the tuner's (equal samples per
    # launch across FFT sizes), the sequential arm one launch per CPI
    cfgs = [sc.make_config(p, max_frames=p.frames_per_cpi, form=abi.RD_FORM_TENSOR) for p in ps]
    coeffs = [sc.coefficients(p.n_fft, p.taps) for p in ps]
    ws = [sc.steering_weights(p.n_chan, p.n_beams) for p in ps]
    devs = [torch.from_numpy(tiled_adc(p, p.cpi_samples, 8192).view(np.int32)).cuda()
            for p in ps]
    ptrs = [d.data_ptr() for d in devs]
    ns = [p.cpi_samples for p in ps]
    samples = sum(p.n_chan * p.cpi_samples for p in ps)
    b = Batch(cfgs, coeffs, ws, n_streams=16, use_graph=True)
    st = torch.cuda.Stream()
    b.run(ptrs, ns, st.cuda_stream)  # sizes every chain's buffers
    t = time.perf_counter()
    # the tuner's choice is kept on disk, keyed by the scenarios and the device
    opt, tuned_ms = b.tune(ptrs, ns, reps=3, cache=ROOT / "agilex-7-radar-detect_gb300" /
                           "_build" / "batch_tune_cache.txt")
    tune_s = time.perf_counter() - t

    def timed(sequential: bool) -> float:
        for _ in range(2):
            b.run(ptrs, ns, st.cuda_stream, sequential=sequential)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(runs):
            b.run(ptrs, ns, st.cuda_stream, sequential=sequential)
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / runs

    batched = timed(False)
    seq = timed(True)
    # the batched run with every scenario's results read back to the host, the
    # work of the per-scenario arm below
    n_pairs = [gc.lib().rd_cov_pairs(gc.C.byref(c)) for c in cfgs]

    # page-locked result buffers per scenario, sized from a first read and
    # reused by both arms: each then times the GPU work and the results'
    # device-to-host copies, not host allocation
    first = [b.fetch(i, p.frames_per_cpi, n_pairs[i]) for i, p in enumerate(ps)]
    outs = [gc.Outputs(c, p.frames_per_cpi, n_pairs[i], False,
                       max(2 * len(f["events"]), 1024), alloc=pinned_alloc(torch))
            for i, (c, p, f) in enumerate(zip(cfgs, ps, first))]
    del first
    L = gc.lib()

    # the batched run writes every scenario's results into them itself, each
    # as its launches end (rd_batch_set_outputs); the host then only reads
    # the counts (rd_batch_results)
    b.set_outputs(outs)

    def batched_fetch_once() -> float:
        torch.cuda.synchronize()
        t = time.perf_counter()
        b.run(ptrs, ns, st.cuda_stream)
        for i, o in enumerate(outs):
            abi.check(L, L.rd_batch_results(b.h, i, abi.C.byref(o.c)), "rd_batch_results")
        return 1e3 * (time.perf_counter() - t)

    batched_fetch_once()
    batched_fetch = min(batched_fetch_once() for _ in range(3))
    # the per-scenario API as a caller uses it: process, then read the results
    chains = [gc.Chain(c, co, w) for c, co, w in zip(cfgs, coeffs, ws)]

    def sequential_fetch_once() -> float:
        torch.cuda.synchronize()
        t = time.perf_counter()
        for ch, d, n, o in zip(chains, devs, ns, outs):
            ch.L.rd_chain_reset(ch.h, abi_ptr(st.cuda_stream))
            ch.process_device(d.data_ptr(), n, n, st.cuda_stream)
            abi.check(L, L.rd_chain_fetch(ch.h, abi.C.byref(o.c)), "rd_chain_fetch")
        return 1e3 * (time.perf_counter() - t)

    sequential_fetch_once()
    seq_fetch = min(sequential_fetch_once() for _ in range(3))
    for ch in chains:
        ch.close()
    b.close()
    return {"scenarios": n_scen, "samples_per_run": samples,
            "geometry": "channels {4,16,32,64}, PFB/FFT {16,64,256,1024}, taps {4,8,16}, "
                        "CPI log-uniform 2^12..2^18 samples/ch, beams = channels",
            "batched_ms": round(batched, 3), "sequential_ms": round(seq, 3),
            "batched_with_fetch_ms": round(batched_fetch, 3),
            "sequential_with_fetch_ms": round(seq_fetch, 3),
            "speedup_vs_sequential": round(seq / batched, 3),
            "speedup_vs_sequential_with_fetch": round(seq_fetch / batched_fetch, 3),
            "batched_msamples_s": round(samples / (batched / 1e3) / 1e6, 1),
            "autotuned": opt, "tune_s": round(tune_s, 2),
            "note": "batched: one CUDA graph replay of every scenario's launches spread "
                    "largest-first over the tuned number of streams; sequential: the same "
                    "launches stream-ordered on one stream, no host waits; with_fetch: "
                    "every scenario's results in page-locked host buffers - written by the "
                    "replay itself as each scenario ends (batched), or read after each "
                    "scenario before the next starts (sequential, the per-scenario API as "
                    "a caller uses it)"}


def abi_ptr(v: int):
    from rdgb import abi

    return abi.C.c_void_p(v)


def run_serving(torch, n_streams: int = 32, n_req: int = 2000, n_burst: int = 400) -> dict:
    """32 resident streams of mixed tiny / medium / full geometry; a request
    is 4096 samples per channel; the saturation rate is the median of five
    bursts of n_burst requests all due at once; then n_req Poisson arrivals
    at 25/50/80/100 % of it; latency = completion - arrival."""
    from rdgb import abi, scenario as sc
    from rdgb.serve import Server

    names = ["tiny", "medium", "full"]
    srv = Server(hbm_budget=64 << 30, max_inflight=16, queue_cap=512, max_chan=64,
                 max_request_samples=4096)
    streams = []
    for i in range(n_streams):
        p = sc.preset(names[i % 3])
        cfg = sc.make_config(p, max_frames=4096 // p.n_fft, form=abi.RD_FORM_TENSOR)
        st, sid = srv.open(cfg, sc.coefficients(p.n_fft, p.taps),
                           sc.steering_weights(p.n_chan, p.n_beams))
        if st != 0:
            raise RuntimeError(f"stream {i} not admitted: {st}")
        blocks = [sc.adc(p, 4096, start=k * 4096, seed=p.seed + i) for k in range(4)]
        streams.append((sid, p, blocks))
    rng = np.random.default_rng(5)

    def trace(n, rate_per_us):
        idx = rng.integers(0, n_streams, n)
        arrival = np.zeros(n) if rate_per_us is None else np.cumsum(rng.exponential(1.0 / rate_per_us, n))
        adcs = [streams[s][2][k % 4] for k, s in enumerate(idx)]
        lat, mk = srv.run_trace([streams[s][0] for s in idx], arrival, adcs)
        samples = sum(streams[s][1].n_chan * 4096 for s in idx)
        return lat, mk, samples

    trace(n_burst, None)  # warm: every stream's buffers and the output pools
    sat = float(np.median([n_burst / trace(n_burst, None)[1] for _ in range(5)]))  # req / us
    loads = []
    for load in (0.25, 0.5, 0.8, 1.0):
        lat, mk, samples = trace(n_req, sat * load)
        loads.append({"load": load, "offered_req_per_s": round(sat * load * 1e6, 1),
                      "p50_us": round(float(np.percentile(lat, 50)), 1),
                      "p99_us": round(float(np.percentile(lat, 99)), 1),
                      "throughput_msamples_s": round(samples / mk, 1)})
    srv.close()
    return {"streams": n_streams, "mix": "tiny / medium / full in turn, tensor form",
            "request": "4096 samples per channel", "max_inflight": 16,
            "requests_per_load": n_req, "saturation": f"median of 5 bursts of {n_burst}",
            "saturation_req_per_s": round(sat * 1e6, 1), "loads": loads,
            "p99_us_at_80pct": next(x["p99_us"] for x in loads if x["load"] == 0.8)}


def workload_desc(p, cpis: int) -> str:
    return (f"{p.name}: {p.n_chan} ch, {p.n_fft}-point PFB x {p.taps} taps, {p.n_fft}-point FFT "
            f"(spc {p.spc}), {p.hist_frames}-frame history, {p.n_beams} beams, {p.n_chan}x{p.n_chan} "
            f"covariance ({p.n_chan * (p.n_chan + 1) // 2} pairs) over {p.cov_window} frames, "
            f"CA-CFAR ref {p.ref[0]}/guard {p.guard[0]} per side, {p.packet_w}-bit packets; "
            f"{cpis} CPIs x {p.cpi_samples} samples/ch per step")


def run_reference(a, rank: int, world: int) -> None:
    """The reference arm: the reference's chain on host cores. The reference
    model (C++ headers) cannot be built on the GPU host (no reference
    checkout there and no cross toolchain here), so its plain-C restatement,
    pinned against the reference's own outputs, stands in. Each step is a
    bounded sample of the workload: 256 frames (one covariance window) of
    every channel, with every host thread."""
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
    frames = 256
    n = frames * p.n_fft
    x = sc.adc(p, n)
    o = orc.Oracle("port")
    threads = os.cpu_count() or 1
    times = []
    for i in range(a.warmup + a.steps):
        ch = o.chain(cfg, coeff, w, pairs[0], pairs[1])
        t = time.perf_counter()
        ch.process(x, taps=False, threads=threads, cap_events=frames * p.n_beams * (2 + p.n_fft // 16))
        if i >= a.warmup:
            times.append(time.perf_counter() - t)
    ms = 1e3 * sum(times) / len(times)
    v = p.n_chan * n / (ms / 1e3) / 1e6
    cpis = a.cpis or p.n_cpi
    sample = (f"{frames} frames x {p.n_fft} samples x {p.n_chan} ch of the {a.workload} workload per "
              f"step (one covariance window)")
    line = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT,
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic (seeded tones + noise, complex int16 12-bit range)",
            "config": {"workload": workload_desc(p, cpis),
                       "sample": sample, "form": a.form, "frames_per_launch": a.max_frames},
            "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def max_over_ranks(torch, dist, x: float) -> float:
    """The largest of every rank's x - a job's time is its slowest rank's -
    or x itself without a process group. NCCL reduces CUDA tensors, gloo CPU
    ones."""
    if not dist:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


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
    form = {"tensor": abi.RD_FORM_TENSOR, "tensor_warp": abi.RD_FORM_TENSOR_WARP}.get(
        a.form, abi.RD_FORM_CUDA_CORE)
    cfg = sc.make_config(p, max_frames=a.max_frames, form=form)
    pairs = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps)
    w = sc.steering_weights(p.n_chan, p.n_beams)
    distinct = min(DISTINCT_CPIS[a.workload], cpis)
    host, x = workload_input(torch, p, cpis, distinct, seed=p.seed + rank)  # a stream per replica
    dev = host.cuda()
    samples = p.n_chan * n
    frames_total = n // p.n_fft
    chain = gc.Chain(cfg, coeff, w, pairs)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream

    for _ in range(a.warmup):
        chain.process_device(dev.data_ptr(), n, n, sh)
    torch.cuda.synchronize()
    warm = chain.fetch(frames_total, cap_events=frames_total * p.n_beams * 8)
    n_events = len(warm["events"])
    del warm

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
    t_max = max_over_ranks(torch, dist, total_ms)
    value = world * samples * a.steps / (t_max / 1e3) / 1e6

    # roofline of the dominant kernel, and of every kernel of the chain
    peak, which = peaks()
    tpeak, tsrc = bf16_peak()
    per_kernel = {}
    for k, v in kernels.items():
        frames_launch = frames_total / max(v["launches"] / a.steps, 1)
        alg = kernel_bytes(cfg, k, frames_launch)
        gbs = alg / (v["avg_ms"] / 1e3) / 1e9
        e = {"avg_us": round(1e3 * v["avg_ms"], 2), "launches": v["launches"],
             "share": round(v["total_ms"] / sum(x["total_ms"] for x in kernels.values()), 4),
             "hbm_gbs": round(gbs, 1), "hbm_frac": round(gbs / peak, 4)}
        fl = kernel_tensor_flops(cfg, k, frames_launch, len(pairs[0])) if form else 0.0
        if fl:
            tf = fl / (v["avg_ms"] / 1e3) / 1e12
            e.update(tensor_tflops=round(tf, 1), tensor_frac=round(tf / tpeak, 4))
        per_kernel[k] = e
    dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
    per_launch_frames = frames_total / max(kernels[dom]["launches"] / a.steps, 1)
    alg = kernel_bytes(cfg, dom, per_launch_frames)
    achieved = alg / (kernels[dom]["avg_ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": f"of {which}",
                "traffic": profile_line(a.workload, "traffic", dom),
                "algorithmic_bytes_per_launch": alg,
                "chain": {"achieved": round(value * 8 / 1e3, 1), "frac": round(value * 8 / 1e3 / peak, 4),
                          "note": "the whole chain at 8 B per sample (ADC read + history write)"},
                "tensor_peak": f"{tpeak} TFLOP/s dense bf16, {tsrc}"}
    # the ceiling that binds the integer kernels: one warp instruction per SM
    # sub-partition per cycle, at the SM clock sampled during the run
    inst = profile_line(a.workload, "instructions", dom)
    if inst:
        n_smsp = 4 * torch.cuda.get_device_properties(local).multi_processor_count
        mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
        got = inst / (kernels[dom]["avg_ms"] / 1e3) / 1e9
        top = n_smsp * mhz / 1e3
        roofline["issue"] = {"achieved": round(got, 1), "peak": round(top, 1),
                             "unit": "G warp instructions/s", "frac": round(got / top, 4),
                             "inst_per_launch": inst, "sm_mhz": mhz,
                             "source": "ncu smsp__inst_executed.sum of the same launch"}

    # e2e through the C ABI from pinned host memory
    e2e = None
    if not a.no_e2e:
        cap = max(2 * n_events, 1024)

        out = gc.Outputs(cfg, frames_total, chain.n_pairs, False, cap, alloc=pinned_alloc(torch))
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
        e2e_ms = max_over_ranks(torch, dist, ms)
        e2e = {"value": round(world * samples / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": samples * 4, "d2h_bytes_per_step": int(d2h),
               "ms_per_step": round(e2e_ms, 3),
               "step_ms": [round(1e3 * x, 3) for x in times],
               "api": "rd_chain_process (host buffers in, page-locked result buffers out)"}
        del out

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cpu = None
    if not a.no_cpu_baseline:
        cpu = cpu_baseline(p, cfg, coeff, w, pairs, x)
    forms = batching = serving = None
    if not a.no_patterns and world == 1:
        del dev
        chain.close()
        forms = run_forms(torch, a, stream)
        batching = run_batching(torch)
        serving = run_serving(torch)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(t_max / a.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
        "data": (f"synthetic (seeded tones + noise, complex int16 12-bit range; {distinct} "
                 f"distinct CPIs of one seeded stream, repeated to {cpis})"),
        "config": {"workload": workload_desc(p, cpis),
                   "form": a.form, "frames_per_launch": a.max_frames,
                   "input_bytes": samples * 4, "l2": "inputs larger than L2 (no flush)"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": launches,
        "kernels": per_kernel,
        "step_ms": [round(s, 4) for s in step_ms],
        "events_per_step": n_events,
        "forms": forms,
        "batching": batching,
        "serving": serving,
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
