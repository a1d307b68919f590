"""Batching and serving on the GPU, through the C ABI. Both must leave every
bit of every scenario's / request's output as a single chain running alone
computes it: the batched graph against standalone chains and against the
sequential per-scenario run; each served request against the same request
sequence run alone through one chain."""
import numpy as np
import pytest

from helpers import CHAIN_KEYS, diff
from rdgb import abi, chain as gc, scenario as sc
from rdgb.batch import Batch
from rdgb.serve import Server

pytestmark = pytest.mark.gpu


def _batch_inputs(n, torch, log2_max=14):
    ps = sc.batch_scenarios(n, log2_min=12, log2_max=log2_max)
    cfgs = [sc.make_config(p, max_frames=min(p.frames_per_cpi, 256)) for p in ps]
    coeffs = [sc.coefficients(p.n_fft, p.taps) for p in ps]
    ws = [sc.steering_weights(p.n_chan, p.n_beams) for p in ps]
    xs = [sc.adc(p, p.cpi_samples) for p in ps]
    devs = [torch.from_numpy(x.view(np.int32)).cuda() for x in xs]
    return ps, cfgs, coeffs, ws, xs, devs


def test_batch_matches_oracle(gpulib, port):
    # 16 scenarios of uneven geometry (channels 4..64, FFT 16..1024, taps
    # 4..16, 2^12..2^14 samples per channel): every batched scenario, in every
    # run mode and after autotuning, equals the CPU oracle's chain on the same
    # input, bit for bit
    torch = pytest.importorskip("torch")
    ps, cfgs, coeffs, ws, xs, devs = _batch_inputs(16, torch)
    ptrs = [d.data_ptr() for d in devs]
    ns = [p.cpi_samples for p in ps]
    b = Batch(cfgs, coeffs, ws, n_streams=4, use_graph=True)
    want = []
    for i, p in enumerate(ps):
        px, py = sc.pair_table(p)
        want.append(port.chain(cfgs[i], coeffs[i], ws[i], px, py).process(xs[i], taps=False,
                                                                           threads=8))
    n_pairs = [gc.lib().rd_cov_pairs(gc.C.byref(c)) for c in cfgs]
    for mode in ("eager-first", "graph", "graph-again", "sequential"):
        b.run(ptrs, ns, sequential=(mode == "sequential"))
        for i, p in enumerate(ps):
            got = b.fetch(i, p.frames_per_cpi, n_pairs[i])
            assert diff(got, want[i], CHAIN_KEYS) == [], (mode, i)
    opt, ms = b.tune(ptrs, ns, reps=2)
    assert opt["n_streams"] >= 1 and ms > 0
    b.run(ptrs, ns)
    for i, p in enumerate(ps):
        assert diff(b.fetch(i, p.frames_per_cpi, n_pairs[i]), want[i], CHAIN_KEYS) == [], i
    # the scenarios cover every FFT size and channel count of the workload
    assert {p.n_fft for p in ps} == {16, 64, 256, 1024}
    assert {p.n_chan for p in ps} == {4, 16, 32, 64}
    b.close()


def test_batch_tune_cache(gpulib, port, tmp_path):
    # the on-disk autotune cache: the first batch tunes and records its choice,
    # a second batch of the same scenarios takes it from the file without
    # timing anything, and its results are unchanged
    torch = pytest.importorskip("torch")
    ps, cfgs, coeffs, ws, xs, devs = _batch_inputs(6, torch, log2_max=13)
    ptrs = [d.data_ptr() for d in devs]
    ns = [p.cpi_samples for p in ps]
    n_pairs = [gc.lib().rd_cov_pairs(gc.C.byref(c)) for c in cfgs]
    cache = tmp_path / "batch_tune.txt"
    b = Batch(cfgs, coeffs, ws, n_streams=4, use_graph=True)
    b.run(ptrs, ns)
    opt1, ms1 = b.tune(ptrs, ns, reps=2, cache=cache)
    assert not opt1["hit"] and ms1 > 0
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and lines[0].split()[1:3] == [str(opt1["n_streams"]),
                                                         str(opt1["launch_frames"])]
    b.close()
    b2 = Batch(cfgs, coeffs, ws, n_streams=1, use_graph=True)
    b2.run(ptrs, ns)
    opt2, ms2 = b2.tune(ptrs, ns, reps=2, cache=cache)
    assert opt2["hit"] and (opt2["n_streams"], opt2["launch_frames"]) == \
        (opt1["n_streams"], opt1["launch_frames"]) and ms2 == pytest.approx(ms1, rel=1e-3)
    assert len(cache.read_text().splitlines()) == 1
    b2.run(ptrs, ns)
    for i, p in enumerate(ps):
        px, py = sc.pair_table(p)
        want = port.chain(cfgs[i], coeffs[i], ws[i], px, py).process(xs[i], taps=False, threads=8)
        assert diff(b2.fetch(i, p.frames_per_cpi, n_pairs[i]), want, CHAIN_KEYS) == [], i
    # other scenarios (one sample count changed: a frame fewer) miss the
    # cache and append
    ns3 = list(ns)
    ns3[0] = ns[0] - cfgs[0].n_fft
    b3 = Batch(cfgs, coeffs, ws, n_streams=2, use_graph=True)
    b3.run(ptrs, ns3)
    opt3, _ = b3.tune(ptrs, ns3, reps=1, cache=cache)
    assert not opt3["hit"] and len(cache.read_text().splitlines()) == 2
    b3.close()
    b2.close()


def _pinned(torch):
    def alloc(shape, dtype):
        dt = np.dtype(dtype)
        k = int(np.prod(shape)) * dt.itemsize
        return torch.empty(max(k, 1), dtype=torch.uint8, pin_memory=True).numpy()[:k] \
            .view(dt).reshape(shape)
    return alloc


def test_batch_exported_outputs(gpulib, port):
    # results written to page-locked host buffers by the run itself (the graph
    # carries the export): every scenario equals the oracle, a replay rewrites
    # them identically, a scenario whose event capacity is too small keeps its
    # first events and reports RD_ETRUNC, and unregistering stops the export
    torch = pytest.importorskip("torch")
    ps, cfgs, coeffs, ws, xs, devs = _batch_inputs(10, torch, log2_max=13)
    ptrs = [d.data_ptr() for d in devs]
    ns = [p.cpi_samples for p in ps]
    n_pairs = [gc.lib().rd_cov_pairs(gc.C.byref(c)) for c in cfgs]
    want = []
    for i, p in enumerate(ps):
        px, py = sc.pair_table(p)
        want.append(port.chain(cfgs[i], coeffs[i], ws[i], px, py).process(xs[i], taps=False,
                                                                           threads=8))
    b = Batch(cfgs, coeffs, ws, n_streams=4, use_graph=True)
    b.run(ptrs, ns)  # eager first run (sizes the chains' buffers)
    small = 3  # this scenario keeps 5 events
    outs = [gc.Outputs(c, p.frames_per_cpi, n_pairs[i], False,
                       5 if i == small else max(2 * len(want[i]["events"]), 64),
                       alloc=_pinned(torch))
            for i, (c, p) in enumerate(zip(cfgs, ps))]
    b.set_outputs(outs)
    for rep in range(3):  # eager, captured, replayed
        for o in outs:
            o.events[...] = 0
            o.flits[...] = 0
        b.run(ptrs, ns)
        for i in range(len(ps)):
            if i == small:
                st = b.L.rd_batch_results(b.h, i, gc.C.byref(outs[i].c))
                assert st == abi.RD_ETRUNC, st
                got = outs[i].result()
                n_ev = len(want[i]["events"])
                assert outs[i].c.n_events == n_ev > 5
                assert np.array_equal(outs[i].events[:5], want[i]["events"][:5])
                nfl = len(want[i]["flits"]) // n_ev
                assert np.array_equal(outs[i].flits[:5 * nfl], want[i]["flits"][:5 * nfl])
                continue
            got = b.results(i)
            assert diff(got, want[i], CHAIN_KEYS) == [], (rep, i)
    # without registered outputs the run exports nothing
    b.set_outputs(None)
    for o in outs:
        o.events[...] = 0
    b.run(ptrs, ns)
    torch.cuda.synchronize()
    assert all(not o.events.view(np.uint8).any() for o in outs)
    for i, p in enumerate(ps):
        assert diff(b.fetch(i, p.frames_per_cpi, n_pairs[i]), want[i], CHAIN_KEYS) == [], i
    # pageable memory is refused
    bad = [gc.Outputs(c, p.frames_per_cpi, n_pairs[i], False, 64) for i, (c, p) in
           enumerate(zip(cfgs, ps))]
    assert b.L.rd_batch_set_outputs(b.h, (abi.RdOutput * len(bad))(*[o.c for o in bad])) == \
        abi.RD_EINVAL
    b.close()


def _serve_streams():
    # mixed stream sizes; every request is 4096 samples per channel
    out = []
    for name in ("tiny", "ref_tiny", "medium", "tiny", "medium"):
        p = sc.preset(name)
        cfg = sc.make_config(p, max_frames=64)
        out.append((p, cfg, sc.coefficients(p.n_fft, p.taps),
                    sc.steering_weights(p.n_chan, p.n_beams)))
    return out


def test_serving_results_equal_alone(gpulib):
    streams = _serve_streams()
    srv = Server(hbm_budget=2 << 30, max_inflight=3, queue_cap=32, max_chan=16,
                 max_request_samples=4096)
    ids = []
    for p, cfg, co, w in streams:
        st, sid = srv.open(cfg, co, w)
        assert st == abi.RD_OK, gc.lib().rd_last_error()
        ids.append(sid)
    n_req = 4
    reqs = {}  # request id -> (stream index, k)
    order = [(s, k) for k in range(n_req) for s in range(len(streams))]
    pending = list(order)
    while pending:  # interleaved submissions; the queue may push back
        s, k = pending[0]
        p = streams[s][0]
        x = sc.adc(p, 4096, start=k * 4096, seed=p.seed + 7 * s)
        st, rid = srv.submit(ids[s], x)
        if st == abi.RD_EAGAIN:
            srv.poll()
            continue
        assert st == abi.RD_OK
        reqs[rid] = (s, k)
        pending.pop(0)
    done = {}
    while len(done) < len(reqs):
        for c in srv.poll():
            assert c["status"] == abi.RD_OK
            s, k = reqs[c["req_id"]]
            done[(s, k)] = srv.take(c["req_id"], ids[s], 4096 // streams[s][0].n_fft)
    for s, (p, cfg, co, w) in enumerate(streams):  # the same requests alone
        ch = gc.Chain(cfg, co, w)
        for k in range(n_req):
            x = sc.adc(p, 4096, start=k * 4096, seed=p.seed + 7 * s)
            alone = ch.process(x)
            assert diff(done[(s, k)], alone, CHAIN_KEYS) == [], (s, k)
    info = srv.info()
    assert info["streams"] == len(streams) and info["inflight"] == 0
    srv.close()


def test_serving_full_tensor_vs_oracle(gpulib, port):
    # a mix with a full-scale stream in the tensor form (64 channels, 1024
    # bins, 64 beams, 2080 pairs; its 8-frame covariance windows close every
    # second request): every served request equals the CPU oracle's chain fed
    # the same request sequence, bit for bit
    mix = [("tiny", abi.RD_FORM_CUDA_CORE, {}), ("full", abi.RD_FORM_TENSOR, {"cov_window": 8}),
           ("medium", abi.RD_FORM_TENSOR, {}), ("ref_tiny", abi.RD_FORM_CUDA_CORE, {}),
           ("full", abi.RD_FORM_CUDA_CORE, {"cov_window": 4})]
    srv = Server(hbm_budget=6 << 30, max_inflight=3, queue_cap=32, max_chan=64,
                 max_request_samples=4096)
    streams, ids = [], []
    for name, form, over in mix:
        p = sc.preset(name, **over)
        cfg = sc.make_config(p, max_frames=64, form=form)
        co, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
        st, sid = srv.open(cfg, co, w, pairs=sc.pair_table(p))
        assert st == abi.RD_OK, gc.lib().rd_last_error()
        streams.append((p, cfg, co, w))
        ids.append(sid)
    n_req = 4
    reqs, done = {}, {}
    pending = [(s, k) for k in range(n_req) for s in range(len(streams))]
    while pending:
        s, k = pending[0]
        p = streams[s][0]
        x = sc.adc(p, 4096, start=k * 4096, seed=p.seed + 11 * s)
        st, rid = srv.submit(ids[s], x)
        if st == abi.RD_EAGAIN:
            srv.poll()
            continue
        assert st == abi.RD_OK
        reqs[rid] = (s, k)
        pending.pop(0)
    while len(done) < len(reqs):
        for c in srv.poll():
            assert c["status"] == abi.RD_OK
            s, k = reqs[c["req_id"]]
            done[(s, k)] = srv.take(c["req_id"], ids[s], 4096 // streams[s][0].n_fft)
    windows = 0
    for s, (p, cfg, co, w) in enumerate(streams):
        px, py = sc.pair_table(p)
        o = port.chain(cfg, co, w, px, py)
        for k in range(n_req):
            x = sc.adc(p, 4096, start=k * 4096, seed=p.seed + 11 * s)
            want = o.process(x, taps=False, threads=8)
            assert diff(done[(s, k)], want, CHAIN_KEYS) == [], (s, k)
            windows += len(want["cov_windows"]) if p.n_fft == 1024 else 0
    assert windows >= 4  # the full-scale streams closed windows
    srv.close()


def test_serving_admission_by_budget(gpulib):
    p = sc.preset("medium")
    cfg = sc.make_config(p, max_frames=64)
    fp = gc.lib().rd_chain_footprint(gc.C.byref(cfg), 4096 // p.n_fft)
    slots = 2 * 16 * 4096 * 4
    srv = Server(hbm_budget=slots + 2 * fp + fp // 2, max_inflight=2, queue_cap=2,
                 max_chan=16, max_request_samples=4096)
    co, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    st0, a = srv.open(cfg, co, w)
    st1, b = srv.open(cfg, co, w)
    st2, _ = srv.open(cfg, co, w)
    assert (st0, st1, st2) == (abi.RD_OK, abi.RD_OK, abi.RD_ENOMEM)
    assert b"admission refused" in gc.lib().rd_last_error()
    assert srv.close_stream(a) == abi.RD_OK
    st3, _ = srv.open(cfg, co, w)
    assert st3 == abi.RD_OK
    x = sc.adc(p, 4096)
    # malformed requests are refused before they take a queue slot: no such
    # stream, samples that are not whole frames, more than a request may
    # hold, none at all
    assert srv.submit(999, x)[0] == abi.RD_EINVAL
    assert srv.submit(b, x[:, :4096 - p.n_fft // 2])[0] == abi.RD_EINVAL
    assert b"a multiple of" in gc.lib().rd_last_error()
    assert srv.submit(b, sc.adc(p, 8192))[0] == abi.RD_EINVAL
    assert srv.submit(b, x[:, :0])[0] == abi.RD_EINVAL
    # the queue holds two requests; the third is pushed back
    assert srv.submit(b, x)[0] == abi.RD_OK
    assert srv.submit(b, x)[0] == abi.RD_OK
    assert srv.submit(b, x)[0] == abi.RD_EAGAIN
    got = 0
    while got < 2:
        got += len(srv.poll())
    srv.close()


def test_serving_trace_latencies(gpulib):
    streams = _serve_streams()
    srv = Server(hbm_budget=2 << 30, max_inflight=4, queue_cap=64, max_chan=16,
                 max_request_samples=4096)
    ids = [srv.open(cfg, co, w)[1] for p, cfg, co, w in streams]
    rng = np.random.default_rng(0)
    n = 40
    sids = rng.integers(0, len(ids), n)
    arrival = np.cumsum(rng.exponential(200.0, n))
    adcs = [sc.adc(streams[s][0], 4096, start=k * 4096) for k, s in enumerate(sids)]
    lat, makespan = srv.run_trace([ids[s] for s in sids], arrival, adcs)
    assert (lat > 0).all() and makespan >= arrival[-1]
    srv.close()
