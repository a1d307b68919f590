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


def test_batch_matches_standalone_chains(gpulib):
    torch = pytest.importorskip("torch")
    ps, cfgs, coeffs, ws, xs, devs = _batch_inputs(12, torch)
    ptrs = [d.data_ptr() for d in devs]
    ns = [p.cpi_samples for p in ps]
    b = Batch(cfgs, coeffs, ws, n_streams=4, use_graph=True)
    want = []
    for i, p in enumerate(ps):
        r = gc.Chain(cfgs[i], coeffs[i], ws[i]).process(xs[i])
        want.append(r)
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
    # the queue holds two requests; the third is pushed back
    x = sc.adc(p, 4096)
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
