"""Packet fabric egress on the GPU, through the C ABI: rd_egress_merge
against the round-robin arbiter simulated grant by grant (bit-exact rings,
source indices and per-port counts), ring overflow, device-side packet
counts, and rd_batch_egress after a batch of chains - every port ring then
passes the fabric scoreboard (packet_model.hpp:323-586) with nothing lost,
duplicated, reordered, corrupted or misrouted."""
import numpy as np
import pytest

import scoreboard as sbm
from rdgb import abi, chain as gc, fabric, scenario as sc
from rdgb.batch import Batch

pytestmark = pytest.mark.gpu


def _events(rng, n):
    ev = np.zeros(n, abi.EVENT_DTYPE)
    ev["w"] = rng.integers(0, 2**63, size=(n, 3), dtype=np.uint64)
    ev["w"][:, 2] &= (1 << 48) - 1
    ev["frame"] = rng.integers(0, 2**16, n)
    return ev


def _expected(packets, dests, n_ports, cap):
    """Per port: the packet rows the arbiter grants (first `cap`), the source
    of each, and the port's packet count."""
    order = sbm.rr_arbiter_order([len(p) for p in packets], dests, n_ports)
    rings, srcs = [], []
    for o in order:
        o = o[:cap]
        rings.append(np.stack([packets[s][r] for s, r in o]) if o else None)
        srcs.append(np.array([s for s, _ in o], np.uint32))
    counts = [sum(len(packets[s]) for s in range(len(packets)) if dests[s] == d)
              for d in range(n_ports)]
    return rings, srcs, counts


def _merge(torch, packets_np, dests, packet_w, n_ports, cap, use_count_dev=False):
    W = fabric.packet_words(packet_w)
    dev = [torch.from_numpy(p.reshape(-1).view(np.int32).copy()).cuda() if len(p) else
           torch.zeros(W, dtype=torch.int32, device="cuda") for p in packets_np]
    cnt = torch.tensor([len(p) for p in packets_np], dtype=torch.int64, device="cuda")
    srcs = []
    for i, (d, p) in enumerate(zip(dev, packets_np)):
        if use_count_dev:  # a bound above the count: the device count wins
            srcs.append(fabric.Source(d.data_ptr(), len(p) + 5, dests[i],
                                      cnt.data_ptr() + 8 * i))
        else:
            srcs.append(fabric.Source(d.data_ptr(), len(p), dests[i]))
    ring = torch.full((n_ports * cap * W,), -1, dtype=torch.int32, device="cuda")
    src_of = torch.full((n_ports * cap,), -1, dtype=torch.int32, device="cuda")
    pc = torch.zeros(n_ports, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    fabric.egress_merge(srcs, packet_w, n_ports, ring.data_ptr(), cap, pc.data_ptr(),
                        src_of.data_ptr(), stream)
    torch.cuda.synchronize()
    return (ring.cpu().numpy().view(np.uint32).reshape(n_ports, cap, W),
            src_of.cpu().numpy().view(np.uint32).reshape(n_ports, cap), pc.cpu().numpy())


@pytest.mark.parametrize("packet_w", [64, 96, 256, 512])
@pytest.mark.parametrize("n_src,n_ports", [(1, 1), (7, 1), (33, 4), (200, 16), (512, 16)])
def test_egress_merge_matches_arbiter(gpulib, port, packet_w, n_src, n_ports):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n_src * 7 + packet_w)
    W = fabric.packet_words(packet_w)
    dests = rng.integers(0, n_ports, n_src)
    packets = []
    for s in range(n_src):
        n = int(rng.integers(0, 40)) if rng.random() < 0.85 else 0
        fl = port.packetize(_events(rng, n), packet_w, s % 16, int(dests[s]), s % 4,
                            int(rng.integers(0, 2**16)))
        packets.append(fl.reshape(n, W))
    cap = max(1, max(sum(len(packets[s]) for s in range(n_src) if dests[s] == d)
                     for d in range(n_ports)))
    for use_count_dev in (False, True):
        ring, src_of, pc = _merge(torch, packets, dests, packet_w, n_ports, cap, use_count_dev)
        rings, srcs, counts = _expected(packets, dests, n_ports, cap)
        assert list(pc) == counts
        for d in range(n_ports):
            k = counts[d]
            if k:
                assert np.array_equal(ring[d, :k], rings[d]), d
                assert np.array_equal(src_of[d, :k], srcs[d]), d
            assert (ring[d, k:] == 0xFFFFFFFF).all()


def test_egress_merge_ring_overflow(gpulib, port):
    # a ring smaller than its port's traffic keeps the first `cap` grants and
    # reports the full count
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    W = fabric.packet_words(128)
    packets = [port.packetize(_events(rng, n), 128, s, 0, 0, 0).reshape(n, W)
               for s, n in enumerate([30, 5, 17, 0, 22])]
    dests = [0] * 5
    ring, src_of, pc = _merge(torch, packets, dests, 128, 1, 20)
    rings, srcs, counts = _expected(packets, dests, 1, 20)
    assert pc[0] == 74
    assert np.array_equal(ring[0], rings[0]) and np.array_equal(src_of[0], srcs[0])


def test_egress_merge_rejects_bad_arguments(gpulib):
    L = gpulib
    arr = (abi.RdEgressSource * 2)()
    arr[0].dest, arr[1].dest = 0, 3
    assert L.rd_egress_merge(arr, 2, 64, 2, abi.C.c_void_p(16), 4, None, abi.C.c_void_p(16),
                             None) == abi.RD_EINVAL  # port 3 of 2
    assert L.rd_egress_merge(arr, 2, 60, 4, abi.C.c_void_p(16), 4, None, abi.C.c_void_p(16),
                             None) == abi.RD_EINVAL  # packet width
    arr[0].n_packets = 3  # packets without a buffer
    assert L.rd_egress_merge(arr, 2, 64, 4, abi.C.c_void_p(16), 4, None, abi.C.c_void_p(16),
                             None) == abi.RD_EINVAL


def test_batch_egress_scoreboard(gpulib):
    # a batch of chains, every scenario its own (src, VC, dest): the merged
    # port rings equal the arbiter's order over the fetched packets and pass
    # the scoreboard clean, each triple delivered in emission order
    torch = pytest.importorskip("torch")
    n, n_ports = 12, 4
    ps = sc.batch_scenarios(n, log2_max=14)
    cfgs, coeffs, ws, xs = [], [], [], []
    for i, p in enumerate(ps):
        c = sc.make_config(p, max_frames=min(p.frames_per_cpi, 256))
        c.packet_w = 128
        c.src_id, c.vc, c.dest = i % 16, i // 4 % 4, i % n_ports
        cfgs.append(c)
        coeffs.append(sc.coefficients(p.n_fft, p.taps))
        ws.append(sc.steering_weights(p.n_chan, p.n_beams))
        xs.append(sc.adc(p, p.cpi_samples))
    devs = [torch.from_numpy(x.view(np.int32)).cuda() for x in xs]
    b = Batch(cfgs, coeffs, ws, n_streams=4)
    stream = torch.cuda.current_stream().cuda_stream
    b.run([d.data_ptr() for d in devs], [p.cpi_samples for p in ps], stream=stream)
    W = fabric.packet_words(128)
    n_pairs = [gc.lib().rd_cov_pairs(gc.C.byref(c)) for c in cfgs]
    outs = [b.fetch(i, p.frames_per_cpi, n_pairs[i]) for i, p in enumerate(ps)]
    packets = [o["flits"].reshape(-1, W) for o in outs]
    assert sum(len(p) for p in packets) > 0
    cap = max(sum(len(packets[i]) for i in range(n) if cfgs[i].dest == d)
              for d in range(n_ports)) + 3
    ring = torch.zeros(n_ports * cap * W, dtype=torch.int32, device="cuda")
    src_of = torch.zeros(n_ports * cap, dtype=torch.int32, device="cuda")
    pc = torch.zeros(n_ports, dtype=torch.int64, device="cuda")
    b.egress(n_ports, ring.data_ptr(), cap, pc.data_ptr(), src_of.data_ptr(), stream)
    torch.cuda.synchronize()
    ring = ring.cpu().numpy().view(np.uint32).reshape(n_ports, cap, W)
    pc = pc.cpu().numpy()
    rings, srcs, counts = _expected(packets, [c.dest for c in cfgs], n_ports, cap)
    assert list(pc) == counts
    sb = sbm.Scoreboard(128, 4, 2)
    for p in packets:
        for pk in sbm.packets_from_flits(p, 128):
            sb.inject(pk)
    for d in range(n_ports):
        if counts[d]:
            assert np.array_equal(ring[d, :counts[d]], rings[d]), d
        sb.observe_rows(d, ring[d, :counts[d]])
    sb.finish()
    assert sb.total_errors() == 0, sb.notes
    assert sb.counts["delivered"] == sum(counts)
    b.close()
