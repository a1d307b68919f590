"""Packet fabric egress on the CPU: the butterfly route through the C ABI
against its restatement and the determinism property (test_packet.cpp:
every (source, destination) pair of the network), the scoreboard
restatement against the reference's own packet_model::Scoreboard on clean
and faulty traffic, and the closed form the egress kernel places packets by
against a grant-by-grant simulation of the round-robin arbiter."""
import numpy as np
import pytest

import scoreboard as sbm
from rdgb import abi, fabric

TOPOLOGIES = [(4, 2), (2, 4), (3, 3), (2, 1), (16, 1), (5, 2)]


@pytest.mark.parametrize("radix,stages", TOPOLOGIES)
def test_route_path_every_pair(radix, stages):
    ports = radix ** stages
    for s in range(ports):
        for d in range(ports):
            p = fabric.route_path(s, d, radix, stages)
            assert p == sbm.route_path(s, d, radix, stages)
            assert p[0] == s and p[-1] == d and len(p) == stages + 1
            assert all(0 <= w < ports for w in p)


def test_route_path_rejects_out_of_range():
    L = abi.load()
    path = (abi.C.c_uint32 * 8)()
    assert L.rd_route_path(16, 0, 4, 2, path) == abi.RD_EINVAL
    assert L.rd_route_path(0, 0, 1, 2, path) == abi.RD_EINVAL
    assert L.rd_route_path(0, 0, 4, 0, path) == abi.RD_EINVAL


def _events(rng, n):
    ev = np.zeros(n, abi.EVENT_DTYPE)
    ev["w"] = rng.integers(0, 2**63, size=(n, 3), dtype=np.uint64)
    ev["w"][:, 2] &= (1 << 48) - 1
    ev["frame"] = rng.integers(0, 2**16, n)
    ev["beam"] = rng.integers(0, 64, n)
    return ev


def _traffic(port, rng, packet_w, triples, n_max=12):
    """Per source: (src, vc, dest, flit rows) of random detection packets."""
    out = []
    for k, (s, vc, d) in enumerate(triples):
        n = int(rng.integers(0, n_max))
        rows = port.packetize(_events(rng, n), packet_w, s, d, vc, seq0=int(rng.integers(0, 2**16)))
        out.append((s, vc, d, rows))
    return out


def _rr_egress(traffic, packet_w, n_ports):
    """Per port, the flit rows in round-robin source order."""
    nfl = sbm.detection_flits(packet_w)
    n = [len(t[3]) // nfl for t in traffic]
    order = sbm.rr_arbiter_order(n, [t[2] for t in traffic], n_ports)
    return [[t for (s, r) in o for t in traffic[s][3][r * nfl:(r + 1) * nfl]] for o in order]


def _run_both(refo, packet_w, radix, stages, injected, ports, observed):
    sb = sbm.Scoreboard(packet_w, radix, stages)
    for p in sbm.packets_from_flits(np.concatenate(injected) if injected else
                                    np.zeros((0, sbm.flit_words(packet_w)), np.uint32), packet_w):
        sb.inject(p)
    for port, row in zip(ports, observed):
        sb.observe(int(port), sbm.Flit.from_row(row, packet_w))
    sb.finish()
    inj = np.concatenate(injected) if injected else np.zeros(0, np.uint32)
    obs = np.asarray(observed, np.uint32) if len(observed) else np.zeros(0, np.uint32)
    counts, log = refo.scoreboard(packet_w, radix, stages, inj, np.asarray(ports, np.uint32), obs)
    return sb, counts, log


def _observed(egress):
    ports, rows = [], []
    for d, fl in enumerate(egress):
        ports += [d] * len(fl)
        rows += list(fl)
    return ports, rows


def _mutate(kind, ports, rows, rng, packet_w):
    nfl = sbm.detection_flits(packet_w)
    rows = [np.array(r, np.uint32) for r in rows]
    ports = list(ports)
    n_pk = len(rows) // nfl
    if n_pk < 2:
        return ports, rows
    k = int(rng.integers(0, n_pk - 1))
    a, b = k * nfl, (k + 1) * nfl
    if kind == "drop":
        del rows[a:b], ports[a:b]
    elif kind == "duplicate":
        rows[b:b] = rows[a:b]
        ports[b:b] = ports[a:b]
    elif kind == "swap":  # two packets of one triple exchanged: reordered
        hdr = [sbm.Flit.from_row(rows[i * nfl], packet_w).header() for i in range(n_pk)]
        key = [(h.src, h.vc, h.dest) for h in hdr]
        pair = next(((i, j) for i in range(n_pk) for j in range(i + 1, n_pk)
                     if key[i] == key[j]), None)
        if pair:
            i, j = pair[0] * nfl, pair[1] * nfl
            rows[i:i + nfl], rows[j:j + nfl] = rows[j:j + nfl], rows[i:i + nfl]
        else:  # neighbours of different triples: a legal order
            rows[a:b + nfl] = rows[b:b + nfl] + rows[a:b]
    elif kind == "payload_bit":
        rows[a + 1][1] ^= 1 << 7
        rows[a + 1][0] ^= 1  # parity re-sealed: a clean flit with a wrong word
    elif kind == "parity":
        rows[a + 1][0] ^= 1
    elif kind == "header_seq":
        v = sbm.to_int(rows[a]) ^ (1 << (5 + 20))
        v ^= 1
        rows[a] = sbm.from_int(v, packet_w)
    elif kind == "misroute":
        ports[a:b] = [(ports[a] + 1) % 16] * nfl
    elif kind == "truncate":
        del rows[b - 1], ports[b - 1]
    elif kind == "body_first":
        del rows[a], ports[a]
    elif kind == "type":
        v = sbm.to_int(rows[a]) | (7 << (5 + 11))
        if bin(v).count("1") % 2 == 0:
            v ^= 1
        rows[a] = sbm.from_int(v, packet_w)
    elif kind == "unexpected":
        v = sbm.to_int(rows[a]) ^ (1 << (5 + 8))  # src bit 4 flipped, parity re-sealed
        v ^= 1
        rows[a] = sbm.from_int(v, packet_w)
    return ports, rows


KINDS = ["clean", "drop", "duplicate", "swap", "payload_bit", "parity", "header_seq",
         "misroute", "truncate", "body_first", "type", "unexpected"]


@pytest.mark.parametrize("packet_w", [64, 128, 512])
@pytest.mark.parametrize("kind", KINDS)
def test_scoreboard_matches_reference(refo, port, packet_w, kind):
    rng = np.random.default_rng(KINDS.index(kind) * 1000 + packet_w)
    triples = [(0, 0, 0), (1, 0, 0), (2, 1, 3), (0, 2, 3), (5, 3, 15), (1, 0, 0)]
    traffic = _traffic(port, rng, packet_w, triples[:5], n_max=10)
    ports, rows = _observed(_rr_egress(traffic, packet_w, 16))
    ports, rows = _mutate(kind, ports, rows, rng, packet_w)
    sb, counts, log = _run_both(refo, packet_w, 4, 2, [t[3] for t in traffic], ports, rows)
    assert sb.counts == counts, (kind, sb.notes)
    assert sb.log == log
    if kind == "clean":
        assert sb.total_errors() == 0 and sb.counts["delivered"] == sum(
            len(t[3]) for t in traffic) // sbm.detection_flits(packet_w)
    else:
        assert sb.total_errors() > 0 or len(rows) < 2 * sbm.detection_flits(packet_w)


def test_scoreboard_unroutable_injection(refo, port):
    # a destination outside the network has no deterministic route
    rng = np.random.default_rng(5)
    traffic = _traffic(port, rng, 64, [(1, 0, 9)], n_max=3)
    sb, counts, log = _run_both(refo, 64, 2, 3, [t[3] for t in traffic], [], [])
    assert sb.counts == counts


@pytest.mark.parametrize("seed", range(6))
def test_rr_closed_form(seed):
    # the position the egress kernel computes for packet r of source s equals
    # where the grant-by-grant arbiter puts it
    rng = np.random.default_rng(seed)
    n_src = int(rng.integers(1, 40))
    n_ports = int(rng.integers(1, 5))
    n = rng.integers(0, 9, n_src) * (rng.random(n_src) < 0.8)
    dests = rng.integers(0, n_ports, n_src)
    for d, order in enumerate(sbm.rr_arbiter_order(n, dests, n_ports)):
        for pos, (s, r) in enumerate(order):
            want = sum(min(int(n[t]), r) + (t < s and n[t] > r)
                       for t in range(n_src) if dests[t] == d)
            assert pos == want
        assert len(order) == int(n[dests == d].sum())


def test_rr_merge_keeps_triple_order(port):
    # round-robin egress of many sources through the restated scoreboard: no
    # errors, and every triple's deliveries in its injection order
    rng = np.random.default_rng(9)
    # sources are ports of the 16-port network, so src < 16
    triples = [(s % 16, s // 16 % 4, s * 7 % 16) for s in range(40)]
    traffic = _traffic(port, rng, 96, triples, n_max=8)
    sb = sbm.Scoreboard(96, 4, 2)
    for t in traffic:
        for p in sbm.packets_from_flits(t[3], 96):
            sb.inject(p)
    for d, fl in enumerate(_rr_egress(traffic, 96, 16)):
        for row in fl:
            sb.observe(d, sbm.Flit.from_row(row, 96))
    sb.finish()
    assert sb.total_errors() == 0, sb.notes
