"""Packet fabric egress: many streams' detection packets merged on the GPU
into per-port DMA rings with the fabric's round-robin arbitration
(rd_egress_merge, rd_batch_egress), and the butterfly route
(rd_route_path) - the ctypes wrapper of include/rd_chain.h.

Buffers are device pointers (integers); the merge is asynchronous on the
given stream (0: the legacy default stream)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import abi


def packet_words(packet_w: int) -> int:
    """u32 words of one detection packet: its flits times the flit's words."""
    L = abi.load()
    return L.rd_detection_flits(packet_w) * L.rd_flit_words(packet_w)


def route_path(src: int, dest: int, radix: int, stages: int) -> list[int]:
    """packet_model::route_path (packet_model.hpp:283-303): the wire out of
    every stage, path[0] = src; the last equals dest."""
    L = abi.load()
    path = (C.c_uint32 * (stages + 1))()
    abi.check(L, L.rd_route_path(src, dest, radix, stages, path), "rd_route_path")
    return list(path)


@dataclass
class Source:
    flits: int            # device pointer to whole packets
    n_packets: int        # packets, or the bound on *count_dev
    dest: int             # egress port
    count_dev: int = 0    # device pointer to a u64 packet count, or 0


def egress_merge(sources: list[Source], packet_w: int, n_ports: int, ring: int,
                 cap_per_port: int, port_count: int, src_of: int = 0, stream: int = 0) -> None:
    """rd_egress_merge: ring [n_ports][cap_per_port] packets, src_of
    [n_ports][cap_per_port] u32, port_count [n_ports] u64 (all device)."""
    L = abi.load()
    arr = (abi.RdEgressSource * len(sources))()
    for a, s in zip(arr, sources):
        a.flits, a.count_dev = s.flits, s.count_dev or None
        a.n_packets, a.dest = s.n_packets, s.dest
    abi.check(L, L.rd_egress_merge(arr, len(sources), packet_w, n_ports, C.c_void_p(ring),
                                   cap_per_port, C.c_void_p(src_of or None),
                                   C.c_void_p(port_count), C.c_void_p(stream)), "rd_egress_merge")
