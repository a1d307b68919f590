"""Test infrastructure: the packet fabric's checkers, restated on the CPU.

Only tests/ may use this module; nothing on the product path imports it.

* ``Scoreboard`` - the reference's ``packet_model::Scoreboard``
  (model/cpp/packet/packet_model.hpp:323-586): packets are injected per
  (src, VC, dest) triple, every flit seen at an egress port is observed, and
  the run is finished; it counts delivered, lost, duplicated, misrouted,
  corrupted, reordered, framing, parity and unexpected packets and keeps the
  "src.vc.dest#seq" delivery log.
* ``rr_arbiter_order`` - the egress order of round-robin arbitration, one
  arbiter per port (rtl/packet/pkt_rr_arb.sv:1-150), simulated grant by grant.
* ``route_path`` - the butterfly route (packet_model.hpp:266-309).

Flits are rows of little-endian 32-bit words (word 0 holds flit bits 31..0),
the layout the chain writes: parity bit 0 (odd over the flit), VC bits 1-2,
SOF bit 3, EOF bit 4, then the packet_w payload bits; a header flit's payload
holds dest 4 | src 5 | vc 2 | type 3 | length 6 | seq 16 from bit 0
(packet_model.hpp:64-98).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

DEST_W, SRC_W, VC_W, TYPE_W, LEN_W, SEQ_W = 4, 5, 2, 3, 6, 16
HDR_W = DEST_W + SRC_W + VC_W + TYPE_W + LEN_W + SEQ_W
MAX_FLITS = 32
CTRL_W = 5
TYPE_RAW = 5
COUNT_KEYS = ("delivered", "lost", "duplicated", "misrouted", "corrupted", "reordered",
              "framing", "parity", "unexpected")


@dataclass(frozen=True)
class Header:
    dest: int = 0
    src: int = 0
    vc: int = 0
    ptype: int = 0
    length: int = 1
    seq: int = 0


def hdr_unpack(v: int) -> Header:
    """packet_model.hpp:155-164"""
    f, o = [], 0
    for w in (DEST_W, SRC_W, VC_W, TYPE_W, LEN_W, SEQ_W):
        f.append((v >> o) & ((1 << w) - 1))
        o += w
    return Header(*f)


def hdr_pack(h: Header) -> int:
    """packet_model.hpp:144-153"""
    v, o = 0, 0
    for x, w in zip((h.dest, h.src, h.vc, h.ptype, h.length, h.seq),
                    (DEST_W, SRC_W, VC_W, TYPE_W, LEN_W, SEQ_W)):
        v |= (x & ((1 << w) - 1)) << o
        o += w
    return v


def flit_words(packet_w: int) -> int:
    return (packet_w + CTRL_W + 31) // 32


def detection_flits(packet_w: int) -> int:
    return 1 + (176 + packet_w - 1) // packet_w


def to_int(row) -> int:
    return int.from_bytes(np.ascontiguousarray(row, np.uint32).tobytes(), "little")


def from_int(v: int, packet_w: int) -> np.ndarray:
    n = flit_words(packet_w)
    return np.frombuffer(v.to_bytes(4 * n, "little"), np.uint32).copy()


class Flit:
    """One flit as an integer of packet_w + 5 bits (packet_model.hpp:173-235)."""

    __slots__ = ("v", "packet_w")

    def __init__(self, v: int, packet_w: int):
        self.v, self.packet_w = v, packet_w

    @classmethod
    def from_row(cls, row, packet_w: int) -> "Flit":
        return cls(to_int(row) & ((1 << (packet_w + CTRL_W)) - 1), packet_w)

    @property
    def vc(self) -> int:
        return (self.v >> 1) & 3

    @property
    def sof(self) -> bool:
        return bool((self.v >> 3) & 1)

    @property
    def eof(self) -> bool:
        return bool((self.v >> 4) & 1)

    @property
    def data(self) -> int:
        return self.v >> CTRL_W

    def parity_ok(self) -> bool:
        return bin(self.v).count("1") & 1 == 1

    def header(self) -> Header:
        return hdr_unpack(self.data & ((1 << HDR_W) - 1))


def make_flit(packet_w: int, vc: int, sof: bool, eof: bool, data: int) -> Flit:
    """packet_model.hpp:237-256: the fields, then odd parity over the flit."""
    v = ((data & ((1 << packet_w) - 1)) << CTRL_W) | (int(eof) << 4) | (int(sof) << 3) | \
        ((vc & 3) << 1)
    if bin(v).count("1") % 2 == 0:
        v |= 1
    return Flit(v, packet_w)


@dataclass
class Packet:
    hdr: Header
    payload: list = field(default_factory=list)  # one int per payload flit

    def flits(self, packet_w: int) -> list:
        n = 1 + len(self.payload)
        out = [make_flit(packet_w, self.hdr.vc, True, n == 1, hdr_pack(self.hdr))]
        for i, d in enumerate(self.payload):
            out.append(make_flit(packet_w, self.hdr.vc, False, i == n - 2, d))
        return out


def packets_from_flits(flits: np.ndarray, packet_w: int) -> list:
    """Split a buffer of whole packets (each starting with its header flit)
    into Packets, the form ``Scoreboard.inject`` takes."""
    rows = np.asarray(flits, np.uint32).reshape(-1, flit_words(packet_w))
    out, i = [], 0
    while i < len(rows):
        h = Flit.from_row(rows[i], packet_w).header()
        n = max(1, h.length)
        out.append(Packet(h, [Flit.from_row(rows[i + k], packet_w).data for k in range(1, n)]))
        i += n
    return out


def route_path(src: int, dest: int, radix: int, stages: int) -> list:
    """packet_model.hpp:283-303: stage s switches on digit stages-1-s, and
    the wire out of it carries the destination's digit there."""
    path, cur = [src], src
    for s in range(stages):
        scale = radix ** (stages - 1 - s)
        sw = cur // (scale * radix) * scale + cur % scale
        cur = sw // scale * scale * radix + (dest // scale) % radix * scale + sw % scale
        path.append(cur)
    return path


def route_path_ok(src: int, dest: int, radix: int, stages: int) -> bool:
    p = route_path(src, dest, radix, stages)
    return bool(p) and p[-1] == dest


def rr_arbiter_order(n_packets, dests, n_ports: int) -> list:
    """Per egress port, the (source, packet index) sequence one round-robin
    arbiter grants when every source of the port has its packets queued
    (pkt_rr_arb.sv: grant the lowest requester at or after the pointer, else
    the lowest requester; the pointer moves one past the grant)."""
    out = []
    for d in range(n_ports):
        srcs = [s for s in range(len(n_packets)) if dests[s] == d]
        left = [int(n_packets[s]) for s in srcs]
        sent = [0] * len(srcs)
        order, ptr = [], 0
        while any(left):
            req = [k for k in range(len(srcs)) if left[k] > 0]
            hi = [k for k in req if k >= ptr]
            g = hi[0] if hi else req[0]
            order.append((srcs[g], sent[g]))
            sent[g] += 1
            left[g] -= 1
            ptr = 0 if g == len(srcs) - 1 else g + 1
        out.append(order)
    return out


class Scoreboard:
    """packet_model::Scoreboard (packet_model.hpp:323-586), check for check."""

    def __init__(self, packet_w: int, radix: int, stages: int):
        self.packet_w, self.radix, self.stages = packet_w, radix, stages
        self.counts = dict.fromkeys(COUNT_KEYS, 0)
        self.injected = 0
        self.expected: dict = {}
        self.open: dict = {}
        self.per_src: dict = {}
        self.per_vc: dict = {}
        self.notes: list = []
        self.log: list = []

    def _note(self, s: str) -> None:
        if len(self.notes) < 64:
            self.notes.append(s)

    def total_errors(self) -> int:
        return sum(v for k, v in self.counts.items() if k != "delivered")

    def inject(self, p: Packet) -> None:
        """packet_model.hpp:346-357"""
        self.expected.setdefault((p.hdr.src, p.hdr.vc, p.hdr.dest), []).append(p)
        self.injected += 1
        if not route_path_ok(p.hdr.src, p.hdr.dest, self.radix, self.stages):
            self.counts["misrouted"] += 1
            self._note(f"injected packet src={p.hdr.src} dest={p.hdr.dest} has no route")

    def observe(self, port: int, f: Flit) -> None:
        """packet_model.hpp:360-432"""
        if not f.parity_ok():
            self.counts["parity"] += 1
            self._note(f"flit at egress {port} failed parity")
        vc = f.vc
        key = (port, vc)
        o = self.open.setdefault(key, {"active": False})
        if f.sof:
            if o["active"]:
                self.counts["framing"] += 1
                self._note(f"SOF inside an open packet at egress {port} VC {vc}")
            h = f.header()
            o = {"active": True, "hdr": h, "remaining": h.length - 1 if h.length > 1 else 0,
                 "payload": []}
            self.open[key] = o
            if not 1 <= h.length <= MAX_FLITS:
                self.counts["framing"] += 1
                self._note(f"illegal declared length {h.length}")
            if h.dest != port:
                self.counts["misrouted"] += 1
                self._note(f"packet for dest {h.dest} arrived at egress {port}")
            if h.vc != vc:
                self.counts["framing"] += 1
                self._note(f"header VC {h.vc} but flit VC {vc}")
            if h.ptype > TYPE_RAW:
                self.counts["framing"] += 1
                self._note(f"reserved packet type {h.ptype}")
            if f.eof != (h.length == 1):
                self.counts["framing"] += 1
                self._note(f"header EOF disagrees with a declared length of {h.length}")
            if o["remaining"] == 0:
                self._complete(port, o)
            return
        if not o["active"]:
            self.counts["framing"] += 1
            self._note(f"body flit with no open packet at egress {port} VC {vc}")
            return
        o["payload"].append(f.data)
        if o["remaining"] > 0:
            o["remaining"] -= 1
        if f.eof:
            if o["remaining"] != 0:
                self.counts["framing"] += 1
                self._note(f"EOF with {o['remaining']} flits still expected")
            self._complete(port, o)
        elif o["remaining"] == 0:
            self.counts["framing"] += 1
            self._note(f"packet ran past its declared length at egress {port}")

    def observe_rows(self, port: int, rows) -> None:
        for row in np.asarray(rows, np.uint32).reshape(-1, flit_words(self.packet_w)):
            self.observe(port, Flit.from_row(row, self.packet_w))

    def finish(self) -> None:
        """packet_model.hpp:435-452"""
        for q in self.expected.values():
            for p in q:
                self.counts["lost"] += 1
                self._note(f"never delivered: src={p.hdr.src} vc={p.hdr.vc} "
                           f"dest={p.hdr.dest} seq={p.hdr.seq}")
        for (port, vc), o in self.open.items():
            if o["active"]:
                self.counts["framing"] += 1
                self._note(f"packet still open at egress {port} VC {vc} at end of run")

    def _complete(self, port: int, o: dict) -> None:
        """packet_model.hpp:511-573"""
        h = o["hdr"]
        q = self.expected.get((h.src, h.vc, h.dest))
        o["active"] = False
        if not q:
            self.counts["unexpected"] += 1
            self._note(f"delivered a packet nobody injected: src={h.src} vc={h.vc} "
                       f"dest={h.dest} seq={h.seq}")
            return
        idx = next((i for i, p in enumerate(q) if p.hdr.seq == h.seq), None)
        if idx is None:
            self.counts["duplicated"] += 1
            self._note(f"duplicate or unknown seq {h.seq} for src={h.src} vc={h.vc} "
                       f"dest={h.dest}")
            return
        if idx != 0:
            self.counts["reordered"] += 1
            self._note(f"out of order within (src={h.src},vc={h.vc},dest={h.dest}): "
                       f"seq {h.seq} arrived {idx} early")
        want = q[idx]
        if want.hdr != h:
            self.counts["corrupted"] += 1
            self._note(f"header mismatch for seq {h.seq}")
        elif len(want.payload) != len(o["payload"]):
            self.counts["corrupted"] += 1
            self._note(f"payload flit count {len(o['payload'])} but expected "
                       f"{len(want.payload)}")
        else:
            for i, (a, b) in enumerate(zip(want.payload, o["payload"])):
                if a != b:
                    self.counts["corrupted"] += 1
                    self._note(f"payload word {i} of seq {h.seq} differs")
                    break
        del q[idx]
        self.counts["delivered"] += 1
        self.per_src[(port, h.src)] = self.per_src.get((port, h.src), 0) + 1
        self.per_vc[(port, h.vc)] = self.per_vc.get((port, h.vc), 0) + 1
        self.log.append(f"{h.src}.{h.vc}.{h.dest}#{h.seq}")
