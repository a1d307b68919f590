"""Generates rdgb/twiddle.py and csrc/twiddle_q15.inc: the 1024-entry Q1.15
twiddle table W_1024^e = exp(-j 2 pi e / 1024), packed {im, re}.

The integers must equal the reference's committed table (model/cpp/fft/
fft_twiddle_table.hpp:43, digest c756048fbc00d64f) bit for bit, because every
FFT quantisation multiplies by them. The method is the published one of the
reference's generator (model/python/gen_fft_twiddles.py:97-162): reduce the
angle to the first quadrant so the four axis points are exact, take cos/sin
in double precision, round to nearest even at 2^15, saturate to 16 bits.

    python agilex-7-radar-detect_gb300/rdgb/gen_twiddle.py
"""
from __future__ import annotations

import hashlib
import math
from pathlib import Path

N = 1024
DIGEST = "c756048fbc00d64f"


def _q15(x: float) -> int:
    v = int(round(x * 32768.0))   # Python round(): ties to even
    return max(-32768, min(32767, v))


def table() -> list[int]:
    out = []
    for e in range(N):
        quadrant, rem = divmod(e, N // 4)
        if rem == 0:
            c0, s0 = 1.0, 0.0
        else:
            th = 2.0 * math.pi * rem / N
            c0, s0 = math.cos(th), math.sin(th)
        c, s = [(c0, s0), (-s0, c0), (-c0, -s0), (s0, -c0)][quadrant]
        re, im = _q15(c), _q15(-s)
        out.append(((im & 0xFFFF) << 16) | (re & 0xFFFF))
    return out


def digest(t: list[int]) -> str:
    h = hashlib.sha256()
    for w in t:
        h.update(w.to_bytes(4, "little"))
    return h.hexdigest()[:16]


def main() -> None:
    t = table()
    d = digest(t)
    if d != DIGEST:
        raise SystemExit(f"twiddle digest {d} != {DIGEST}")
    here = Path(__file__).resolve().parent
    rows = [", ".join(f"0x{w:08X}u" for w in t[i:i + 8]) for i in range(0, N, 8)]
    (here.parent / "csrc" / "twiddle_q15.inc").write_text(
        "/* Generated by rdgb/gen_twiddle.py: W_1024^e, Q1.15 packed {im, re}.\n"
        f" * digest {d} (sha256 of the little-endian words, first 16 hex). */\n"
        + ",\n".join(rows) + "\n")
    (here / "twiddle.py").write_text(
        '"""Generated by rdgb/gen_twiddle.py: W_1024^e, Q1.15 packed {im, re}."""\n'
        f"DIGEST = \"{d}\"\nTWIDDLES = [\n"
        + "".join(f"    {', '.join(f'0x{w:08X}' for w in t[i:i + 8])},\n" for i in range(0, N, 8))
        + "]\n")
    print(f"wrote twiddle tables, digest {d}")


if __name__ == "__main__":
    main()
