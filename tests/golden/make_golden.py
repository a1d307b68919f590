"""Generates the golden fixtures under tests/golden/ (run where the reference
checkout exists; the GPU host only reads the committed .npz files).

  block_vectors.npz  the reference's own golden vectors, parsed from
                     model/vectors: fxp_ops.vec (1457 ops), fxp_accum.vec
                     (251 accumulator steps in 19 sequences), cmult.vec (864
                     products), fft64.vec (36 records, N=64, spc=2) and the
                     ten pfb_<set>_<geometry>.{coeff,vec} files (96 beats each)
  chain_<name>.npz   seeded chain scenarios run through oracle/_ref (the
                     composition driver over the reference's model/cpp
                     headers): inputs, configuration and every output

    python tests/golden/make_golden.py [--reference /path/to/reference] [--blocks-only]
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "oracle"))
sys.path.insert(0, str(REPO / "agilex-7-radar-detect_gb300"))

import orc  # noqa: E402
from rdgb import abi, scenario as sc  # noqa: E402


def _lines(path: Path):
    for line in path.read_text().splitlines():
        line = line.strip()
        if line and not line.startswith("#"):
            yield line.split()


def _header(path: Path) -> dict:
    h = {}
    for line in path.read_text().splitlines():
        if line.startswith("#") and ":" in line:
            k, v = line[1:].split(":", 1)
            h[k.strip()] = v.strip()
    return h


def parse_fxp_ops(path: Path) -> dict:
    rows = list(_lines(path))
    return {
        "op": np.array([abi.OP_CODE[r[1]] for r in rows], np.uint32),
        "a": np.array([int(r[2]) for r in rows], np.int64),
        "b": np.array([int(r[3]) for r in rows], np.int64),
        "sh": np.array([int(r[4]) for r in rows], np.uint32),
        "w": np.array([int(r[5]) for r in rows], np.uint32),
        "y": np.array([int(r[6]) for r in rows], np.int64),
        "flags": np.array([int(r[7]) for r in rows], np.uint8),
    }


def parse_fxp_accum(path: Path) -> dict:
    """fxp_accum.vec: sequences of saturating accumulator steps (fxp::Acc,
    fxp.hpp:384-420), each from a cleared accumulator at its step 0; per
    step the width, the addend, the value after it, the step's flags, the
    sticky flags and the flagged-step count (fxp_vectors.hpp:73-90)."""
    rows = list(_lines(path))
    names, seq = [], []
    for r in rows:
        if int(r[1]) == 0:
            names.append(r[0])
        assert names and r[0] == names[-1], r
        seq.append(len(names) - 1)
    return {
        "names": np.array(names),
        "seq": np.array(seq, np.uint32),
        "step": np.array([int(r[1]) for r in rows], np.uint32),
        "w": np.array([int(r[2]) for r in rows], np.uint32),
        "x": np.array([int(r[3]) for r in rows], np.int64),
        "y": np.array([int(r[4]) for r in rows], np.int64),
        "step_flags": np.array([int(r[5]) for r in rows], np.uint8),
        "sticky": np.array([int(r[6]) for r in rows], np.uint8),
        "count": np.array([int(r[7]) for r in rows], np.uint32),
    }


def parse_cmult(path: Path) -> dict:
    rows = np.array([[int(v) for v in r[1:]] for r in _lines(path)], np.int64)
    return {"a": sc.pack(rows[:, 0], rows[:, 1]), "b": sc.pack(rows[:, 2], rows[:, 3]),
            "p_re": rows[:, 4], "p_im": rows[:, 5], "y": sc.pack(rows[:, 6], rows[:, 7]),
            "f_re": rows[:, 8].astype(np.uint8), "f_im": rows[:, 9].astype(np.uint8)}


def parse_fft(path: Path) -> dict:
    h = _header(path)
    n = int(h["fft_size"])
    stages = int(h["stages"])
    recs, cur = [], None
    for r in _lines(path):
        if r[0] == "vec":
            cur = {"sched": int(r[2], 16), "reorder": int(r[3]), "flags": int(r[4], 16),
                   "x": [], "y": []}
            recs.append(cur)
        else:
            cur["x"].append((int(r[2]), int(r[3])))
            cur["y"].append((int(r[4]), int(r[5])))
    x = np.array([sc.pack([v[0] for v in c["x"]], [v[1] for v in c["x"]]) for c in recs])
    y = np.array([sc.pack([v[0] for v in c["y"]], [v[1] for v in c["y"]]) for c in recs])
    fl = np.array([[(c["flags"] >> (2 * g)) & 3 for g in range(stages)] for c in recs], np.uint8)
    return {"n": np.uint32(n), "spc": np.uint32(int(h["spc"])),
            "sched": np.array([c["sched"] for c in recs], np.uint32),
            "reorder": np.array([c["reorder"] for c in recs], np.uint32),
            "x": x, "y": y, "stage_flags": fl}


def parse_pfb(coeff: Path, vec: Path) -> dict:
    ch = _header(coeff)
    P, T = int(ch["phases"]), int(ch["taps"])
    crow = np.array([[int(v) for v in r] for r in _lines(coeff)], np.int64)
    assert (crow[:, 0] == np.arange(P * T)).all()
    c = sc.pack(crow[:, 3], crow[:, 4])
    rows = np.array([[int(v) for v in r] for r in _lines(vec)], np.int64)
    xs = rows[:, 1:1 + 2 * P]
    ys = rows[:, 1 + 2 * P:1 + 4 * P]
    fs = rows[:, 1 + 4 * P:]
    return {"P": np.uint32(P), "T": np.uint32(T), "coeff": c,
            "x": sc.pack(xs[:, 0::2], xs[:, 1::2]), "y": sc.pack(ys[:, 0::2], ys[:, 1::2]),
            "f_re": fs[:, 0::2].astype(np.uint8), "f_im": fs[:, 1::2].astype(np.uint8)}


def block_vectors(ref: Path) -> dict:
    v = ref / "model" / "vectors"
    out = {}
    for k, a in parse_fxp_ops(v / "fxp_ops.vec").items():
        out[f"fxp_{k}"] = a
    for k, a in parse_fxp_accum(v / "fxp_accum.vec").items():
        out[f"accum_{k}"] = a
    for k, a in parse_cmult(v / "cmult.vec").items():
        out[f"cmult_{k}"] = a
    for k, a in parse_fft(v / "fft64.vec").items():
        out[f"fft_{k}"] = a
    names = []
    for cf in sorted(v.glob("pfb_*.coeff")):
        name = cf.stem
        names.append(name)
        for k, a in parse_pfb(cf, v / f"{name}.vec").items():
            out[f"{name}_{k}"] = a
    out["pfb_sets"] = np.array(names)
    return out


# ---------------------------------------------------------------------------
# chain scenarios
# ---------------------------------------------------------------------------

def _cfg_dict(cfg) -> dict:
    return {f"cfg_{k}": np.uint32(v) for k, v in cfg.as_dict().items()}


def chain_case(name, p, frames_per_call, coeff=None, weights=None, mod=None, taps=True):
    cfg = sc.make_config(p, max_frames=max(frames_per_call))
    if mod:
        mod(cfg)
    px, py = sc.pair_table(p)
    coeff = sc.coefficients(p.n_fft, p.taps) if coeff is None else coeff
    weights = sc.steering_weights(p.n_chan, p.n_beams) if weights is None else weights
    total = sum(frames_per_call)
    adc = sc.adc(p, total * p.n_fft)
    o = orc.Oracle("ref")
    ch = o.chain(cfg, coeff, weights, px, py)
    out = {"adc": adc, "coeff": coeff, "weights": weights, "px": px, "py": py,
           "calls": np.array(frames_per_call, np.uint32), **_cfg_dict(cfg)}
    f0 = 0
    for i, nf in enumerate(frames_per_call):
        r = ch.process(adc[:, f0 * p.n_fft:(f0 + nf) * p.n_fft], taps=taps)
        for k, v in r.items():
            if isinstance(v, np.ndarray):
                out[f"c{i}_{k}"] = v
        st = ch.stats()
        out[f"c{i}_stats_keys"] = np.array(list(st.keys()))
        out[f"c{i}_stats_vals"] = np.array([np.array(v, np.uint64).sum() if isinstance(v, list) else v
                                            for v in st.values()], np.uint64)
        out[f"c{i}_fft_stage_flags"] = np.array(st["fft_stage_flags"], np.uint32)
        f0 += nf
    fl = ch.flush_cov()
    out["flush_cov_windows"] = fl["cov_windows"]
    out["flush_cov_acc"] = fl["cov_acc"]
    # the history as align would read it, after the last call
    hv = [ch.read_history(b, off) for off in range(0, min(p.hist_frames, 6)) for b in (0, 1, p.n_fft - 1)]
    out["hist_vec"] = np.array([h[0] for h in hv])
    out["hist_fid"] = np.array([h[1] for h in hv], np.uint32)
    out["hist_flags"] = np.array([h[2] for h in hv], np.uint32)
    np.savez_compressed(HERE / f"chain_{name}.npz", **out)
    n_ev = sum(len(out[f"c{i}_events"]) for i in range(len(frames_per_call)))
    print(f"chain_{name}: {total} frames, {n_ev} events")


def chain_fixtures() -> None:
    rng = np.random.default_rng(7)
    chain_case("tiny", sc.preset("tiny"), [256])
    chain_case("tiny_calls", sc.preset("tiny"), [17, 100, 139], taps=False)
    chain_case("ref_tiny", sc.preset("ref_tiny"), [64])
    chain_case("medium_slice", sc.preset("medium", cov_window=16), [40], taps=False)

    def go_dense(c):
        c.cfar_mode, c.cfar_out_mode = abi.RD_CFAR_GO, abi.RD_CFAR_DENSE
    chain_case("tiny_go_dense", sc.preset("tiny"), [64], mod=go_dense, taps=False)

    def sat(c):
        c.scale_sched = 0b10101
        c.cov_mode, c.cov_exp_k, c.cov_window, c.cov_acc_w = abi.RD_COV_EXP, 3, 7, 34
    p = sc.preset("tiny")
    chain_case("tiny_sat", p, [64], mod=sat,
               coeff=rng.integers(0, 2**32, size=p.n_fft * p.taps, dtype=np.uint64).astype(np.uint32),
               weights=np.full(p.n_chan * p.n_beams, 0x80008000, np.uint32))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(orc.REF_SOURCES))
    ap.add_argument("--blocks-only", action="store_true",
                    help="write block_vectors.npz alone (the chain fixtures stay as they are)")
    args = ap.parse_args()
    ref = Path(args.reference)
    orc.REF_SOURCES = ref
    np.savez_compressed(HERE / "block_vectors.npz", **block_vectors(ref))
    print("block_vectors.npz written")
    if args.blocks_only:
        return
    orc.build("port")
    orc.build("ref")
    chain_fixtures()


if __name__ == "__main__":
    main()
