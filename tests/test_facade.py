"""The C++ facade (include/rd_model.hpp) as a caller of the reference model's
C++ API uses it: tests/cpp/facade_check.cpp is compiled against the header
and the CUDA library with the committed recipe (tests/cpp/Makefile), run on
inputs written here, and its outputs are compared with the CPU oracle.

  * CPU: the header compiles under -Wall -Wextra -Werror; the .coeff / .vec
    loaders (pfb_model.hpp:356-544) parse the reference's PFB golden files,
    written out here in their format from the parsed fixture (and the
    reference's own files, where a reference checkout is present), and refuse
    a truncated file with a diagnosis.
  * GPU: PfbModel (beat by beat, a bank swap that keeps the history, then
    step_many), fft::transform_many / transform, BeamformerModel::step (whole
    BeamBeat: y, flags, exact accumulators, saturating; a weight swap) in
    both contraction forms, split_beat, the directed weight sets, power and
    cross power, cfar::run_frame / run_frames, detection packets read back
    through Flit and Header, and rdgb::Chain - bit for bit; an invalid
    geometry comes back as a status, not an exception.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN
from rdgb import abi, scenario as sc

ROOT = Path(__file__).resolve().parent.parent
CPP = ROOT / "tests" / "cpp"
PROG = CPP / "_build" / "facade_check"
PFB_SETS = [f"pfb_{s}_{g}" for s in ("ident", "max", "mixed", "proto", "random")
            for g in ("p4t8", "p8t16")]


@pytest.fixture(scope="module")
def prog():
    from rdgb import build
    build.build()
    subprocess.run(["make", "-s", "-C", str(CPP)], check=True)
    return PROG


def _run(prog, *args):
    r = subprocess.run([str(prog), *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def _status(d):
    out = {}
    for ln in (Path(d) / "status.txt").read_text().splitlines():
        name, state, *why = ln.split(" ", 2)
        out[name] = (state, " ".join(why))
    return out


def _out(d, name, dtype):
    return np.fromfile(Path(d) / f"{name}.out", dtype=dtype)


def _write_pfb_files(z, name, d):
    """The fixture's parsed PFB set back in the reference's file format."""
    P, T = int(z[f"{name}_P"]), int(z[f"{name}_T"])
    re, im = sc.unpack(z[f"{name}_coeff"])
    lines = ["# pfb coefficient file", "# schema: 1", "# kind: pfb_coeff", f"# set: {name}",
             f"# phases: {P}", f"# taps: {T}", "# rounding_mode: nearest_even",
             f"# count: {P * T}"]
    lines += [f"{p * T + t} {p} {t} {re[p * T + t]} {im[p * T + t]}"
              for p in range(P) for t in range(T)]
    (Path(d) / f"{name}.coeff").write_text("\n".join(lines) + "\n")
    x, y = z[f"{name}_x"], z[f"{name}_y"]
    fr, fi = z[f"{name}_f_re"], z[f"{name}_f_im"]
    acc_w = 32 + int(np.ceil(np.log2(2 * T)))
    lines = ["# pfb vector file", "# schema: 1", "# kind: pfb_io", f"# phases: {P}", f"# taps: {T}",
             f"# acc_w: {acc_w}", f"# count: {len(x)}", "# columns: beat x y f"]
    for b in range(len(x)):
        xr, xi = sc.unpack(x[b])
        yr, yi = sc.unpack(y[b])
        cols = [b] + [v for p in range(P) for v in (xr[p], xi[p])] + \
            [v for p in range(P) for v in (yr[p], yi[p])] + \
            [v for p in range(P) for v in (fr[b][p], fi[b][p])]
        lines.append(" ".join(str(int(c)) for c in cols))
    (Path(d) / f"{name}.vec").write_text("\n".join(lines) + "\n")


def _check_loaded(d, z, names):
    st = _status(d)
    for name in names:
        assert st[name][0] == "ok", st[name]
        assert st[name + "_truncated"][0] == "ok", st[name + "_truncated"]
        P, T = int(z[f"{name}_P"]), int(z[f"{name}_T"])
        geo = _out(d, f"{name}_geo", np.uint32)
        assert geo.tolist() == [P, T, P, T, 32 + int(np.ceil(np.log2(2 * T))), 96]
        assert np.array_equal(_out(d, f"{name}_coeff", np.uint32), z[f"{name}_coeff"])
        assert np.array_equal(_out(d, f"{name}_x", np.uint32), z[f"{name}_x"].reshape(-1))
        assert np.array_equal(_out(d, f"{name}_y", np.uint32), z[f"{name}_y"].reshape(-1))
        f = (z[f"{name}_f_re"].astype(np.uint32) << 2) | z[f"{name}_f_im"]
        assert np.array_equal(_out(d, f"{name}_f", np.uint32), f.reshape(-1))


def test_header_compiles_strict(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text('#include "rd_model.hpp"\nint main() { return rdgb::last_status(); }\n')
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    f"-I{ROOT / 'include'}", "-fsyntax-only", str(src)], check=True)


def test_loaders_parse_the_golden_files(prog, tmp_path):
    z = np.load(GOLDEN / "block_vectors.npz")
    for name in PFB_SETS:
        _write_pfb_files(z, name, tmp_path)
    _run(prog, "loaders", tmp_path, *PFB_SETS)
    _check_loaded(tmp_path, z, PFB_SETS)


def test_loaders_parse_the_reference_files(prog, tmp_path):
    import shutil

    import orc
    vec = orc.REF_SOURCES / "model" / "vectors"
    if not vec.exists():
        pytest.skip("no reference checkout here")
    for name in PFB_SETS:
        for ext in (".coeff", ".vec"):
            shutil.copy(vec / (name + ext), tmp_path / (name + ext))
    _run(prog, "loaders", tmp_path, *PFB_SETS)
    _check_loaded(tmp_path, np.load(GOLDEN / "block_vectors.npz"), PFB_SETS)


def _rnd(rng, n):
    return rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)


@pytest.mark.gpu
@pytest.mark.parametrize("form", [abi.RD_FORM_CUDA_CORE, abi.RD_FORM_TENSOR])
def test_facade_vs_oracle(gpulib, port, prog, tmp_path, form):
    rng = np.random.default_rng(41 + form)
    d = tmp_path
    par = {}

    def put(name, arr):
        np.ascontiguousarray(arr).tofile(d / f"{name}.bin")

    # PFB: 8 phases x 16 taps, 40 beats, a bank swap half way
    P, T, beats = 8, 16, 40
    c1, c2 = _rnd(rng, P * T), sc.coefficients(P, T)
    x = _rnd(rng, beats * P)
    par.update(pfb_phases=P, pfb_taps=T, pfb_beats=beats)
    put("pfb_coeff", c1), put("pfb_coeff2", c2), put("pfb_x", x)
    # FFT: 256 points, 2 samples a cycle, a schedule that saturates
    n, frames = 256, 6
    fx = _rnd(rng, n * frames)
    par.update(fft_n=n, fft_spc=2, fft_sched=0xFFFFFFF0, fft_reorder=1, fft_frames=frames)
    put("fft_x", fx)
    # beamformer: 64 antennas, 16 beams, 2 bins a beat, 12 beats, a weight swap
    A, B, J, nb = 64, 16, 2, 12
    w1, w2 = _rnd(rng, A * B), sc.steering_weights(A, B)
    bx = _rnd(rng, nb * J * A)
    par.update(bf_ant=A, bf_beams=B, bf_binpar=J, bf_beats=nb, bf_form=form, bf_beam_par=4)
    put("bf_w", w1), put("bf_w2", w2), put("bf_x", bx)
    # power and cross power
    cx, cy = _rnd(rng, 1000), _rnd(rng, 1000)
    put("cv_x", cx), put("cv_y", cy)
    # CFAR: GO mode, 64 cells, 40 frames; 128-bit packets
    cfn, cff = 64, 40
    cells = rng.integers(0, 1 << 20, cfn * cff).astype(np.int64)
    cells[::7] *= 40
    fid = np.arange(1000, 1000 + cff, dtype=np.uint32)
    par.update(cf_n=cfn, cf_mode=1, cf_out=0, cf_gl=2, cf_gg=3, cf_rl=8, cf_rg=6, cf_alpha=0x300,
               cf_max_guard=2, cf_max_ref=8, pk_w=128, pk_src=5, pk_dest=9, pk_vc=2, pk_seq0=65530)
    put("cf_cells", cells), put("cf_fid", fid)
    # the chain: the tiny workload's geometry
    p = sc.preset("tiny")
    cfg = sc.make_config(p, max_frames=32, form=form)
    coeff, w = sc.coefficients(p.n_fft, p.taps), sc.steering_weights(p.n_chan, p.n_beams)
    adc = sc.adc(p, 300 * p.n_fft)
    par.update(ch_chan=p.n_chan, ch_n=p.n_fft, ch_taps=p.taps, ch_beams=p.n_beams,
               ch_window=100, ch_max_frames=32, ch_form=form)
    put("ch_coeff", coeff), put("ch_w", w), put("ch_adc", adc)
    (d / "params.txt").write_text("".join(f"{k} {v}\n" for k, v in par.items()))

    _run(prog, "gpu", d)
    st = _status(d)
    assert {k: v[0] for k, v in st.items()} == {k: "ok" for k in st}, st

    # PFB against the oracle with the same swap
    state = np.zeros((T - 1) * P, np.uint32)
    y1, f1, state = port.pfb(P, T, c1, state, x[:beats // 2 * P])
    y2, f2, _ = port.pfb(P, T, c2, state, x[beats // 2 * P:])
    assert np.array_equal(_out(d, "pfb_y", np.uint32), np.concatenate([y1, y2]))
    assert np.array_equal(_out(d, "pfb_f", np.uint8), np.concatenate([f1, f2]))
    # FFT
    out, bins, sf = port.fft(n, 2, 0xFFFFFFF0, 1, fx)
    assert np.array_equal(_out(d, "fft_out", np.uint32), out)
    assert np.array_equal(_out(d, "fft_bins", np.uint32), bins)
    assert np.array_equal(_out(d, "fft_sf", np.uint8), sf)
    # beamformer: the oracle's per-vector results in [beat][beam][bin] order
    nv = nb * J
    half = nb // 2 * J
    ya, acca, fla = port.bf(A, B, w1, bx[:half * A])
    yb, accb, flb = port.bf(A, B, w2, bx[half * A:])
    yv = np.concatenate([ya, yb]).reshape(nb, J, B).transpose(0, 2, 1)
    av = np.concatenate([acca, accb]).reshape(nb, J, B, 2).transpose(0, 2, 1, 3)
    fv = np.concatenate([fla, flb]).reshape(nb, J, B).transpose(0, 2, 1)
    assert np.array_equal(_out(d, "bf_y", np.uint32), yv.reshape(-1))
    assert np.array_equal(_out(d, "bf_acc", np.int64), av.reshape(-1))
    assert np.array_equal(_out(d, "bf_f", np.uint8), fv.reshape(-1))
    assert nv == len(yv) * J
    # split_beat: beam groups of 4, seq with the 2-bit group index appended
    sp = _out(d, "bf_split", np.uint32).reshape(nb, B // 4, 5 + 4 * J)
    for t in range(nb):
        for g in range(B // 4):
            e = sp[t, g]
            assert e[:4].tolist() == [((100 + t) << 2) | g, g, int(t == 0 and g == 0),
                                      int(t == nb - 1 and g == B // 4 - 1)]
            assert e[4] == int(fv[t, 4 * g:4 * g + 4].any())
            assert np.array_equal(e[5:], yv[t, 4 * g:4 * g + 4].reshape(-1))
    # the directed weight sets
    sel = [(3 * b + 1) % A for b in range(B)]
    unit = np.zeros((B, A), np.uint32)
    unit[np.arange(B), sel] = sc.pack(32767, 0)
    assert np.array_equal(_out(d, "bf_unit_w", np.uint32), unit.reshape(-1))
    assert not _out(d, "bf_zero_w", np.uint32).any()
    assert (_out(d, "bf_max_w", np.uint32) == sc.pack(-32768, -32768)).all()
    perm = [(a * 5 + 3) % A for a in range(A)]
    pw = np.zeros((B, A), np.uint32)
    pw[:, perm] = w1.reshape(B, A)
    assert np.array_equal(_out(d, "bf_perm_w", np.uint32), pw.reshape(-1))
    # power, cross power
    assert np.array_equal(_out(d, "cv_power", np.int64), port.power(cx))
    assert np.array_equal(_out(d, "cv_cross", np.int64), port.cross_power(cx, cy))
    # CFAR and packets
    c = abi.RdConfig()
    gpulib.rd_config_default(abi.C.byref(c))
    c.cfar_mode, c.cfar_out_mode, c.alpha = 1, 0, 0x300
    c.guard_lead, c.guard_lag, c.ref_lead, c.ref_lag, c.max_guard, c.max_ref = 2, 3, 8, 6, 2, 8
    want_ev = port.cfar(cells, cfn, c, fid)
    got_ev = np.fromfile(d / "cf_events.out", dtype=abi.EVENT_DTYPE)
    assert len(got_ev) == len(want_ev) > cff
    assert np.array_equal(got_ev["w"], want_ev["w"])
    flits = port.packetize(got_ev, 128, 5, 9, 2, 65530)
    assert np.array_equal(_out(d, "pk_flits", np.uint32), flits.reshape(-1))
    # the chain
    px, py = sc.pair_table(p)
    c2 = abi.RdConfig()  # as the program builds it: the defaults, then its fields
    gpulib.rd_config_default(abi.C.byref(c2))
    c2.n_chan, c2.n_fft, c2.taps, c2.n_beams = p.n_chan, p.n_fft, p.taps, p.n_beams
    c2.cov_window, c2.max_frames, c2.form = 100, 32, form
    c2.guard_lead = c2.guard_lag = 1
    c2.ref_lead = c2.ref_lag = 4
    c2.alpha = 0x800
    ro = port.chain(c2, coeff, w, px, py).process(adc, taps=False, threads=4)
    got = np.fromfile(d / "ch_events.out", dtype=abi.EVENT_DTYPE)
    assert np.array_equal(got, ro["events"])
    assert np.array_equal(_out(d, "ch_flits", np.uint32), ro["flits"].reshape(-1))
    assert np.array_equal(_out(d, "ch_cov", np.int64), ro["cov_acc"].reshape(-1))
    assert os.path.getsize(d / "ch_cov.out") > 0
    # the checkpointed stream: the second half's events as one stream's
    # second call
    h = (adc.shape[1] // p.n_fft // 2) * p.n_fft
    o2 = port.chain(c2, coeff, w, px, py)
    o2.process(np.ascontiguousarray(adc[:, :h]), taps=False, threads=4)
    r2 = o2.process(np.ascontiguousarray(adc[:, h:]), taps=False, threads=4)
    got2 = np.fromfile(d / "ck_events.out", dtype=abi.EVENT_DTYPE)
    assert len(got2) > 0 and np.array_equal(got2, r2["events"])
