"""Per-block parity on the GPU, through the C ABI: the reference's golden
vectors and the CPU oracle on seeded random and directed cases. Bit-exact."""
import numpy as np
import pytest

from helpers import (accum_replay, cfar_config, clutter_edge_cells, event_fields, hadamard_case,
                     orthogonal_pair, rne15)
from rdgb import abi, chain as gc, scenario as sc

pytestmark = pytest.mark.gpu


def rnd(rng, n):
    return rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)


def test_fxp_ops_vectors(gpulib, blockvec):
    z = blockvec
    y, fl = gc.fxp(z["fxp_op"], z["fxp_a"], z["fxp_b"], z["fxp_sh"], z["fxp_w"])
    assert np.array_equal(y, z["fxp_y"])
    assert np.array_equal(fl, z["fxp_flags"])


def test_fxp_accum_vectors(gpulib, blockvec):
    # the saturating accumulator sequences of fxp_accum.vec, step by step
    # through the GPU's add-and-saturate
    z = blockvec
    y, fl, st, ct = accum_replay(gc.fxp, z)
    assert np.array_equal(y, z["accum_y"])
    assert np.array_equal(fl, z["accum_step_flags"])
    assert np.array_equal(st, z["accum_sticky"])
    assert np.array_equal(ct, z["accum_count"])


def test_cmult_vectors(gpulib, blockvec):
    z = blockvec
    a, b = z["cmult_a"], z["cmult_b"]
    n = len(a)
    ops = np.concatenate([np.full(n, abi.OP_CODE["cmul_re"]), np.full(n, abi.OP_CODE["cmul_im"])])
    y, fl = gc.fxp(ops, np.concatenate([a, a]).astype(np.int64),
                   np.concatenate([b, b]).astype(np.int64), np.zeros(2 * n), np.zeros(2 * n))
    yre, yim = sc.unpack(z["cmult_y"])
    assert np.array_equal(y[:n], yre) and np.array_equal(y[n:], yim)
    assert np.array_equal(fl[:n], z["cmult_f_re"]) and np.array_equal(fl[n:], z["cmult_f_im"])


def test_fxp_random_vs_oracle(gpulib, port):
    rng = np.random.default_rng(3)
    n = 20000
    op = rng.integers(0, 15, n).astype(np.uint32)
    a = rng.integers(-2**62, 2**62, n, dtype=np.int64)
    b = rng.integers(-2**62, 2**62, n, dtype=np.int64)
    sh = rng.integers(0, 70, n).astype(np.uint32)
    w = rng.integers(0, 70, n).astype(np.uint32)
    yg, fg = gc.fxp(op, a, b, sh, w)
    yo, fo = port.fxp(op, a, b, sh, w)
    assert np.array_equal(yg, yo) and np.array_equal(fg, fo)


def test_fft64_vectors(gpulib, blockvec):
    z = blockvec
    n, spc = int(z["fft_n"]), int(z["fft_spc"])
    for r in range(len(z["fft_sched"])):
        out, _, sf = gc.fft(n, spc, int(z["fft_sched"][r]), int(z["fft_reorder"][r]), z["fft_x"][r])
        assert np.array_equal(out, z["fft_y"][r]), f"record {r}"
        assert np.array_equal(sf, z["fft_stage_flags"][r]), f"record {r} flags"


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("spc", [1, 2])
def test_fft_random_vs_oracle(gpulib, port, n, spc):
    rng = np.random.default_rng(n * 10 + spc)
    frames = 37
    x = rnd(rng, frames * n)
    # small-amplitude frames too, so both saturating and clean paths run
    x[: 10 * n] = sc.pack(rng.integers(-900, 900, 10 * n), rng.integers(-900, 900, 10 * n))
    for sched in (0xFFFFFFFF, 0, int(rng.integers(0, 2**32))):
        for reorder in (0, 1):
            g = gc.fft(n, spc, sched, reorder, x)
            o = port.fft(n, spc, sched, reorder, x)
            for a, b in zip(g, o):
                assert np.array_equal(a, b), (n, spc, sched, reorder)


def test_fft_directed(gpulib, port):
    # impulse, DC, Nyquist, negative and two tones, full-scale (test_fft.cpp cases)
    n = 256
    t = np.arange(n)
    cases = [np.eye(1, n, 0)[0] * 32767, np.full(n, 12000.0),
             20000 * np.cos(np.pi * t), 15000 * np.exp(-2j * np.pi * 37 * t / n),
             9000 * np.exp(2j * np.pi * 5 * t / n) + 9000 * np.exp(2j * np.pi * 77 * t / n),
             np.full(n, -32768 - 32768j)]
    x = np.concatenate([sc.pack(np.clip(np.round(np.real(c)), -32768, 32767),
                                np.clip(np.round(np.imag(c)), -32768, 32767)) for c in cases])
    for sched in (0xFFFFFFFF, 0x0, 0x155):
        g = gc.fft(n, 2, sched, 1, x)
        o = port.fft(n, 2, sched, 1, x)
        for a, b in zip(g, o):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("idx", range(10))
def test_pfb_vectors(gpulib, blockvec, idx):
    z = blockvec
    name = str(z["pfb_sets"][idx])
    P, T = int(z[f"{name}_P"]), int(z[f"{name}_T"])
    x = z[f"{name}_x"]
    y, fl, _ = gc.pfb(P, T, z[f"{name}_coeff"], np.zeros((T - 1) * P, np.uint32), x)
    assert np.array_equal(y.reshape(x.shape), z[f"{name}_y"]), name
    assert np.array_equal((fl >> 2).reshape(x.shape), z[f"{name}_f_re"]), name
    assert np.array_equal((fl & 3).reshape(x.shape), z[f"{name}_f_im"]), name


@pytest.mark.parametrize("P,T", [(4, 8), (16, 4), (256, 8), (1024, 16), (7, 3), (64, 1)])
def test_pfb_random_vs_oracle(gpulib, port, P, T):
    rng = np.random.default_rng(P + T)
    c = rnd(rng, P * T)
    st = rnd(rng, max(T - 1, 1) * P) if T > 1 else np.zeros(P, np.uint32)
    x = rnd(rng, 23 * P)
    g = gc.pfb(P, T, c, st[: (T - 1) * P] if T > 1 else st[:0], x)
    o = port.pfb(P, T, c, st[: (T - 1) * P] if T > 1 else st[:0], x)
    for a, b in zip(g, o):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("A,B", [(4, 2), (16, 16), (64, 64), (5, 3), (128, 7)])
def test_bf_random_vs_oracle(gpulib, port, A, B):
    rng = np.random.default_rng(A * B)
    w, x = rnd(rng, A * B), rnd(rng, 300 * A)
    for a, b in zip(gc.bf(A, B, w, x), port.bf(A, B, w, x)):
        assert np.array_equal(a, b)


def test_bf_directed(gpulib, port):
    # beamformer_model.hpp:375-427: unit, zero, max and permuted weights
    A, B = 16, 8
    rng = np.random.default_rng(5)
    x = rnd(rng, 50 * A)
    unit = np.zeros(A * B, np.uint32)
    for b in range(B):
        unit[b * A + (b * 3) % A] = sc.pack(32767, 0)
    y, _, fl = gc.bf(A, B, unit, x)
    xr, xi = sc.unpack(x.reshape(50, A))

    def rne15(v):  # round_sat(v, 15, 16) for |v| < 2^31
        q, rem = v >> 15, v & 0x7FFF
        return np.clip(q + (rem > 0x4000) + ((rem == 0x4000) & (q & 1)), -32768, 32767)
    yr, yi = sc.unpack(y.reshape(50, B))
    for b in range(B):
        a = (b * 3) % A  # the passthrough gain is 32767/32768 (beamformer_model.hpp:366-391)
        assert np.array_equal(yr[:, b], rne15(xr[:, a] * 32767))
        assert np.array_equal(yi[:, b], rne15(xi[:, a] * 32767))
    assert not fl.any()
    y0, acc0, f0 = gc.bf(A, B, np.zeros(A * B, np.uint32), x)
    assert not y0.any() and not acc0.any() and not f0.any()
    mx = np.full(A * B, 0x80008000, np.uint32)
    full = np.full(20 * A, 0x80008000, np.uint32)
    for a_, b_ in zip(gc.bf(A, B, mx, full), port.bf(A, B, mx, full)):
        assert np.array_equal(a_, b_)
    ym, _, fm = gc.bf(A, B, mx, full)
    assert (fm != 0).all()
    # consistent antenna permutation is exact (metamorphic relation)
    perm = rng.permutation(A)
    w = rnd(rng, A * B)
    wp = np.zeros_like(w)
    for b in range(B):
        wp[b * A + perm] = w[b * A:(b + 1) * A]
    xp = np.zeros_like(x).reshape(50, A)
    xp[:, perm] = x.reshape(50, A)
    assert np.array_equal(gc.bf(A, B, w, x)[0], gc.bf(A, B, wp, xp.reshape(-1))[0])


def test_power_cross_vs_oracle(gpulib, port):
    rng = np.random.default_rng(9)
    x, y = rnd(rng, 5000), rnd(rng, 5000)
    x[:4] = [0x80008000, 0x7FFF7FFF, 0x80007FFF, 0]
    assert np.array_equal(gc.power(x), port.power(x))
    assert gc.power(x)[0] == 2**31
    assert np.array_equal(gc.cross_power(x, y), port.cross_power(x, y))
    # X = Y gives a real result (covariance directed case)
    c = gc.cross_power(x, x).reshape(-1, 2)
    assert (c[:, 1] == 0).all() and np.array_equal(c[:, 0], gc.power(x))


def cfar_cfg(mode, out, gl, gg, rl, rg, alpha, mg=4, mr=16, enable=1):
    c = sc.make_config(sc.preset("tiny"))
    c.cfar_mode, c.cfar_out_mode, c.cfar_enable = mode, out, enable
    c.guard_lead, c.guard_lag, c.ref_lead, c.ref_lag = gl, gg, rl, rg
    c.alpha, c.max_guard, c.max_ref = alpha, mg, mr
    return c


@pytest.mark.parametrize("mode", [abi.RD_CFAR_CA, abi.RD_CFAR_GO])
@pytest.mark.parametrize("out", [abi.RD_CFAR_EVENTS, abi.RD_CFAR_DENSE])
def test_cfar_random_vs_oracle(gpulib, port, mode, out):
    rng = np.random.default_rng(mode * 2 + out)
    for n in (16, 64, 256, 1000, 1024):
        frames = 9
        cells = rng.exponential(1000.0, frames * n).astype(np.int64)
        cells[rng.integers(0, cells.size, 30)] *= 40      # targets
        cells[:3] = [-5, 2**31, 0]                       # clamp and the largest power
        fid = rng.integers(0, 2**16, frames).astype(np.uint32)
        for geo in ((2, 2, 8, 8), (0, 3, 5, 0), (4, 4, 16, 16), (6, 1, 40, 2)):
            cfg = cfar_cfg(mode, out, *geo, int(rng.integers(0, 5000)))
            g, o = gc.cfar(cells, n, cfg, fid), port.cfar(cells, n, cfg, fid)
            assert np.array_equal(g, o), (n, geo)


@pytest.mark.parametrize("mode", [abi.RD_CFAR_CA, abi.RD_CFAR_GO])
def test_cfar_large_cells_vs_oracle(gpulib, port, mode):
    # cells near 2^26: a frame's total passes 2^32 while every window sum
    # stays below it (the 32-bit scan, wrapping), and frames with a cell
    # whose windows may pass 2^32 (the 64-bit scan) in the same launch
    rng = np.random.default_rng(11 + mode)
    n, frames = 1024, 12
    cells = rng.integers(2**25, 2**26, frames * n).astype(np.int64)
    cells[rng.integers(0, cells.size, 40)] = 2**26 - 1
    cells[3 * n + 500] = 2**27          # 33 x 2^27 > 2^32: that frame scans in 64 bits
    cells[7 * n + 9] = 2**32 + 5        # a cell above 32 bits
    cells[9 * n:10 * n] = 2**31 - 1     # every cell at the 31-bit power limit
    fid = np.arange(frames, dtype=np.uint32)
    for out in (abi.RD_CFAR_EVENTS, abi.RD_CFAR_DENSE):
        for geo, alpha in (((4, 4, 16, 16), 333), ((2, 2, 8, 8), 320), ((0, 3, 5, 0), 256)):
            cfg = cfar_cfg(mode, out, *geo, alpha)
            g, o = gc.cfar(cells, n, cfg, fid), port.cfar(cells, n, cfg, fid)
            assert np.array_equal(g, o), (out, geo)
            if out == abi.RD_CFAR_EVENTS and geo[2] == 16:
                assert (event_fields(g)["kind"] == 0).any()


@pytest.mark.parametrize("mode", [abi.RD_CFAR_CA, abi.RD_CFAR_GO])
@pytest.mark.parametrize("out", [abi.RD_CFAR_EVENTS, abi.RD_CFAR_DENSE])
def test_cfar_short_frames_vs_oracle(gpulib, port, mode, out):
    # frames of at most 64 cells run several to a warp (16, 32 or 64 cells a
    # frame slot): every length around the slot sizes, lengths that are not
    # a multiple of 4 (scalar loads), frame counts that leave a warp's last
    # slots empty, and cells past 32 bits in some frames (the 64-bit scan)
    rng = np.random.default_rng(40 + mode * 2 + out)
    for n in (1, 3, 5, 12, 15, 16, 17, 20, 31, 32, 33, 36, 47, 63, 64):
        for frames in (1, 3, 9, 37):
            cells = rng.exponential(1000.0, frames * n).astype(np.int64)
            cells[rng.integers(0, cells.size, 8)] *= 40
            if frames > 3:
                cells[n + rng.integers(0, n)] = 2**33 + 7
            fid = rng.integers(0, 2**16, frames).astype(np.uint32)
            for geo in ((1, 1, 4, 4), (0, 2, 3, 0), (2, 0, 6, 6), (1, 1, 2, 1)):
                cfg = cfar_cfg(mode, out, *geo, int(rng.integers(0, 3000)))
                g, o = gc.cfar(cells, n, cfg, fid), port.cfar(cells, n, cfg, fid)
                assert np.array_equal(g, o), (n, frames, geo)


@pytest.mark.parametrize("n,frames", [(16, 50000), (48, 40000), (1024, 5000)])
def test_cfar_many_frames_vs_oracle(gpulib, port, n, frames):
    # more frames than one wave of the persistent decide grid holds, so warps
    # take several frame groups each
    rng = np.random.default_rng(n + frames)
    cells = rng.exponential(1000.0, frames * n).astype(np.int64)
    cells[rng.integers(0, cells.size, frames // 4)] *= 40
    fid = (np.arange(frames) % 65536).astype(np.uint32)
    for mode in (abi.RD_CFAR_CA, abi.RD_CFAR_GO):
        cfg = cfar_cfg(mode, abi.RD_CFAR_EVENTS, 1, 1, 4, 4, 2600)
        g, o = gc.cfar(cells, n, cfg, fid), port.cfar(cells, n, cfg, fid)
        assert np.array_equal(g, o), mode


def test_cfar_directed(gpulib, port):
    n = 128
    cells = np.full(n, 100, np.int64)
    cells[60] = 100 * 9          # injected target: CUT*N*256 vs alpha*sum
    cells[100], cells[102] = 5000, 5000  # closely spaced pair, outside bin 60's window
    # threshold flip: alpha exactly at the boundary and one LSB below
    for alpha, want in ((9 * 256 - 1, True), (9 * 256, False)):
        cfg = cfar_cfg(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS, 2, 2, 8, 8, alpha)
        ev = gc.cfar(cells[None, :].repeat(1, 0), n, cfg, [3])
        f = event_fields(ev)
        assert (60 in set(f["bin"][f["kind"] == 0])) == want
        assert np.array_equal(ev, port.cfar(cells, n, cfg, [3]))
    # disabled CFAR: every bin suppressed, only the summary
    cfg = cfar_cfg(abi.RD_CFAR_CA, abi.RD_CFAR_EVENTS, 2, 2, 8, 8, 256, enable=0)
    ev = gc.cfar(cells, n, cfg, [0])
    f = event_fields(ev)
    assert len(ev) == 1 and f["kind"][0] == 3 and f["sup"][0] == n
    # a window that does not fit the frame suppresses the edges
    cfg = cfar_cfg(abi.RD_CFAR_CA, abi.RD_CFAR_DENSE, 4, 4, 16, 16, 256)
    f = event_fields(gc.cfar(cells, n, cfg, [0]))
    assert (f["kind"][:20] == 2).all() and (f["kind"][-21:-1] == 2).all()


@pytest.mark.parametrize("pw", [64, 96, 128, 256, 512])
def test_packetize_vs_oracle(gpulib, port, pw):
    rng = np.random.default_rng(pw)
    ev = np.zeros(200, abi.EVENT_DTYPE)
    ev["w"] = rng.integers(0, 2**63, size=(200, 3), dtype=np.int64).astype(np.uint64)
    ev["w"][:, 2] &= (1 << 48) - 1
    g = gc.packetize(ev, pw, src=3, dest=9, vc=2, seq0=65530)
    o = port.packetize(ev, pw, src=3, dest=9, vc=2, seq0=65530)
    assert np.array_equal(g, o)
    # every flit has odd parity (packet_model.hpp:221-226)
    pop = np.array([sum(bin(int(v)).count("1") for v in row) for row in g])
    assert (pop % 2 == 1).all()


# ---- directed and metamorphic cases of the reference's block tests (their
# oracle-side twins are in test_oracle.py)

def test_hadamard_bank_directed(gpulib, port):
    A, frames = 16, 200
    w, x, row, s = hadamard_case(A, frames, np.random.default_rng(21))
    g = gc.bf(A, A, w, x)
    for a, b in zip(g, port.bf(A, A, w, x)):
        assert np.array_equal(a, b)
    yr, yi = sc.unpack(g[0].reshape(frames, A))
    want = np.zeros((frames, A), np.int64)
    want[np.arange(frames), row] = rne15(A * 32767 * s)
    assert np.array_equal(yr, want) and not yi.any() and not g[2].any()


def test_cfar_clutter_edge_ca_vs_go(gpulib, port):
    cells = clutter_edge_cells()
    got = {}
    for mode in (abi.RD_CFAR_CA, abi.RD_CFAR_GO):
        cfg = cfar_config(mode, abi.RD_CFAR_EVENTS, 2, 2, 8, 8, 384)
        ev = gc.cfar(cells, 128, cfg, [0])
        assert np.array_equal(ev, port.cfar(cells, 128, cfg, [0]))
        got[mode] = event_fields(ev)
    ca, go = got[abi.RD_CFAR_CA], got[abi.RD_CFAR_GO]
    det_ca = set(ca["bin"][ca["kind"] == 0].tolist())
    assert det_ca and det_ca <= set(range(64, 72))
    assert not (go["kind"] == 0).any()


@pytest.mark.parametrize("mode", [abi.RD_CFAR_CA, abi.RD_CFAR_GO])
def test_cfar_halving_invariance(gpulib, port, mode):
    rng = np.random.default_rng(22 + mode)
    n, frames = 256, 12
    half = rng.integers(0, 4000, frames * n).astype(np.int64)
    half[rng.integers(0, half.size, 60)] *= 30
    cfg = cfar_config(mode, abi.RD_CFAR_DENSE, 2, 3, 8, 12, 900)
    ea = gc.cfar(half, n, cfg, np.arange(frames))
    eb = gc.cfar(2 * half, n, cfg, np.arange(frames))
    assert np.array_equal(ea, port.cfar(half, n, cfg, np.arange(frames)))
    assert np.array_equal(eb, port.cfar(2 * half, n, cfg, np.arange(frames)))
    a, b = event_fields(ea), event_fields(eb)
    assert (a["kind"] == 0).sum() > 20
    for k in ("kind", "bin", "frame_id", "ref_cnt", "det", "sup"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(2 * a["cut"], b["cut"]) and np.array_equal(2 * a["sum"], b["sum"])


def test_cross_power_orthogonal(gpulib, port):
    rng = np.random.default_rng(23)
    x = rnd(rng, 4000)
    re, im = sc.unpack(x)
    x = sc.pack(re, np.where(im == -32768, 0, im))
    y = orthogonal_pair(x)
    c = gc.cross_power(x, y)
    assert np.array_equal(c, port.cross_power(x, y))
    c = c.reshape(-1, 2)
    assert not c[:, 0].any() and np.array_equal(c[:, 1], -gc.power(x))
