"""The host code that runs on the CPU, built with AddressSanitizer and
UndefinedBehaviorSanitizer (any finding aborts the process):

  * the C oracle (oracle/Makefile `san`): the oracle's own tests run against
    it in a child process that preloads libasan;
  * the C++ facade's file loaders (tests/cpp/Makefile `san`): the golden PFB
    coefficient and vector files parse, and malformed variants - truncated at
    many offsets, tokens replaced by garbage, huge or negative numbers,
    header counts that disagree with the rows, lines dropped or repeated -
    come back as a failed load with a diagnosis, never as a sanitizer report
    or a crash.

No GPU is used: the facade binary links the CUDA library but the loaders
never call it."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
SAN_MARKERS = ("AddressSanitizer", "runtime error", "UndefinedBehaviorSanitizer", "LeakSanitizer")


def _libasan() -> str:
    return subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True,
                          check=True).stdout.strip()


def _clean(r):
    out = r.stdout + r.stderr
    return not any(m in out for m in SAN_MARKERS), out[-3000:]


def test_oracle_under_sanitizers():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "san"], check=True)
    env = dict(os.environ, RD_ORACLE_LIB="san", LD_PRELOAD=_libasan(),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=0")
    r = subprocess.run([sys.executable, "-m", "pytest", str(ROOT / "tests" / "test_oracle.py"),
                        "-q", "-m", "not gpu", "-p", "no:cacheprovider"],
                       capture_output=True, text=True, env=env, cwd=str(ROOT), timeout=900)
    ok, tail = _clean(r)
    assert r.returncode == 0 and ok, tail
    assert " passed" in r.stdout


def _variants(text: str, rng) -> list[tuple[bool, str]]:
    """Malformed copies of a loader file's text, each with whether the
    reference's loader (pfb_model.hpp:356-544) refuses it for certain. It is
    lenient by design: a header-only file is an empty bank, an out-of-range
    integer is taken as strtoll leaves it, unknown header values are ignored;
    the facade keeps that, so only the certain refusals are asserted."""
    lines = text.splitlines()
    head = [i for i, ln in enumerate(lines) if ln.startswith("#")]
    body = [i for i, ln in enumerate(lines) if not ln.startswith("#")]
    out = []
    # truncated mid-file: before the schema line (refused), inside the header
    # (may be an empty bank), inside the rows (fewer than declared: refused),
    # inside the last row (a shortened last number may still parse)
    for frac, refused in ((0.0, True), (0.01, True), (0.1, False), (0.33, True), (0.5, True),
                          (0.77, True), (0.99, False)):
        out.append((refused, text[: int(len(text) * frac)]))
    for tok in ("x", "99999999999999999999", "-1", "", "1e9", "0x10", "nan"):
        i = body[int(rng.integers(0, len(body)))]
        cols = lines[i].split(" ")
        cols[int(rng.integers(0, len(cols)))] = tok
        v = list(lines)
        v[i] = " ".join(cols)
        out.append((False, "\n".join(v) + "\n"))
    for i in head:  # a header line with a garbage value, or dropped
        key = lines[i].split(":")[0]
        v = list(lines)
        v[i] = f"{key}: 4294967296000"
        out.append((False, "\n".join(v) + "\n"))
        out.append((False, "\n".join(lines[:i] + lines[i + 1:]) + "\n"))
    v = list(lines)  # a row repeated, a row dropped, a row cut short
    out.append((False, "\n".join(v + [v[body[-1]]]) + "\n"))
    out.append((False, "\n".join(v[:body[0]] + v[body[0] + 1:]) + "\n"))
    v[body[0]] = " ".join(v[body[0]].split(" ")[:2])
    out.append((True, "\n".join(v) + "\n"))
    return out


def test_facade_loaders_under_sanitizers(tmp_path):
    sys.path.insert(0, str(ROOT / "tests"))
    import test_facade as tf
    from conftest import GOLDEN
    from rdgb import build

    build.build()
    subprocess.run(["make", "-s", "-C", str(ROOT / "tests" / "cpp"), "san"], check=True)
    prog = ROOT / "tests" / "cpp" / "_build" / "facade_check_san"
    z = np.load(GOLDEN / "block_vectors.npz")
    good = ["pfb_mixed_p4t8", "pfb_random_p8t16"]
    for name in good:
        tf._write_pfb_files(z, name, tmp_path)
    rng = np.random.default_rng(7)
    bad, refused = [], []
    for name in good:
        for ext, other in ((".coeff", ".vec"), (".vec", ".coeff")):
            text = (tmp_path / (name + ext)).read_text()
            for k, (must_fail, v) in enumerate(_variants(text, rng)):
                vn = f"{name}_bad{ext[1:]}{k}"
                (tmp_path / (vn + ext)).write_text(v)
                (tmp_path / (vn + other)).write_text((tmp_path / (name + other)).read_text())
                bad.append(vn)
                if must_fail:
                    refused.append(vn)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([str(prog), "loaders", str(tmp_path), *good, *bad], capture_output=True,
                       text=True, env=env, timeout=600)
    ok, tail = _clean(r)
    assert r.returncode == 0 and ok, tail
    status = {}
    for ln in (tmp_path / "status.txt").read_text().splitlines():
        name, state, *why = ln.split(" ", 2)
        status[name] = (state, " ".join(why))
    for name in good:
        assert status[name][0] == "ok", status[name]
    assert len(bad) > 60 and all(n in status for n in bad)
    # the certain refusals are refused; every refusal says why
    assert all(status[n][0] == "fail" for n in refused), [(n, status[n]) for n in refused]
    assert all(status[n][1].strip() for n in bad if status[n][0] == "fail")
