"""A C program written against the reference's API (tests/c/dropin_caller.c)
compiles against include/fmftsaxs_gb300.h, links against the product
library, and on a GPU scores the golden fixtures to the reference's outputs.

The CPU tests compile and link only (strict C11 with warnings as errors, and
the header parsed as C++); the GPU test runs the program.
"""
import glob
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "dropin_caller.c")
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dimer_*.npz")))
CHI_TOL = 1e-8
C_TOL = 1e-6


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler on this host")
    return cc


def _build(lib, out_dir):
    so = lib.LIB_PATH
    exe = os.path.join(str(out_dir), "dropin_caller")
    cmd = [_cc(), "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O1",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(so), "-l:" + os.path.basename(so),
           "-Wl,-rpath," + os.path.dirname(so), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_style_caller_compiles_and_links(lib, tmp_path):
    exe = _build(lib, tmp_path)
    assert os.path.exists(exe)
    # every reference symbol the caller uses resolves in the product library
    need = subprocess.run(["nm", "-u", exe], capture_output=True, text=True, check=True).stdout
    used = {line.split()[-1] for line in need.splitlines() if line.split()[-1].startswith("sxs_")}
    assert "sxs_compute_saxs_scores" in used and len(used) >= 8
    have = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True,
                          check=True).stdout
    exported = {line.split()[-1] for line in have.splitlines()}
    assert not (used - exported), sorted(used - exported)


def test_header_parses_as_cplusplus(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler on this host")
    src = tmp_path / "h.cpp"
    src.write_text('#include "fmftsaxs_gb300.h"\nint main() { return sizeof(sxs_profile) > 0 ? 0 : 1; }\n')
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _write_input(path, g):
    L, Q = int(g["L"]), len(g["q"])
    idx = np.ascontiguousarray(g["index"], dtype=np.int32)
    with open(path, "wb") as f:
        f.write(struct.pack("<6i", L, Q, len(g["exp_q"]), len(g["z"]), len(idx), int(g["skip"])))
        f.write(np.array([g["rmA"], g["rmB"], g["rm"]], dtype="<f8").tobytes())
        for k in ("q", "z", "exp_q", "exp_i", "exp_err", "A", "B"):
            f.write(np.ascontiguousarray(g[k], dtype="<f8").tobytes())
        f.write(idx.astype("<i4").tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_reference_style_caller_matches_reference(gpu, tmp_path, path):
    g = dict(np.load(path, allow_pickle=False))
    exe = _build(gpu, tmp_path)
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.txt")
    _write_input(inp, g)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    res = np.loadtxt(out, ndmin=2)
    assert res.shape == (len(g["index"]), 3)
    np.testing.assert_allclose(res[:, 0], g["chi"], rtol=CHI_TOL, atol=0)
    np.testing.assert_allclose(res[:, 1], g["c1"], rtol=0, atol=C_TOL)
    np.testing.assert_allclose(res[:, 2], g["c2"], rtol=0, atol=C_TOL)
