"""Parity of the GPU path with the reference at the benchmark shapes.

Fixtures (tests/golden/make_golden.py, outputs of the reference's own code):
  c0_shape.npz  receptor 1,500 / ligand 1,000 atoms, L = 15, 51 q; 1,354
                poses: every pose of z = 30 and z = 36 in the 10,000-pose
                list, and a 34-pose triple that the reference scores on its
                FFTW branch
  c1_shape.npz  receptor 3,500 / ligand 2,000 atoms, L = 20, 101 q; 400
                poses: every pose of 24 triples of the 210,000-pose list and
                two 40-pose FFTW-branch triples
The GPU expands the stored atoms itself, so each test runs the product path
from atoms to chi.

Plain FP64 path (the bound: 1e-10 relative in I(q) and chi, identical best
grid cells):
  * expansion: each sampled A_lm, B_lm within 1e-12 of the largest |A_lm| of
    its channel and q;
  * raw cross terms of the detail poses (the first three triples) within
    1e-10 of the largest |term| of the same pose and channel;
  * chi^2 over the (c1, c2) grid of the detail poses: 1e-10 relative;
  * best grid chi of every pose: 1e-10 relative; best cell identical, or
    tied with the reference's best within 1e-10;
  * I(q) of every pose at the reference's best cell: 1e-10 relative;
  * L-BFGS-B fit: chi within 1e-8 relative, c1 and c2 within 1e-6 of the
    reference's own fit (its iterates follow rounding-level differences).
Mixed path (the bound: |dchi| <= 1e-4 chi, top-100 overlap >= 99 %):
  * best grid chi of every pose within 1e-4 relative of the reference's;
  * of the reference's 100 best poses by chi, at least 99 among the mixed
    path's 100 best;
  * I(q) of every pose at the reference's best cell within 1e-5 relative.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SHAPES = ["c0_shape", "c1_shape"]
TOL = 1e-10


def load_shape(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz"), allow_pickle=False))


def expand_pair(gpu, g):
    L, q, h2o = int(g["L"]), g["q"], float(g["h2o"])
    A = gpu.expand(g["rec_xyz"], g["rec_vac"], g["rec_dum"], g["rec_sasa"], h2o, q, L)
    B = gpu.expand(g["lig_xyz"], g["lig_vac"], g["lig_dum"], g["lig_sasa"], h2o, q, L)
    return A, B


def sample_err(full, at, want, Q):
    """max |full[at] - want| relative to the largest |entry| of the same channel and q"""
    f = full.reshape(3, Q, -1)
    scale = np.abs(f).max(axis=2).reshape(-1)          # [3 Q]
    row = at // f.shape[2]
    return float(np.max(np.abs(full[at] - want) / scale[row]))


def chan_err(x, y):
    sc = np.max(np.abs(y), axis=-1, keepdims=True)
    sc[sc == 0] = 1.0
    return float(np.max(np.abs(x - y) / sc))


def intensities(oracle, g, cross):
    """I(q) of each pose from raw cross terms, at the reference's best cell
    (peak rescale, then sxs_compile_intensity)"""
    n2 = len(g["c2g"])
    out = np.empty((len(cross), len(g["q"])))
    for i, c in enumerate(cross):
        s = oracle.rescale(c.reshape(-1), float(g["peak"]))
        cell = int(g["cell"][i])
        out[i] = oracle.compile_intensity(s, g["q"], float(g["rm"]), g["c1g"][cell // n2], g["c2g"][cell % n2])[0]
    return out


def run_plan(gpu, g, A, B, precision, fit):
    p = gpu.Plan(A, B, g["q"], g["z"], int(g["L"]), g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"],
                 precision=precision)
    p.set_poses(g["index"], skip=int(g["skip"]))
    p.run(fit)
    r = p.results(cross=True, grid=fit == gpu.FIT_GRID)
    p.close()
    return r


@pytest.mark.parametrize("name", SHAPES)
def test_fp64_matches_reference_at_benchmark_shape(gpu, oracle, name):
    g = load_shape(name)
    Q = len(g["q"])
    A, B = expand_pair(gpu, g)
    assert sample_err(A, g["A_at"], g["A_val"], Q) <= 1e-12
    assert sample_err(B, g["B_at"], g["B_val"], Q) <= 1e-12
    r = run_plan(gpu, g, A, B, gpu.FP64, gpu.FIT_GRID)
    d = g["detail"]
    assert chan_err(r["cross"][d], g["raw"]) <= TOL
    np.testing.assert_allclose(r["grid"][d], g["grid"], rtol=TOL, atol=0)
    best = g["best"]
    np.testing.assert_allclose(r["chi"], np.sqrt(best), rtol=TOL, atol=0)
    grid = r["grid"].reshape(len(best), -1)
    same = r["cell"] == g["cell"]
    # a different cell only where the reference's own grid ties it
    tied = np.abs(grid[np.arange(len(best)), g["cell"]] - best) <= TOL * best
    assert np.all(same | tied), "best cells differ"
    iq = intensities(oracle, g, r["cross"])
    np.testing.assert_allclose(iq, g["iq"], rtol=TOL, atol=0)


@pytest.mark.parametrize("name", SHAPES)
def test_fp64_lbfgsb_matches_reference_at_benchmark_shape(gpu, name):
    g = load_shape(name)
    A, B = expand_pair(gpu, g)
    r = run_plan(gpu, g, A, B, gpu.FP64, gpu.FIT_LBFGSB)
    np.testing.assert_allclose(r["chi"], g["chi"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(r["c1"], g["c1"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(r["c2"], g["c2"], rtol=0, atol=1e-6)


@pytest.mark.parametrize("name", SHAPES)
def test_mixed_within_bound_of_reference_at_benchmark_shape(gpu, oracle, name):
    g = load_shape(name)
    A, B = expand_pair(gpu, g)
    r = run_plan(gpu, g, A, B, gpu.MIXED, gpu.FIT_GRID)
    chi_ref = np.sqrt(g["best"])
    dchi = np.abs(r["chi"] - chi_ref) / chi_ref
    assert dchi.max() <= 1e-4, "max |dchi|/chi %.3g" % dchi.max()
    top_ref = set(np.argsort(chi_ref, kind="stable")[:100].tolist())
    top_mix = set(np.argsort(r["chi"], kind="stable")[:100].tolist())
    overlap = len(top_ref & top_mix) / 100.0
    assert overlap >= 0.99, "top-100 overlap %.2f" % overlap
    iq = intensities(oracle, g, r["cross"])
    rel = np.abs(iq - g["iq"]) / np.abs(g["iq"])
    assert rel.max() <= 1e-5, "max I(q) relative error %.3g" % rel.max()
