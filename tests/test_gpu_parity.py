"""Parity of the GPU scoring path (through the C ABI) with the reference.

Comparands: the golden fixtures (the reference's own code, see
tests/golden/make_golden.py) and the CPU oracle on fresh seeded inputs.

Tolerances (plain FP64 path, stated by the task as 1e-10 relative in I(q)
and chi with identical best grid cells):
  * cross terms: |gpu - ref| <= 1e-10 x max_q |ref| of the same pose and
    channel (individual cross terms cross zero, so a per-entry relative
    test would divide by ~0);
  * intensity I(q) at any grid cell: 1e-10 relative;
  * chi^2 at every grid cell and the best chi: 1e-10 relative;
  * best (c1, c2) cell identical, or tied with the reference's best within
    the same 1e-10.
The GPU evaluates the reference's angular DFT in factorized form with
per-angle phases; with the truncated-pi twiddles of the reference's
simple_ft branch this moves I(q) by ~1e-12 relative (measured), well
inside the bound.
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dimer_*.npz")))
TOL = 1e-10


def load(path):
    return dict(np.load(path, allow_pickle=False))


def chan_err(x, y):
    sc = np.max(np.abs(y), axis=-1, keepdims=True)
    sc[sc == 0] = 1.0
    return float(np.max(np.abs(x - y) / sc))


def intensity(oracle, cross_scaled, q, rm, c1, c2):
    return np.array([oracle.compile_intensity(c.reshape(-1), q, rm, c1, c2)[0] for c in cross_scaled])


def check_fit(res, grid_ref, c1g, c2g):
    """best cell identical (or tied within TOL) and chi within TOL"""
    g = grid_ref.reshape(len(grid_ref), -1)
    best = g.min(axis=1)
    cell = res["cell"][:len(g)]
    chosen = g[np.arange(len(g)), cell]
    assert np.all(np.abs(chosen - best) <= TOL * np.abs(best))
    np.testing.assert_allclose(res["chi"][:len(g)], np.sqrt(best), rtol=TOL, atol=0)
    np.testing.assert_array_equal(res["c1"][:len(g)], c1g[cell // len(c2g)])
    np.testing.assert_array_equal(res["c2"][:len(g)], c2g[cell % len(c2g)])


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_expansion_matches_reference_fixture(gpu, path):
    g = load(path)
    L = int(g["L"])
    A = gpu.expand(g["rec_xyz"], g["rec_vac"], g["rec_dum"], g["rec_sasa"], float(g["h2o"]), g["q"], L)
    B = gpu.expand(g["lig_xyz"], g["lig_vac"], g["lig_dum"], g["lig_sasa"], float(g["h2o"]), g["q"], L)
    A0 = gpu.expand(g["rec_xyz"], g["rec_vac"], g["rec_dum"], None, float(g["h2o"]), g["q"], L)
    Q = len(g["q"])
    for got, want in ((A, g["A"]), (B, g["B"]), (A0, g["A_nowater"])):
        assert chan_err(got.reshape(3, Q, -1), want.reshape(3, Q, -1)) <= 1e-12


def test_expansion_edge_cases_match_oracle(gpu, oracle):
    q = oracle.mkarray(0.0, 0.5, 7)
    L = 5
    # no atoms: all zero
    z = gpu.expand(np.zeros((0, 3)), np.zeros(0), np.zeros(0), None, 3.5, q, L)
    assert np.all(z == 0)
    # one atom, and atoms on the z axis / at the origin (the reference's
    # spherical coordinates give NaN there: acos(0/0))
    xyz = np.array([[1.0, 2.0, -3.0], [0.0, 0.0, 4.0], [0.0, 0.0, 0.0], [-7.5, 0.2, 1.0]])
    vac, dum, sasa = np.array([6.0, 7.0, 8.0, 16.0]), np.array([5.5, 0.8, 3.0, 6.6]), np.array([0.3, 0.0, 1.0, 0.5])
    for sel in ([0], [0, 3], [1], [2]):
        got = gpu.expand(xyz[sel], vac[sel], dum[sel], sasa[sel], 3.5, q, L)
        want = oracle.expand(xyz[sel], vac[sel], dum[sel], sasa[sel], 3.5, q, L)
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        if ok.any():
            np.testing.assert_allclose(got[ok], want[ok], rtol=1e-12, atol=1e-12 * np.abs(want[ok]).max())


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_scoring_matches_reference_fixture(gpu, oracle, path):
    g = load(path)
    L, skip = int(g["L"]), int(g["skip"])
    p = gpu.Plan(g["A"], g["B"], g["q"], g["z"], L, g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"])
    p.set_poses(g["index"], skip=skip)
    p.run(gpu.FIT_GRID)
    res = p.results(cross=True, grid=True)
    assert chan_err(res["cross"], g["raw"]) <= TOL
    rows = g["grid"].shape[0]
    np.testing.assert_allclose(res["grid"][:rows], g["grid"], rtol=TOL, atol=0)
    check_fit(res, g["grid"], g["c1g"], g["c2g"])
    # I(q) at the best cell and at two corner cells, from the rescaled cross terms
    scaled = np.array([oracle.rescale(c.reshape(-1), float(g["peak"])) for c in res["cross"]])
    for c1, c2 in ((g["c1g"][0], g["c2g"][0]), (g["c1g"][-1], g["c2g"][-1]), (1.0, 1.0)):
        ig = intensity(oracle, scaled, g["q"], float(g["rm"]), c1, c2)
        ir = intensity(oracle, g["scaled"].reshape(len(scaled), -1), g["q"], float(g["rm"]), c1, c2)
        np.testing.assert_allclose(ig, ir, rtol=TOL, atol=0)
    p.close()


def _random_case(oracle, L, Q, nr, na, npose, seed):
    from libfmftsaxs_gb300 import synth
    import libfmftsaxs_gb300 as g
    rng = np.random.default_rng(seed)
    rec = synth.make_molecule(nr, 8.0, seed).with_sasa()
    lig = synth.make_molecule(na, 7.0, seed + 1).with_sasa()
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    q = oracle.mkarray(0.0, 0.5, Q) if Q > 1 else np.zeros(1)
    ffr = np.array([g.ff_type(e) for e in rec.elements])
    ffl = np.array([g.ff_type(e) for e in lig.elements])
    A = oracle.expand(rec.xyz, ffr[:, 0], ffr[:, 1], rec.sasa, g.ff_water(), q, L)
    B = oracle.expand(lig.xyz, ffl[:, 0], ffl[:, 1], lig.sasa, g.ff_water(), q, L)
    I = np.exp(-np.arange(Q) * 0.3) * 1e6
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    rm = 1.7
    a, mult, peak = oracle.opt_params(eq, ei, ee, q, rm)
    z = np.arange(8.0, 15.0)
    N, nb = 2 * L + 1, L + 1
    idx = rng.integers(0, len(z) * nb * nb * N ** 3, size=npose).astype(np.int32)
    return dict(A=A, B=B, q=q, z=z, L=L, a=a, mult=mult, peak=peak, index=idx)


@pytest.mark.parametrize("L,Q,skip", [(1, 4, 1), (2, 3, 0), (4, 9, 1), (9, 12, 0), (15, 8, 1)])
def test_scoring_matches_oracle_random(gpu, oracle, L, Q, skip):
    from libfmftsaxs_gb300 import synth
    c = _random_case(oracle, L, Q, 60, 40, 120, seed=L * 100 + Q)
    raw, scl, grid, br = oracle.score(c["A"], c["B"], c["q"], c["z"], L, c["index"], skip, c["peak"], c["a"],
                                      c["mult"], synth.C1_GRID, synth.C2_GRID)
    p = gpu.Plan(c["A"], c["B"], c["q"], c["z"], L, c["a"], c["mult"], c["peak"], synth.C1_GRID, synth.C2_GRID)
    p.set_poses(c["index"], skip=skip)
    p.run(gpu.FIT_GRID)
    res = p.results(cross=True, grid=True)
    assert chan_err(res["cross"], raw) <= TOL
    np.testing.assert_allclose(res["grid"], grid, rtol=TOL, atol=0)
    check_fit(res, grid, synth.C1_GRID, synth.C2_GRID)


def test_single_q_point(gpu, oracle):
    from libfmftsaxs_gb300 import synth
    c = _random_case(oracle, 3, 1, 30, 20, 25, seed=5)
    raw, scl, grid, br = oracle.score(c["A"], c["B"], c["q"], c["z"], 3, c["index"], 1, c["peak"], c["a"],
                                      c["mult"], synth.C1_GRID, synth.C2_GRID)
    r = gpu.score_flat(c["A"], c["B"], c["q"], c["z"], 3, c["index"], c["a"], c["mult"], c["peak"], 1, gpu.FIT_NONE,
                       cross=True)
    assert chan_err(r["cross"], raw) <= TOL


def test_chunked_translation_is_identical(gpu, oracle):
    g = load(GOLDEN[-1])
    L = int(g["L"])
    out = []
    for budget in (None, 1):
        p = gpu.Plan(g["A"], g["B"], g["q"], g["z"], L, g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"])
        if budget:
            p.set_budget(budget)  # one (z, b2, g2) combo per chunk
        p.set_poses(g["index"], skip=1)
        p.run(gpu.FIT_GRID)
        out.append(p.results(cross=True))
        p.close()
    np.testing.assert_array_equal(out[0]["cross"], out[1]["cross"])
    np.testing.assert_array_equal(out[0]["chi"], out[1]["chi"])


def test_plan_reuse_and_pose_list_changes(gpu):
    g = load(GOLDEN[0])
    L = int(g["L"])
    p = gpu.Plan(g["A"], g["B"], g["q"], g["z"], L, g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"])
    p.set_poses(g["index"], skip=1)
    p.run(gpu.FIT_GRID)
    r1 = p.results(cross=True)
    p.run(gpu.FIT_GRID)
    r2 = p.results(cross=True)
    np.testing.assert_array_equal(r1["cross"], r2["cross"])
    # a sub-list alone: same cross terms as in the full list (each pose is independent)
    sub = np.arange(0, len(g["index"]), 7)
    p.set_poses(g["index"][sub], skip=1)
    p.run(gpu.FIT_GRID)
    r3 = p.results(cross=True)
    np.testing.assert_array_equal(r3["cross"], r1["cross"][sub])
    # empty list
    p.set_poses(np.zeros(0, dtype=np.int64), skip=1)
    p.run(gpu.FIT_GRID)
    assert len(p.results()["chi"]) == 0
    p.close()


def test_invalid_pose_indices_are_rejected(gpu):
    g = load(GOLDEN[0])
    L = int(g["L"])
    N, nb = 2 * L + 1, L + 1
    p = gpu.Plan(g["A"], g["B"], g["q"], g["z"], L, g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"])
    with pytest.raises(gpu.SxsError, match="negative"):
        p.set_poses(np.array([5, -1]), skip=1)
    with pytest.raises(gpu.SxsError, match="znum"):
        p.set_poses(np.array([len(g["z"]) * nb * nb * N ** 3]), skip=1)
    # the first bad pose in list order is the one reported, as in the
    # reference's sequential check
    far = len(g["z"]) * nb * nb * N ** 3
    with pytest.raises(gpu.SxsError, match=r"pose 2: negative grid index -7"):
        p.set_poses(np.array([5, 6, -7, far, -1]), skip=1)
    with pytest.raises(gpu.SxsError, match=r"pose 1: translation slot %d >= znum" % len(g["z"])):
        p.set_poses(np.array([5, far, -7, far + 3]), skip=1)
    # the plan is still usable after a rejected list
    p.set_poses(g["index"][:5], skip=1)
    p.run(gpu.FIT_GRID)
    assert np.isfinite(p.results()["chi"]).all()
    p.close()


def test_one_shot_matches_plan_and_counts_launches(gpu):
    g = load(GOLDEN[0])
    L = int(g["L"])
    n0 = gpu.launch_count()
    r = gpu.score_flat(g["A"], g["B"], g["q"], g["z"], L, g["index"], g["a"], float(g["mult"]), float(g["peak"]), 1,
                       gpu.FIT_GRID, g["c1g"], g["c2g"], cross=True)
    assert gpu.launch_count() > n0
    assert chan_err(r["cross"], g["raw"]) <= TOL
    rows = g["grid"].shape[0]
    np.testing.assert_allclose(r["chi"][:rows], np.sqrt(g["grid"].reshape(rows, -1).min(1)), rtol=TOL)
