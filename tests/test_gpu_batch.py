"""Batches of dimers (sxsg_batch_*): one CUDA graph over many
mixed-precision plans of different L, q grids and pose counts (sparse and
dense lists; stored translated rows, and the fused translation on every
third plan) gives every plan bit
for bit the results of its own sxsg_plan_run, in every launch form
(persistent or one block per item, one arena or two halves), with one phase
or many (a small arena), on every replay, with or without the fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (L, Q, receptor atoms, ligand atoms, poses[, |t| range]): every translation
# column class (L + 1 up to 32), q tiles with and without padding, pose
# counts from a few blocks to many chunks; sparse lists and two dense ones
# (|t| within 2 A: tens of poses per translated row)
SPECS = [(4, 9, 120, 80, 300), (10, 51, 400, 250, 3000), (15, 101, 600, 300, 8000), (20, 51, 500, 300, 2500),
         (20, 101, 900, 500, 20000), (25, 37, 700, 400, 6000), (30, 201, 800, 450, 1500), (31, 12, 300, 200, 4000),
         (10, 201, 300, 200, 500), (12, 24, 300, 200, 20000, (25.0, 26.0)), (20, 51, 400, 300, 30000, (30.0, 31.5))]


def _dimer(g, L, Q, nrec, nlig, npose, trange=(25.0, 40.0), seed=0):
    from libfmftsaxs_gb300 import synth, workload as wl
    rng = np.random.default_rng(seed)
    rec = synth.make_molecule(nrec, 2.2 * (nrec / 8.0) ** 0.38, seed).with_sasa()
    lig = synth.make_molecule(nlig, 2.2 * (nlig / 8.0) ** 0.38, seed + 1).with_sasa()
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    q = g.mkarray(0.0, 0.5, Q)
    A = g.expand(rec.xyz, *wl.form_factors(g, rec), rec.sasa, g.ff_water(), q, L)
    B = g.expand(lig.xyz, *wl.form_factors(g, lig), lig.sasa, g.ff_water(), q, L)
    c1, c2 = rng.uniform(0.97, 1.03), rng.uniform(0.0, 3.0)
    I, _ = g.profile_from_spf(A, L, q, 1.7, c1, c2)
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = g.bin_experiment(eq, ei, ee, q, 1.7)
    z = np.arange(np.floor(trange[0]), np.ceil(trange[1]) + 1.0)
    R = synth.random_rotations(npose, rng)
    T = synth.random_translations(npose, trange[0], trange[1], rng)
    idx, _ = g.poses_to_indices(R, T, z, L)
    p = g.Plan(A, B, q, z, L, a, mult, peak, synth.C1_GRID, synth.C2_GRID, precision=g.MIXED)
    p.set_poses(idx, skip=1)
    return p


@pytest.fixture(scope="module")
def plans(gpu):
    ps = [_dimer(gpu, *s, seed=700 + 13 * i) for i, s in enumerate(SPECS)]
    for p in ps[1::3]:
        p.set_fused(gpu.FUSE_ON)   # some dimers on the fused translation
    yield ps
    for p in ps:
        p.close()


def _alone(plans, fit, cross=True):
    out = []
    for p in plans:
        p.run(fit)
        out.append(p.results(cross=cross))
    return out


def _batched(gpu, plans, fit, arena=0, reps=1, cross=True, flags=None):
    b = gpu.Batch(plans, fit=fit, arena_bytes=arena, flags=flags)
    runs = []
    for _ in range(reps):
        b.run()
        runs.append([p.results(cross=cross) for p in plans])
    st = b.stats()
    b.close()
    return runs, st


def _same(x, y):
    for k in x:
        np.testing.assert_array_equal(x[k], y[k], err_msg=k)


@pytest.mark.parametrize("flags", [0, 1, 2, 3, 5, 7])
def test_batch_equals_plan_runs(gpu, plans, flags):
    runs, st = _batched(gpu, plans, gpu.FIT_GRID, reps=2, flags=flags)
    alone = _alone(plans, gpu.FIT_GRID)
    assert st["plans"] == len(plans) and st["poses"] == sum(p.n for p in plans)
    assert st["total_ms"] > 0 and st["launches"] > 0
    for r in runs:
        for a, b in zip(alone, r):
            _same(a, b)
    assert all(np.isfinite(a["chi"]).all() for a in alone)


@pytest.mark.parametrize("flags", [1, 3, 5])
def test_batch_many_phases(gpu, plans, flags):
    # an arena of 96 MB holds a few slices of the largest tables (40 MB per
    # slice at L = 30, Q = 201): many chunks and phases
    runs, st = _batched(gpu, plans, gpu.FIT_GRID, arena=96 << 20, flags=flags)
    assert st["phases"] > 4 and st["arena_bytes"] <= 96 << 20
    alone = _alone(plans, gpu.FIT_GRID)
    for a, b in zip(alone, runs[0]):
        _same(a, b)


def test_batch_without_fit(gpu, plans):
    sub = plans[1:5]
    runs, st = _batched(gpu, sub, gpu.FIT_NONE)
    alone = _alone(sub, gpu.FIT_NONE)
    for a, b in zip(alone, runs[0]):
        np.testing.assert_array_equal(a["cross"], b["cross"])


def test_topk_after_batch(gpu, plans):
    sub = plans[2:4]
    b = gpu.Batch(sub, fit=gpu.FIT_GRID)
    b.run()
    for p in sub:
        r = p.results()
        t = p.topk(50)
        order = np.argsort(r["chi"], kind="stable")[:50]
        np.testing.assert_array_equal(t["pose"], order)
        np.testing.assert_array_equal(t["chi"], r["chi"][order])
    b.close()


def test_batch_rejects_bad_plans(gpu, plans):
    from libfmftsaxs_gb300 import SxsError, synth
    with pytest.raises(SxsError, match="listed twice"):
        gpu.Batch([plans[0], plans[0]])
    p = plans[0]
    f = gpu.Plan(p.A, p.B, p.q, p.z, p.L, p.a, 1.0, 1.0, synth.C1_GRID, synth.C2_GRID, precision=gpu.FP64)
    try:
        with pytest.raises(SxsError, match="not mixed precision"):
            gpu.Batch([plans[1], f])
    finally:
        f.close()
    g = gpu.Plan(p.A, p.B, p.q, p.z, p.L, p.a, 1.0, 1.0, precision=gpu.MIXED)
    try:
        with pytest.raises(SxsError, match="grid"):
            gpu.Batch([g], fit=gpu.FIT_GRID)
    finally:
        g.close()
