"""The large-expansion configuration (L = 30, q on [0, 0.6]): the widest
kernels (31 x 31 translation blocks) against the oracle at Q = 9 (the
oracle's cost per (z, beta1, beta2) triple grows with Q; L drives the
kernels' shapes), and the mixed path against the FP64 path at Q = 201 (26 q
tiles) on 3,000 poses.  Beyond L = 31 the translation runs the slice kernel
and the rotation 12 gamma pairs per thread: L = 34 against the oracle at
Q = 5, L = 40 mixed against FP64."""
import numpy as np
import pytest

from test_gpu_mixed import CHI_TOL, CROSS_TOL, check_grid
from test_gpu_parity import TOL, chan_err

pytestmark = pytest.mark.gpu


def _make(oracle, Q, npose, L=30):
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import synth
    rec = synth.make_molecule(400, 14.0, 31).with_sasa()
    lig = synth.make_molecule(300, 12.0, 32).with_sasa()
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    q = oracle.mkarray(0.0, 0.6, Q)
    ffr = np.array([g.ff_type(e) for e in rec.elements])
    ffl = np.array([g.ff_type(e) for e in lig.elements])
    A = oracle.expand(rec.xyz, ffr[:, 0], ffr[:, 1], rec.sasa, g.ff_water(), q, L)
    B = oracle.expand(lig.xyz, ffl[:, 0], ffl[:, 1], lig.sasa, g.ff_water(), q, L)
    rng = np.random.default_rng(7)
    I = np.exp(-np.arange(Q) * 0.05) * 1e6
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = oracle.opt_params(eq, ei, ee, q, 1.7)
    z = np.arange(40.0, 46.0)
    R = synth.random_rotations(npose, rng)
    T = synth.random_translations(npose, 40.0, 45.0, rng)
    idx, _ = g.poses_to_indices(R, T, z, L)
    return dict(A=A, B=B, q=q, z=z, L=L, a=a, mult=mult, peak=peak, index=idx)


@pytest.fixture(scope="module")
def case(oracle):
    return _make(oracle, 201, 3000)


def _run(gpu, c, idx, prec):
    from libfmftsaxs_gb300 import synth
    p = gpu.Plan(c["A"], c["B"], c["q"], c["z"], c["L"], c["a"], c["mult"], c["peak"], synth.C1_GRID, synth.C2_GRID,
                 precision=prec)
    p.set_poses(idx, skip=1)
    p.run(gpu.FIT_GRID)
    r = p.results(cross=True, grid=True)
    p.close()
    return r


@pytest.mark.parametrize("L,Q", [(30, 9), (34, 5)])
def test_large_l_fp64_matches_oracle(gpu, oracle, L, Q):
    from libfmftsaxs_gb300 import synth
    from libfmftsaxs_gb300.workload import decode
    c = _make(oracle, Q, 400, L=L)
    z, b1, b2 = decode(c["index"], c["L"])[:3]
    key = (z * (L + 1) + b1) * (L + 1) + b2
    idx = c["index"][key == key[0]][:4].astype(np.int32)   # poses of one triple
    raw, scl, grid, br = oracle.score(c["A"], c["B"], c["q"], c["z"], c["L"], idx, 1, c["peak"], c["a"], c["mult"],
                                      synth.C1_GRID, synth.C2_GRID)
    r = _run(gpu, c, idx, gpu.FP64)
    assert chan_err(r["cross"], raw) <= TOL
    np.testing.assert_allclose(r["grid"], grid, rtol=TOL, atol=0)


def test_lmax30_mixed_matches_fp64(gpu, case):
    ref = _run(gpu, case, case["index"], gpu.FP64)
    mix = _run(gpu, case, case["index"], gpu.MIXED)
    assert chan_err(mix["cross"], ref["cross"]) <= CROSS_TOL
    check_grid(mix, ref["grid"])
    assert np.max(np.abs(mix["chi"] - ref["chi"]) / ref["chi"]) <= CHI_TOL


def test_lmax40_mixed_matches_fp64(gpu, oracle):
    c = _make(oracle, 51, 1000, L=40)
    ref = _run(gpu, c, c["index"], gpu.FP64)
    mix = _run(gpu, c, c["index"], gpu.MIXED)
    assert chan_err(mix["cross"], ref["cross"]) <= CROSS_TOL
    check_grid(mix, ref["grid"])
    assert np.max(np.abs(mix["chi"] - ref["chi"]) / ref["chi"]) <= CHI_TOL
