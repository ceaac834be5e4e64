"""The mixed path's translation fused with the per-pose contraction
(sxsg_plan_set_fused): against the stored-row path on the same plans (the
same sums in another FP32 order), against the FP64 path within the mixed
path's bound, across every column class, with several passes per combo
(dense lists forced onto it) and several chunks, deterministic; the
automatic choice keeps the stored rows."""
import numpy as np
import pytest

from test_gpu_batch import _dimer

pytestmark = pytest.mark.gpu


def _run(p, mode, budget=0):
    import libfmftsaxs_gb300 as g
    p.set_fused(mode)
    if budget:
        p.set_budget(budget)
    p.run(g.FIT_GRID)
    return p.results(cross=True)


def _close(a, b):
    # cross terms: the same FP32 sums in another order, against each
    # (channel, q) column's scale; chi: the fit of those terms
    scale = np.abs(b["cross"]).max(axis=0, keepdims=True)
    assert (np.abs(a["cross"] - b["cross"]) <= 2e-5 * scale).all()
    np.testing.assert_allclose(a["chi"], b["chi"], rtol=2e-5)
    assert np.mean(a["cell"] == b["cell"]) >= 0.999


@pytest.mark.parametrize("L,Q,npose,trange", [(10, 51, 3000, (25.0, 40.0)), (20, 101, 6000, (25.0, 40.0)),
                                              (25, 37, 5000, (25.0, 40.0)), (30, 201, 1200, (25.0, 40.0)),
                                              (31, 12, 4000, (25.0, 40.0)), (12, 24, 20000, (25.0, 26.0))])
def test_fused_matches_stored_rows(gpu, L, Q, npose, trange):
    p = _dimer(gpu, L, Q, 400, 250, npose, trange, seed=31 * L + Q)
    try:
        on = _run(p, gpu.FUSE_ON)
        on2 = _run(p, gpu.FUSE_ON)
        off = _run(p, gpu.FUSE_OFF)
        for k in ("chi", "c1", "c2", "cell", "cross"):
            np.testing.assert_array_equal(on[k], on2[k])
        _close(on, off)
        auto = _run(p, gpu.FUSE_AUTO)   # the stored rows
        for k in ("chi", "cross"):
            np.testing.assert_array_equal(auto[k], off[k])
    finally:
        p.close()


def test_fused_chunks(gpu):
    p = _dimer(gpu, 20, 51, 500, 300, 8000, seed=5)
    try:
        one = _run(p, gpu.FUSE_ON)
        many = _run(p, gpu.FUSE_ON, budget=8 << 20)
        assert p.chunks() > 3
        for k in ("chi", "cross"):
            np.testing.assert_array_equal(one[k], many[k])
    finally:
        p.close()


def test_fused_within_mixed_bound_of_fp64(gpu):
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import synth
    p = _dimer(gpu, 20, 101, 600, 400, 10000, seed=9)
    try:
        mix = _run(p, gpu.FUSE_ON)
        f = g.Plan(p.A, p.B, p.q, p.z, p.L, p.a, p.mult, p.peak, synth.C1_GRID, synth.C2_GRID, precision=g.FP64)
        f.set_poses(p.index, skip=1)
        f.run(g.FIT_GRID)
        ref = f.results()
        f.close()
        d = np.abs(mix["chi"] - ref["chi"]) / ref["chi"]
        assert d.max() <= 1e-4
        top = lambda c: set(np.argsort(c, kind="stable")[:100])
        assert len(top(mix["chi"]) & top(ref["chi"])) >= 99
    finally:
        p.close()


def test_fused_rejected_where_unavailable(gpu):
    from libfmftsaxs_gb300 import SxsError, synth
    p = _dimer(gpu, 10, 51, 200, 100, 500, seed=3)
    try:
        f = gpu.Plan(p.A, p.B, p.q, p.z, p.L, p.a, 1.0, 1.0, synth.C1_GRID, synth.C2_GRID, precision=gpu.FP64)
        with pytest.raises(SxsError, match="mixed-precision"):
            f.set_fused(gpu.FUSE_ON)
        f.close()
    finally:
        p.close()
