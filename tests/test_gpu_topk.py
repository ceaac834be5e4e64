"""Device top-k (sxsg_plan_topk): the k best poses of a fitted run in the
order of a stable argsort of the run's chi (ascending, ties in list order),
on the benchmark-shape fixtures (c0_shape: 1,354 poses, c1_shape: 400) in
both precisions, with pose lists that repeat poses (exact ties), after an
L-BFGS-B fit, and at the largest k."""
import numpy as np
import pytest

from test_gpu_shapes import expand_pair, load_shape

pytestmark = pytest.mark.gpu


def _plan(gpu, g, A, B, precision, index):
    p = gpu.Plan(A, B, g["q"], g["z"], int(g["L"]), g["a"], float(g["mult"]), float(g["peak"]), g["c1g"], g["c2g"],
                 precision=precision)
    p.set_poses(index, skip=1)
    return p


def _check(p, k):
    r = p.results()
    t = p.topk(k)
    want = np.argsort(r["chi"], kind="stable")[:min(k, len(r["chi"]))]
    np.testing.assert_array_equal(t["pose"], want)
    np.testing.assert_array_equal(t["chi"], r["chi"][want])
    np.testing.assert_array_equal(t["c1"], r["c1"][want])
    np.testing.assert_array_equal(t["c2"], r["c2"][want])


@pytest.mark.parametrize("name", ["c0_shape", "c1_shape"])
def test_topk_is_stable_argsort_of_chi(gpu, name):
    g = load_shape(name)
    A, B = expand_pair(gpu, g)
    for prec in (gpu.FP64, gpu.MIXED):
        p = _plan(gpu, g, A, B, prec, g["index"])
        p.run(gpu.FIT_GRID)
        for k in (1, 7, 100, 1000, len(g["index"]), len(g["index"]) + 5):
            _check(p, k)
        p.close()


def test_topk_with_repeated_poses_keeps_list_order(gpu):
    g = load_shape("c1_shape")
    A, B = expand_pair(gpu, g)
    rng = np.random.default_rng(5)
    idx = np.concatenate([g["index"], g["index"][::-1], g["index"][rng.permutation(len(g["index"]))]])
    p = _plan(gpu, g, A, B, gpu.MIXED, idx)
    p.run(gpu.FIT_GRID)
    for k in (3, 64, 333, 1200):
        _check(p, k)
    p.run(gpu.FIT_LBFGSB)
    _check(p, 500)
    p.close()


def test_topk_needs_a_fitted_run(gpu):
    g = load_shape("c1_shape")
    A, B = expand_pair(gpu, g)
    p = _plan(gpu, g, A, B, gpu.MIXED, g["index"])
    with pytest.raises(gpu.SxsError, match="fitted"):
        p.topk(10)
    p.run(gpu.FIT_NONE)
    with pytest.raises(gpu.SxsError, match="fitted"):
        p.topk(10)
    p.close()


def test_topk_at_its_largest_k(gpu):
    """20,000 poses (the C1 fixture's list 50 times): k = 16,384, the
    largest, matches the stable argsort; one more is refused."""
    g = load_shape("c1_shape")
    A, B = expand_pair(gpu, g)
    p = _plan(gpu, g, A, B, gpu.MIXED, np.tile(g["index"], 50))
    p.run(gpu.FIT_GRID)
    _check(p, 16384)
    with pytest.raises(gpu.SxsError, match="16384"):
        p.topk(16385)
    p.close()
