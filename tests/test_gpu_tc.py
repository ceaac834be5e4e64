"""The tcgen05 tensor-core rotation (3xTF32, FP32 accumulation) against the
CUDA-core FP32 rotation on the same mixed plans: raw cross terms within
1e-5 of each channel's scale and chi within 1e-5 relative, on the
reference fixtures and on L from 3 to 30."""
import glob
import os

import numpy as np
import pytest

from test_gpu_parity import _random_case, chan_err, load

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dimer_*.npz")))


def _both(gpu, A, B, q, z, L, a, mult, peak, idx, skip=1):
    from libfmftsaxs_gb300 import synth
    out = []
    for eng in (gpu.ROT_CUDA, gpu.ROT_TC):
        p = gpu.Plan(A, B, q, z, L, a, mult, peak, synth.C1_GRID, synth.C2_GRID, precision=gpu.MIXED)
        p.set_rotation(eng)
        p.set_poses(idx, skip=skip)
        p.run(gpu.FIT_GRID)
        out.append(p.results(cross=True))
        p.close()
    return out


def _check(cu, tc):
    assert chan_err(tc["cross"], cu["cross"]) <= 1e-5
    assert np.max(np.abs(tc["chi"] - cu["chi"]) / cu["chi"]) <= 1e-5


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_tc_rotation_matches_cuda_cores_fixture(gpu, path):
    g = load(path)
    cu, tc = _both(gpu, g["A"], g["B"], g["q"], g["z"], int(g["L"]), g["a"], float(g["mult"]), float(g["peak"]),
                   g["index"], int(g["skip"]))
    _check(cu, tc)


@pytest.mark.parametrize("L,Q", [(3, 9), (10, 16), (20, 24), (30, 12)])
def test_tc_rotation_matches_cuda_cores_random(gpu, oracle, L, Q):
    c = _random_case(oracle, L, Q, 80, 50, 200, seed=L * 13 + Q)
    cu, tc = _both(gpu, c["A"], c["B"], c["q"], c["z"], L, c["a"], c["mult"], c["peak"], c["index"])
    _check(cu, tc)
