"""The L-BFGS-B restatement (libfmftsaxs_gb300/csrc/lbfgsb_core.h, the
solver the GPU runs one thread per pose) compiled for the host and checked
against the reference's own fit: bit-exact on every fixture pose and on
fits with interior optima."""
import ctypes as C
import glob
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dimer_*.npz")))
DP = C.POINTER(C.c_double)

SRC = r'''
#include "lbfgsb_core.h"
int fit(const double *cross, const double *q, const double *a, double mult, int Q, double *out)
{
	lb_saxs o = {cross, 1, q, a, mult, Q};
	double chi, c1, c2, sc;
	int ne = lb_saxs_fit(&o, &chi, &c1, &c2, &sc, 100000);
	out[0] = chi; out[1] = c1; out[2] = c2; out[3] = sc;
	return ne;
}
'''


@pytest.fixture(scope="module")
def solver(tmp_path_factory):
    d = tmp_path_factory.mktemp("lb")
    src = d / "fit.c"
    src.write_text(SRC)
    so = d / "libfit.so"
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                           "-I", os.path.join(ROOT, "libfmftsaxs_gb300", "csrc"), str(src), "-o", str(so), "-lm"])
    lib = C.CDLL(str(so))
    lib.fit.argtypes = [DP, DP, DP, C.c_double, C.c_int, DP]

    def run(cross, q, a, mult):
        cross, q, a = (np.ascontiguousarray(x, dtype=np.float64) for x in (cross, q, a))
        out = np.zeros(4)
        ne = lib.fit(cross.ctypes.data_as(DP), q.ctypes.data_as(DP), a.ctypes.data_as(DP), mult, len(q),
                     out.ctypes.data_as(DP))
        return out, ne
    return run


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_fit_bit_exact_vs_reference_fixtures(solver, path):
    g = dict(np.load(path))
    for i in range(len(g["index"])):
        out, ne = solver(g["scaled"][i].reshape(-1), g["q"], g["a"], float(g["mult"]))
        assert (out[0], out[1], out[2]) == (g["chi"][i], g["c1"][i], g["c2"][i]), i
        assert 1 <= ne < 1000


def test_fit_bit_exact_vs_reference_interior_optima(solver, oracle, ref):
    g = dict(np.load(GOLDEN[0]))
    q = g["q"]
    rng = np.random.default_rng(7)
    for _ in range(120):
        raw = g["raw"][rng.integers(len(g["index"]))].reshape(-1)
        I, _ = oracle.compile_intensity(raw, q, float(g["rm"]), rng.uniform(0.965, 1.035), rng.uniform(-1.5, 3.5))
        ei = I * (1 + rng.uniform(0, 0.03) * rng.normal(size=len(q)))
        ee = 0.01 * np.abs(I) + 1e-12
        scaled, chi, c1, c2, sc, _ = ref.fit_cross(raw, q, ei, ee, q, float(g["rm"]))
        a, mult, _ = oracle.opt_params(q, ei, ee, q, float(g["rm"]))
        out, _ = solver(scaled.reshape(-1), q, a, mult)
        assert (out[0], out[1], out[2], out[3]) == (chi, c1, c2, sc)
