"""The double-float grid fit of the mixed path (libfmftsaxs_gb300/csrc/
fitdf_core.h, the arithmetic the GPU runs on its FP32 pipe) compiled for the
host without contraction and checked against the reference's own chi^2 grids
(golden fixtures): the best chi within 1e-9 relative and a best cell whose
reference score is within 1e-9 of the reference's best.  The mixed path's
bound is 1e-4; double-float arithmetic carries ~2^-48, so the fit itself
adds nothing measurable to the error of the FP32 contractions."""
import ctypes as C
import glob
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "dimer_*.npz")))
DP = C.POINTER(C.c_double)

# host restatement of the kernel's staging (normalised model, constants
# scaled by peak and peak^2) around the shared double-float core
SRC = r'''
#include <stdlib.h>
#include "fitdf_core.h"
void fit(const double *cross, int npose, int Q, const double *q, const double *a, double mult, double peak,
         const double *c1g, int n1, const double *c2g, int n2, double *chi, int *cell)
{
	dfl *fs = malloc(sizeof(dfl) * 5 * Q), *c = malloc(sizeof(dfl) * 8 * Q), *G = malloc(sizeof(dfl) * n1 * Q);
	dfl *c2s = malloc(sizeof(dfl) * n2);
	double a0 = 0;
	for (int i = 0; i < Q; i++) {
		double qi = q[i], h = 1.0 / (qi - (i > 0 ? q[i - 1] : -1.0));
		const double *ai = a + 6 * i;
		double f[5] = {ai[3], (ai[4] - qi * ai[3]) * h, ((ai[5] - 2.0 * qi * ai[4]) + qi * qi * ai[3]) * (h * h),
		               ai[1], (ai[2] - qi * ai[1]) * h};
		for (int k = 0; k < 5; k++) fs[k * Q + i] = df_from(f[k] * (k < 3 ? peak * peak : peak));
		a0 += ai[0];
	}
	for (int j = 0; j < n1; j++) {
		double c1 = c1g[j], corr = -mult * (c1 * c1 - 1.0), c1c = c1 * c1 * c1;
		for (int i = 0; i < Q; i++) {
			double g = c1c * exp(corr * q[i] * q[i]);
			float hi = (float)g;
			G[j * Q + i] = df_mk(hi, (float)(g - (double)hi));
		}
	}
	for (int k = 0; k < n2; k++) c2s[k] = df_from(c2g[k]);
	for (int p = 0; p < npose; p++) {
		const double *x = cross + (size_t)p * 6 * Q;
		double sc = x[0] + x[3 * Q] + x[5 * Q] + x[2 * Q] - x[Q] - x[4 * Q];
		double inv = 1.0 / sc;
		for (int r = 0; r < 6 * Q; r++) c[r] = df_from(x[r] * inv);
		dfl U2, D4;
		df_pose_prep(c, fs, Q, 0, 1, &U2, &D4);
		U2 = df_from(df_to(U2));
		D4 = df_from(df_to(D4));
		double best = 1.0 / 0.0;
		int bc = -1;
		for (int j = 0; j < n1; j++) {
			dfl u[2], d[4], bu, bd;
			df_row(c, fs, G + (size_t)j * Q, Q, u, d);
			int bi = df_best_c2(u, U2, d, D4, c2s, n2, &bu, &bd);
			if (bi < 0) continue;
			double uu = df_to(bu), dd = df_to(bd), k = uu / dd;
			double s = a0 + k * (-2.0 * uu + k * dd);
			if (s < best) { best = s; bc = j * n2 + bi; }
		}
		chi[p] = sqrt(best);
		cell[p] = bc;
	}
	free(fs); free(c); free(G); free(c2s);
}
'''


@pytest.fixture(scope="module")
def dffit(tmp_path_factory):
    d = tmp_path_factory.mktemp("df")
    src = d / "fit.c"
    src.write_text(SRC)
    so = d / "libdffit.so"
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                           "-I", os.path.join(ROOT, "libfmftsaxs_gb300", "csrc"), str(src), "-o", str(so), "-lm"])
    lib = C.CDLL(str(so))

    def run(g):
        cross = np.ascontiguousarray(g["raw"], dtype=np.float64)
        n, Q = len(cross), len(g["q"])
        chi, cell = np.zeros(n), np.zeros(n, dtype=np.int32)
        lib.fit(cross.ctypes.data_as(DP), C.c_int(n), C.c_int(Q), g["q"].ctypes.data_as(DP),
                np.ascontiguousarray(g["a"]).ctypes.data_as(DP), C.c_double(float(g["mult"])),
                C.c_double(float(g["peak"])), g["c1g"].ctypes.data_as(DP), C.c_int(len(g["c1g"])),
                g["c2g"].ctypes.data_as(DP), C.c_int(len(g["c2g"])), chi.ctypes.data_as(DP),
                cell.ctypes.data_as(C.POINTER(C.c_int)))
        return chi, cell
    return run


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_double_float_fit_matches_reference_grid(dffit, path):
    g = dict(np.load(path))
    chi, cell = dffit(g)
    rows = g["grid"].shape[0]
    grid = g["grid"].reshape(rows, -1)
    best = grid.min(axis=1)
    np.testing.assert_allclose(chi[:rows], np.sqrt(best), rtol=1e-9, atol=0)
    chosen = grid[np.arange(rows), cell[:rows]]
    assert np.all(chosen <= best * (1 + 1e-9))
