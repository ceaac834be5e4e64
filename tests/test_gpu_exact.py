"""Exact per-pose scoring (sxsg_score_exact, the reference's score_ft_naive
flow) against an independent restatement: the moves and the centring in
Python scalar arithmetic (same operation order), the oracle's expansion
and single-molecule cross terms (bit-exact with the reference's code), and
the restated L-BFGS-B (tests/test_lbfgsb_host.py: bit-exact with the
reference's fit) run on the host.  Tolerances as for the drop-in fit:
cross terms 1e-10 of each channel's scale, chi 1e-8 relative, (c1, c2)
1e-6."""
import ctypes as C
import math
import os
import subprocess

import numpy as np
import pytest

from test_gpu_parity import chan_err
from test_lbfgsb_host import SRC as LB_SRC

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DP = C.POINTER(C.c_double)


def active(a, b, g):
    """sxs_fill_active_rotation_matrix (src/saxs_utils.c), row-major m11..m33"""
    ca, sa, cb, sb, cg, sg = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(g), math.sin(g)
    return [cg * cb * ca - sg * sa, -sg * cb * ca - cg * sa, sb * ca,
            cg * cb * sa + sg * ca, -sg * cb * sa + cg * ca, sb * sa,
            -cg * sb, sg * sb, cb]


def pose_coords(rec, lig, eu):
    z, b1, g1, a2, b2, g2 = (float(x) for x in eu)
    out = []
    for xyz, m, tz in ((rec, active(0.0, b1, g1), 0.0), (lig, active(a2, b2, g2), z)):
        for x, y, w in xyz.tolist():
            out.append([m[0] * x + m[1] * y + m[2] * w + 0.0, m[3] * x + m[4] * y + m[5] * w + 0.0,
                        m[6] * x + m[7] * y + m[8] * w + tz])
    n = len(out)
    c = [0.0, 0.0, 0.0]
    for p in out:
        for k in range(3):
            c[k] += p[k]
    c = [-(v / n) for v in c]
    return np.array([[p[0] + c[0], p[1] + c[1], p[2] + c[2]] for p in out])


@pytest.fixture(scope="module")
def host_fit(tmp_path_factory):
    d = tmp_path_factory.mktemp("lbx")
    (d / "fit.c").write_text(LB_SRC)
    so = d / "libfit.so"
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                           "-I", os.path.join(ROOT, "libfmftsaxs_gb300", "csrc"), str(d / "fit.c"), "-o", str(so), "-lm"])
    lib = C.CDLL(str(so))
    lib.fit.argtypes = [DP, DP, DP, C.c_double, C.c_int, DP]

    def run(cross, q, a, mult):
        cross, q, a = (np.ascontiguousarray(x, dtype=np.float64) for x in (cross, q, a))
        out = np.zeros(4)
        lib.fit(cross.ctypes.data_as(DP), q.ctypes.data_as(DP), a.ctypes.data_as(DP), mult, len(q),
                out.ctypes.data_as(DP))
        return out
    return run


def test_exact_scoring_matches_restatement(gpu, oracle, host_fit):
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(21)
    L, Q = 6, 12
    rec = synth.make_molecule(70, 8.0, 41).with_sasa()
    lig = synth.make_molecule(45, 7.0, 42).with_sasa()
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    ffr = np.array([gpu.ff_type(e) for e in rec.elements])
    ffl = np.array([gpu.ff_type(e) for e in lig.elements])
    vac = np.concatenate([ffr[:, 0], ffl[:, 0]])
    dum = np.concatenate([ffr[:, 1], ffl[:, 1]])
    sasa = np.concatenate([rec.sasa, lig.sasa])
    h2o = gpu.ff_water()
    water_w = np.array([h2o * s for s in sasa.tolist()])
    q = oracle.mkarray(0.0, 0.5, Q)
    I = np.exp(-np.arange(Q) * 0.2) * 1e5
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = oracle.opt_params(eq, ei, ee, q, 1.7)
    n = 9
    eu = np.column_stack([rng.uniform(14, 20, n), rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n),
                          rng.uniform(0, 2 * np.pi, n), rng.uniform(0, np.pi, n), rng.uniform(0, 2 * np.pi, n)])
    got = gpu.score_exact(rec.xyz, lig.xyz, vac, dum, water_w, eu, q, L, a, mult, cross=True)
    for i in range(n):
        xyz = pose_coords(rec.xyz, lig.xyz, eu[i])
        spf = oracle.expand(xyz, vac, dum, sasa, h2o, q, L)
        cr = oracle.spf2cross_terms(spf, L, Q).reshape(6, Q)
        assert chan_err(got["cross"][i], cr) <= 1e-10
        chi, c1, c2, _ = host_fit(cr, q, a, mult)
        assert abs(got["chi"][i] - chi) <= 1e-8 * chi
        assert abs(got["c1"][i] - c1) <= 1e-6 and abs(got["c2"][i] - c2) <= 1e-6
