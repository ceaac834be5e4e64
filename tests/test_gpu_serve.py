"""The serving loop (sxsg_server_*): jobs of different sizes and precisions
submitted together give bitwise the results of each job run alone; the
rotation-table cache is hit by a repeated molecule key without changing
results; a cap too small for two jobs serialises them without deadlock; a
failing job reports its error and the server keeps serving."""
import glob
import os

import numpy as np
import pytest

from test_gpu_parity import _random_case, load

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _jobs(oracle):
    from libfmftsaxs_gb300 import synth
    jobs = []
    for path in GOLDEN:
        g = load(path)
        for prec in (0, 1):
            jobs.append(dict(A=g["A"], B=g["B"], qvals=g["q"], zvals=g["z"], L=int(g["L"]), a=g["a"],
                             mult=float(g["mult"]), peak=float(g["peak"]), index=g["index"], c1grid=g["c1g"],
                             c2grid=g["c2g"], skip=int(g["skip"]), precision=prec))
    for L, Q in ((4, 9), (9, 12), (15, 8)):
        c = _random_case(oracle, L, Q, 60, 40, 300, seed=L * 31 + Q)
        jobs.append(dict(A=c["A"], B=c["B"], qvals=c["q"], zvals=c["z"], L=L, a=c["a"], mult=c["mult"],
                         peak=c["peak"], index=c["index"], c1grid=synth.C1_GRID, c2grid=synth.C2_GRID, skip=1,
                         precision=1))
    return jobs


def _alone(gpu, j):
    p = gpu.Plan(j["A"], j["B"], j["qvals"], j["zvals"], j["L"], j["a"], j["mult"], j["peak"], j["c1grid"],
                 j["c2grid"], precision=j["precision"])
    p.set_poses(j["index"], skip=j["skip"])
    p.run(gpu.FIT_GRID)
    r = p.results()
    p.close()
    return r


def test_results_are_the_same_alone_and_in_the_mix(gpu, oracle):
    jobs = _jobs(oracle)
    alone = [_alone(gpu, j) for j in jobs]
    srv = gpu.Server(max_active=3)
    tickets = [srv.submit(**j) for j in jobs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["done"] == len(jobs)
    for a, m in zip(alone, mixed):
        for k in ("chi", "c1", "c2"):
            np.testing.assert_array_equal(m[k], a[k])
        assert m["latency_ms"] >= m["run_ms"] > 0


def test_table_cache_hits_keep_results(gpu, oracle):
    g = load(GOLDEN[-1])
    base = dict(A=g["A"], B=g["B"], qvals=g["q"], zvals=g["z"], L=int(g["L"]), a=g["a"], mult=float(g["mult"]),
                peak=float(g["peak"]), c1grid=g["c1g"], c2grid=g["c2g"], skip=1, precision=1, keyA=11, keyB=12)
    idx = g["index"]
    srv = gpu.Server(max_active=1)
    r1 = srv.wait(srv.submit(index=idx, **base))
    r2 = srv.wait(srv.submit(index=idx[::2], **base))
    st = srv.stats()
    srv.close()
    assert st["cache_hits"] >= 2 and st["cache_entries"] == 2
    np.testing.assert_array_equal(r2["chi"], r1["chi"][::2])
    np.testing.assert_array_equal(r1["chi"], _alone(gpu, dict(base, index=idx))["chi"])


def test_small_cap_serialises_jobs(gpu, oracle):
    jobs = _jobs(oracle)[:4]
    alone = [_alone(gpu, j) for j in jobs]
    srv = gpu.Server(hbm_cap=1 << 20, max_active=4)
    out = [srv.wait(t) for t in [srv.submit(**j) for j in jobs]]
    srv.close()
    for a, m in zip(alone, out):
        np.testing.assert_array_equal(m["chi"], a["chi"])


def test_failing_job_is_isolated(gpu, oracle):
    jobs = _jobs(oracle)
    bad = dict(jobs[0])
    L = bad["L"]
    N, nb = 2 * L + 1, L + 1
    bad["index"] = np.array([len(bad["zvals"]) * nb * nb * N ** 3 + 5], dtype=np.int64)   # z slot out of range
    srv = gpu.Server(max_active=2)
    tb = srv.submit(**bad)
    tg = srv.submit(**jobs[1])
    with pytest.raises(gpu.SxsError, match="znum"):
        srv.wait(tb)
    good = srv.wait(tg)
    srv.close()
    np.testing.assert_array_equal(good["chi"], _alone(gpu, jobs[1])["chi"])
