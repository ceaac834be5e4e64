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

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dimer_*.npz")))


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


def _same_molecule_base(g, keyA, keyB, precision):
    return dict(A=g["A"], B=g["B"], qvals=g["q"], zvals=g["z"], L=int(g["L"]), a=g["a"], mult=float(g["mult"]),
                peak=float(g["peak"]), c1grid=g["c1g"], c2grid=g["c2g"], skip=1, precision=precision, keyA=keyA,
                keyB=keyB)


def test_same_molecule_jobs_at_once_match_alone(gpu, oracle):
    """Jobs with the same receptor and ligand submitted together, three on
    the device at once: the first fills the shared tables while the others,
    finding them still being filled, fill private copies; jobs admitted
    later read the completed tables.  Every result is bitwise the job run
    alone, over repeated rounds and both precisions."""
    g = load(GOLDEN[-1])
    idx = g["index"]
    subsets = [idx, idx[::2], idx[1::3], idx[::-1].copy(), idx[5:], idx[:40]]
    jobs = [dict(_same_molecule_base(g, 21, 22, prec), index=s) for prec in (1, 0) for s in subsets]
    alone = [_alone(gpu, j)["chi"] for j in jobs]
    srv = gpu.Server(max_active=3)
    for _ in range(3):
        tickets = [srv.submit(**j) for j in jobs]
        for t, a in zip(tickets, alone):
            np.testing.assert_array_equal(srv.wait(t)["chi"], a)
    st = srv.stats()
    srv.close()
    # two tables per precision are shared; later rounds hit them
    assert st["cache_entries"] == 4
    assert st["cache_hits"] >= 2 * len(jobs)


def test_reused_key_with_other_coefficients_does_not_alias(gpu, oracle):
    """A caller key reused for a different molecule (same L and q grid)
    gets that molecule's own tables: the cache key covers the coefficients."""
    g = load(GOLDEN[-1])
    base = _same_molecule_base(g, 41, 42, 1)
    other = dict(base, A=g["A"] * 0.75, B=g["B"][::-1].copy())
    j1, j2 = dict(base, index=g["index"]), dict(other, index=g["index"])
    a1, a2 = _alone(gpu, j1)["chi"], _alone(gpu, j2)["chi"]
    assert not np.array_equal(a1, a2)
    srv = gpu.Server(max_active=2)
    r1 = srv.wait(srv.submit(**j1))
    r2 = srv.wait(srv.submit(**j2))
    t = [srv.submit(**j) for j in (j1, j2, j2, j1)]
    rr = [srv.wait(x)["chi"] for x in t]
    st = srv.stats()
    srv.close()
    np.testing.assert_array_equal(r1["chi"], a1)
    np.testing.assert_array_equal(r2["chi"], a2)
    for got, want in zip(rr, (a1, a2, a2, a1)):
        np.testing.assert_array_equal(got, want)
    assert st["cache_entries"] == 4
