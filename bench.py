"""Benchmark of the FFT-correlation dimer scoring path on one GB300.

Workload (default c1): receptor 3,500 atoms (Rg 21 A) and ligand 2,000 atoms
(Rg 17 A), L = 20, 101 q on [0, 0.5], 210,000 seeded poses (three lists of
70,000, |t| in [30, 50] A), grid fit over c1 in [0.95, 1.05] x c2 in [0, 4].
A step scores the whole pose list: rotation and translation tables, per-pose
cross terms, chi^2 over the fit grid.

  value   poses/s with inputs resident on the device (CUDA events on the
          library's stream, K steps back to back)
  e2e     poses/s through the one-shot C-ABI call from host buffers
          (host->device inputs and device->host chi/c1/c2 inside the timing)
  cpu_baseline  the CPU oracle on a bounded sample of the same workload,
          one process per host core

`--impl reference` times the reference algorithm on the host cores instead
(the reference's own code compiled here when present, else the C oracle).
"""
import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


# ---------------------------------------------------------------- CPU side
def _cpu_worker(args):
    """Three calls of a CPU implementation on one z slice: no pose (the
    per-call setup), the poses of the first triple, the poses of all the
    worker's triples (per-z setup shared, as in a full run).  Returns
    (poses of the last call, [seconds of the three calls])."""
    kind, A, B, q, z, L, idx1, idx, a, mult, peak, c1g, c2g, exp, rms = args
    from oracle import bind
    if kind == "reference":
        r = bind.Ref()

        def call(ix):
            r.score(A, B, rms[0], rms[1], rms[2], exp, q, z, L, ix, 1, c1g, c2g)
    else:
        o = bind.Oracle()

        def call(ix):
            o.score(A, B, q, z, L, ix, 1, peak, a, mult, c1g, c2g)
    times = []
    for ix in (idx[:0], idx1, idx):
        t = time.perf_counter()
        call(ix)
        times.append(time.perf_counter() - t)
    return len(idx), times


def cpu_sample(w, kind, workers, triples_per_worker=4, seed=11):
    """CPU throughput on a bounded sample: each worker takes one touched z
    slice (slices drawn at random, seeded) and scores every listed pose of
    `triples_per_worker` of that slice's (z, beta1, beta2) triples in one
    call, so the per-z work (Bessel values, T matrix, ligand sums) is shared
    by its triples as in a full run.  Returns the measured rate (poses / the
    slowest worker's time) and the costs that extrapolate to the whole list
    (per call, per touched z, per touched triple; means over workers)."""
    from libfmftsaxs_gb300.workload import decode
    L = w.L
    K = L + 1
    zi, b1, b2 = decode(w.index, L)[:3]
    key = (zi * K + b1) * K + b2
    rng = np.random.default_rng(seed)
    zt = np.unique(zi)
    zpick = rng.choice(zt, size=workers, replace=workers > len(zt))
    jobs, ntrip = [], []
    for k in range(workers):
        trip = np.unique(key[zi == zpick[k]])
        sel = rng.choice(trip, size=min(triples_per_worker, len(trip)), replace=False)
        ntrip.append(len(sel))
        idx = w.index[np.isin(key, sel)].astype(np.int32)
        idx1 = w.index[key == sel[0]].astype(np.int32)
        jobs.append((kind, w.A, w.B, w.q, w.z, L, idx1, idx, w.a, w.mult, w.peak, w.c1g, w.c2g, w.exp,
                     (w.rmA, w.rmB, w.rm)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_worker, jobs)
    n = sum(r[0] for r in res)
    wall = max(r[1][2] for r in res)
    per_call = float(np.mean([r[1][0] for r in res]))
    multi = [(r[1][2] - r[1][1]) / (nt - 1) for r, nt in zip(res, ntrip) if nt > 1]
    per_trip = float(np.mean(multi)) if multi else float(np.mean([r[1][1] - r[1][0] for r in res]))
    per_z = float(np.mean([r[1][1] - r[1][0] for r in res])) - per_trip
    return dict(rate=n / wall, poses=n, wall=wall, per_call_s=per_call, per_z_s=max(per_z, 0.0),
                per_triple_s=per_trip, workers=workers, triples_per_worker=triples_per_worker)


def cpu_extrapolate(w, cs, ranks=8):
    """Whole-list CPU time from the sample's costs, serial and as correlate
    runs it on `ranks` MPI processes (z values dealt round-robin,
    tools/correlate.c:142-147; wall = the slowest rank, whose only exchange
    is the final gather)."""
    from libfmftsaxs_gb300.workload import decode
    L = w.L
    K = L + 1
    zi, b1, b2 = decode(w.index, L)[:3]
    trips = {}
    for z, t in zip(zi.tolist(), ((zi * K + b1) * K + b2).tolist()):
        trips.setdefault(z, set()).add(t)
    cost = {z: cs["per_z_s"] + len(t) * cs["per_triple_s"] for z, t in trips.items()}
    serial = cs["per_call_s"] + sum(cost.values())
    rank_s = [cs["per_call_s"] + sum(c for z, c in cost.items() if z % ranks == r) for r in range(ranks)]
    n = len(w.index)
    return {"serial": {"poses_per_s": n / serial, "seconds": serial, "cores": 1},
            "mpi_emulated": {"poses_per_s": n / max(rank_s), "seconds": max(rank_s), "cores": ranks,
                             "ranks": ranks},
            "touched_triples": int(sum(len(t) for t in trips.values())), "touched_z": len(trips),
            "label": "extrapolated from the sample's per-call, per-z and per-triple costs"}


def metric_name(w):
    return "poses/s @lmax=%d, grid fit %dx%d (c1 x c2)" % (w.L, len(w.c1g), len(w.c2g))


def cpu_baseline_entry(w, cs, kind):
    return {"value": cs["rate"], "unit": "poses/s", "cores": cs["workers"], "kind": kind,
            "sample": "%d poses: %d processes, each every listed pose of %d (z, beta1, beta2) triples of one z slice "
                      "in one call (per-z setup shared), grid fit; %.2f s per touched triple, %.2f s per call"
                      % (cs["poses"], cs["workers"], cs["triples_per_worker"], cs["per_triple_s"], cs["per_call_s"]),
            "whole_list": cpu_extrapolate(w, cs)}


def cpu_kind():
    from oracle import bind
    if bind.have_ref():
        try:
            bind.build_ref()
            return "reference"
        except Exception:
            pass
    bind.build_oracle()
    return "port"


# ---------------------------------------------------------------- clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()

    def summary(self):
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[0] == "0":
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][2]), "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- GPU side
# DRAM bytes per pose of the dominant kernel from ncu captures of the same
# kernel on the poses of this workload with translation z index < 3 (the
# same poses per translated row as the whole list, profiles/): the traffic
# of a launch scales with the poses it processes at that density.
TRAFFIC_PER_POSE = {("c1", "mixed"): 9.13e4, ("c1", "fp64"): 4.47e5}
# L2-to-SM bytes per pose of the FP32 per-pose kernel (ncu
# l1tex__m_xbar2l1tex_read_sectors on the same capture): the P row of every
# pose (no block shares one) and the R rows, which the poses of a warp share.
L2_TO_SM_PER_POSE = {("c1", "mixed"): 6.18e5}


def pose_flops(L, Q, precision):
    """Algorithmic FLOPs of the per-pose contraction for one pose (both
    precisions run the same kernel): over the (L+1)(L+2)/2 pairs
    (m >= 0, l >= m) and Q q values, the phase w_m applied to the 3 channels
    of R (3 complex multiplies, 18 FLOPs) and the real parts of the 9
    channel products (36 FLOPs)."""
    NP = (L + 1) * (L + 2) // 2
    return Q * NP * 54


def reference_flops(w):
    """F_ref of the reference algorithm on this pose list: per touched
    (z, beta1, beta2) triple 72 Q N S(L) (sum2) + 30 Q N^3 log2 N (6-channel DFT),
    per touched (z, beta2) 24 Q sum_{m,m2} sum_{l>=|m|} (K - max(|m|,|m2|,l))."""
    from libfmftsaxs_gb300.workload import decode
    L, Q = w.L, w.Q
    K, N = L + 1, 2 * L + 1
    S = sum(K - max(abs(m), abs(m1)) for m in range(-L, L + 1) for m1 in range(-L, L + 1))
    s1 = sum(max(0, K - max(abs(m), abs(m2), l)) for m in range(-L, L + 1) for m2 in range(-L, L + 1)
             for l in range(abs(m), K))
    z, b1, b2 = decode(w.index, L)[:3]
    ntrip = len(np.unique((z * K + b1) * K + b2))
    nzb2 = len(np.unique(z * K + b2))
    return ntrip * (72.0 * Q * N * S + 30.0 * Q * N ** 3 * np.log2(N)) + nzb2 * 24.0 * Q * s1


def time_plan(g, w, precision, args, clocks=None):
    """K timed runs of a resident plan (inputs on the device); returns
    (ms per run from events on the library stream, stage ms, launches, results)."""
    plan = g.Plan(w.A, w.B, w.q, w.z, w.L, w.a, w.mult, w.peak, w.c1g, w.c2g, precision=precision)
    plan.set_rotation(g.ROT_TC if args.rotation == "tc" else g.ROT_CUDA)
    if args.budget_gb:
        plan.set_budget(int(args.budget_gb * 2 ** 30))
    plan.set_poses(w.index, skip=1)
    for _ in range(args.warmup):
        plan.run(g.FIT_GRID)
    l0 = g.launch_count()
    stage = np.zeros(5)
    ctx = clocks if clocks is not None else _Null()
    with ctx:
        g.timer_start()
        for _ in range(args.steps):
            plan.run(g.FIT_GRID)
            t = plan.timings()
            stage += np.array([t["tables"], t["translate"], t["pose"], t["fit"], t["total"]])
        ms = g.timer_stop()
    launches = g.launch_count() - l0
    res = plan.results()
    nchunks = plan.chunks()
    plan.close()
    return ms / args.steps, stage / args.steps, launches, res, nchunks


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass


def model_intensity(cross, q, mult, c1, c2):
    """point_score's model I(q) (src/min_saxs.c:391-448) of raw cross terms
    [n][6][Q] at per-pose (c1, c2); the peak rescale is a common factor and
    leaves relative errors unchanged."""
    c1 = np.asarray(c1)[:, None]
    c2 = np.asarray(c2)[:, None]
    G = c1 ** 3 * np.exp(-mult * (c1 * c1 - 1.0) * q[None, :] ** 2)
    VV, VD, VW, DD, DW, WW = (cross[:, c, :] for c in range(6))
    return VV - G * VD + c2 * VW + G * G * DD - G * c2 * DW + c2 * c2 * WW


def iq_accuracy(g, w, n=4000):
    """I(q) of the mixed path against the FP64 path on the first n poses, at
    the FP64 path's best (c1, c2) cell of each pose."""
    idx = w.index[:n]
    out = {}
    for prec in (g.FP64, g.MIXED):
        p = g.Plan(w.A, w.B, w.q, w.z, w.L, w.a, w.mult, w.peak, w.c1g, w.c2g, precision=prec)
        p.set_poses(idx, skip=1)
        p.run(g.FIT_GRID)
        out[prec] = p.results(cross=True)
        p.close()
    ref = out[g.FP64]
    i_ref = model_intensity(ref["cross"], w.q, w.mult, ref["c1"], ref["c2"])
    i_mix = model_intensity(out[g.MIXED]["cross"], w.q, w.mult, ref["c1"], ref["c2"])
    rel = np.abs(i_mix - i_ref) / np.abs(i_ref)
    return {"iq_rel_max": float(rel.max()), "iq_rel_median": float(np.median(rel)), "iq_poses": len(idx)}


def accuracy(mix, ref, k=100, topk=None):
    rel = np.abs(mix["chi"] - ref["chi"]) / ref["chi"]
    top_m = set(np.argsort(mix["chi"], kind="stable")[:k].tolist())
    top_r = set(np.argsort(ref["chi"], kind="stable")[:k].tolist())
    out = {"vs": "FP64 GPU path (within 1e-10 of the reference build on the C0/C1-shape fixtures)",
           "dchi_rel_max": float(rel.max()), "dchi_rel_median": float(np.median(rel)), "bound": 1e-4,
           "top%d_overlap" % k: len(top_m & top_r) / k, "same_cell": float(np.mean(mix["cell"] == ref["cell"]))}
    if topk is not None:
        out["top%d_device" % k] = {
            "mixed_equals_argsort": bool(np.array_equal(topk["mixed"], np.argsort(mix["chi"], kind="stable")[:k])),
            "fp64_equals_argsort": bool(np.array_equal(topk["fp64"], np.argsort(ref["chi"], kind="stable")[:k])),
            "overlap": len(set(topk["mixed"].tolist()) & set(topk["fp64"].tolist())) / k}
    return out


def expansion_timing(g, w, fp64_peak):
    """The A_lm expansion per molecule (sxsg_expand, with its transfers of a
    few MB) and its FP64 rate over the accumulation's 12 FLOPs per atom, q
    and (l, m) (3 channels of complex-by-real multiply-adds)."""
    out = {}
    water = g.ff_water()
    for name, m in (("receptor", w.rec), ("ligand", w.lig)):
        v = np.array([g.ff_type(e)[0] for e in m.elements])
        d = np.array([g.ff_type(e)[1] for e in m.elements])
        g.expand(m.xyz, v, d, m.sasa, water, w.q, w.L)
        ts = []
        for _ in range(3):
            g.timer_start()
            g.expand(m.xyz, v, d, m.sasa, water, w.q, w.L)
            ts.append(g.timer_stop())
        ms = float(np.median(ts))
        tf = 12.0 * m.natoms * w.Q * (w.L + 1) ** 2 / (ms * 1e-3) / 1e12
        out[name] = {"atoms": m.natoms, "ms": ms, "fp64_tflops": tf,
                     "fp64_frac": tf / fp64_peak if fp64_peak > 0 else None}
    return out


def run_serving(g, args):
    """Serving scenario: Poisson arrivals of scoring requests (each one dimer
    with its own lmax, q grid, experiment and pose list) into the serving
    loop; latency = submit to results on the host.  Requests draw their pose
    lists as windows of one seeded list per L (generated once and ingested on
    the GPU), so that long windows need no per-request pose generation; a
    waiter thread collects results while requests keep arriving."""
    import threading
    from libfmftsaxs_gb300 import synth, workload as wl
    rng = np.random.default_rng(args.seed + 77)
    Ls, Qs = (10, 15, 20, 25, 30), (51, 101, 201)
    nrec, nlig = 4, 4
    def mol(lo, hi, seed):
        na = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        return synth.make_molecule(na, 2.2 * (na / 8.0) ** 0.38, seed)   # Rg of a compact protein of na/8 residues
    recs = [mol(500, 8000, 900 + i) for i in range(nrec)]
    ligs = [mol(300, 5000, 950 + i) for i in range(nlig)]
    recs = [m.translated(-m.center_of_extrema()).with_sasa() for m in recs]
    ligs = [m.translated(-m.centroid()).with_sasa() for m in ligs]
    expd = {}

    def expansion(kind, i, L, Q):
        key = (kind, i, L, Q)
        if key not in expd:
            m = (recs if kind == "r" else ligs)[i]
            v, d = wl.form_factors(g, m)
            q = g.mkarray(0.0, 0.5, Q)
            expd[key] = g.expand(m.xyz, v, d, m.sasa, g.ff_water(), q, L)
        return expd[key]

    z = np.arange(25.0, 46.0)
    pool_n = args.serve_max_poses
    pools = {}
    for L in Ls:
        r = np.random.default_rng(args.seed + 500 + L)
        idx = []
        while sum(len(x) for x in idx) < pool_n:
            m = min(1 << 20, 2 * pool_n)
            R = synth.random_rotations(m, r)
            T = synth.random_translations(m, 25.0, 45.0, r)
            idx.append(g.poses_to_indices_gpu(R, T, z, L)[0])
        pools[L] = np.concatenate(idx)[:pool_n]
    profiles = {}

    def request(k, used_rec):
        if used_rec and rng.random() < 0.3:
            ri, L, Q = used_rec[rng.integers(len(used_rec))]
        else:
            ri, L, Q = int(rng.integers(nrec)), int(rng.choice(Ls)), int(rng.choice(Qs))
            used_rec.append((ri, L, Q))
        li = int(rng.integers(nlig))
        q = g.mkarray(0.0, 0.5, Q)
        A, B = expansion("r", ri, L, Q), expansion("l", li, L, Q)
        if (ri, L, Q) not in profiles:
            profiles[(ri, L, Q)] = g.profile_from_spf(A, L, q, 1.7, 1.0, 1.0)[0]
        exp = synth.noisy_experiment(q, profiles[(ri, L, Q)], 0.01, rng)
        a, mult, peak = g.bin_experiment(exp[0], exp[1], exp[2], q, 1.7)
        npose = int(np.exp(rng.uniform(np.log(args.serve_min_poses), np.log(args.serve_max_poses))))
        off = int(rng.integers(0, pool_n - npose + 1))
        return dict(A=A, B=B, qvals=q, zvals=z, L=L, a=a, mult=mult, peak=peak, index=pools[L][off:off + npose],
                    c1grid=synth.C1_GRID, c2grid=synth.C2_GRID, keyA=1000 * ri + 1, keyB=2000 * li + 2)

    out = {}
    for prec, name in ((g.MIXED, "mixed"), (g.FP64, "fp64")):
        if name == "fp64" and not args.serve_fp64:
            continue
        window = args.serve_window if name == "mixed" else (args.serve_fp64_window or args.serve_window)
        nreq = max(1, int(round(args.serve_rate * window)))
        arrivals = np.cumsum(rng.exponential(1.0 / args.serve_rate, size=nreq))
        used_rec = []
        reqs = [request(k, used_rec) for k in range(nreq)]
        srv = g.Server(hbm_cap=int(args.serve_cap_gb * 2 ** 30), max_active=args.serve_active)
        tickets, lat = [], []
        cv = threading.Condition()

        def waiter():
            k = 0
            while k < nreq:
                with cv:
                    while k >= len(tickets):
                        cv.wait()
                    t = tickets[k]
                lat.append(srv.wait(t)["latency_ms"])
                k += 1
        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        for r, ta in zip(reqs, arrivals):
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            t = srv.submit(precision=prec, **r)
            with cv:
                tickets.append(t)
                cv.notify()
        t_sub = time.perf_counter() - t0
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        lat = np.array(lat)
        poses = sum(len(r["index"]) for r in reqs)
        out[name] = {"requests": nreq, "window_s": window, "p50_ms": float(np.percentile(lat, 50)),
                     "p95_ms": float(np.percentile(lat, 95)), "p99_ms": float(np.percentile(lat, 99)),
                     "max_ms": float(lat.max()), "poses": int(poses), "poses_per_s": poses / wall,
                     "offered_poses_per_s": poses / t_sub, "requests_per_s": nreq / wall, "drain_s": wall - t_sub,
                     "cache_hits": st["cache_hits"], "cache_misses": st["cache_misses"]}
    out["scenario"] = ("Poisson arrivals at %.0f/s; each request one dimer: receptor %d-%d atoms, ligand %d-%d "
                       "(pools of %d and %d molecules, 30%% of requests reuse a served receptor), L in %s, Q in %s, "
                       "%d-%d poses log-uniform (windows of one seeded list per L), |t| in [25,45] A, grid fit "
                       "11x41; up to %d jobs on the device under a %.0f GB cap; poses_per_s = all poses over "
                       "first arrival to last result"
                       % (args.serve_rate, min(r.natoms for r in recs), max(r.natoms for r in recs),
                          min(m.natoms for m in ligs), max(m.natoms for m in ligs), nrec, nlig, list(Ls), list(Qs),
                          args.serve_min_poses, args.serve_max_poses, args.serve_active, args.serve_cap_gb))
    return out


def run_batch(g, args):
    """Many uneven dimers (workload.batch_specs, mixed precision, grid fit)
    scored three ways:
      graph    the resident plans of a wave of dimers that fit in device
               memory scored by one CUDA graph of persistent kernels
               (sxsg_batch_run); checked bit for bit against the plan runs
      plans    the same resident plans run one after another (sxsg_plan_run)
      serving  the same dimers submitted at once to the serving loop, which
               sets up each job (uploads, pose decode, tables) itself
    Times are host wall clock around synchronous calls; the graph's device
    time per stage comes from event nodes in the graph."""
    from libfmftsaxs_gb300 import workload as wl
    specs, rpool, lpool = wl.batch_specs(args.batch_dimers * (1 if args.batch_lmax >= 30 else 4), seed=args.seed + 3,
                                         max_poses=args.batch_max_poses)
    specs = [sp for sp in specs if sp["L"] <= args.batch_lmax][:args.batch_dimers]   # profiling cases
    t0 = time.perf_counter()
    ur = sorted({sp["rec"] for sp in specs})
    ul = sorted({sp["lig"] for sp in specs})
    nw = min(16, os.cpu_count() or 1)
    recs = dict(zip(ur, wl.pool_molecules([rpool[i] for i in ur], workers=nw)))
    ligs = dict(zip(ul, wl.pool_molecules([lpool[i] for i in ul], workers=nw)))
    dims = [wl.build_dimer(sp, recs[sp["rec"]], ligs[sp["lig"]], g) for sp in specs]
    t_build = time.perf_counter() - t0
    poses = sum(len(d.index) for d in dims)
    free, total = g.device_memory()
    budget = int(0.7 * free)
    waves, cur, used = [], [], 0
    for i, d in enumerate(dims):
        nb = wl.plan_bytes(d.L, d.Q, len(d.index), len(d.z))
        if cur and used + nb > budget:
            waves.append(cur)
            cur, used = [], 0
        cur.append(i)
        used += nb
    if cur:
        waves.append(cur)
    graph_s, plans_s, same = 0.0, 0.0, True
    forms, seq_stage = {}, np.zeros(4)
    dev = np.zeros(3)
    phases = launches = items = 0
    create_s = 0.0
    for wv in waves:
        plans = []
        for i in wv:
            d = dims[i]
            p = g.Plan(d.A, d.B, d.q, d.z, d.L, d.a, d.mult, d.peak, d.c1g, d.c2g, precision=g.MIXED)
            p.set_poses(d.index, skip=1)
            plans.append(p)
        t0 = time.perf_counter()
        b = g.Batch(plans, fit=g.FIT_GRID)
        create_s += time.perf_counter() - t0
        for _ in range(args.warmup):
            b.run()
        ts, ds = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            b.run()
            ts.append(time.perf_counter() - t0)
            st = b.stats()
            ds.append((st["tables_ms"], st["phases_ms"], st["fit_ms"]))
        graph_s += float(np.median(ts))
        dev += np.median(np.array(ds), axis=0)
        phases += st["phases"]
        launches += st["launches"]
        items += st["items"]
        got = [p.results() for p in plans]
        arena = st["arena_bytes"]
        b.close()
        # the other launch forms, briefly (each checked bit for bit below)
        for fl in (0, g.BATCH_PERSISTENT, g.BATCH_OVERLAP | g.BATCH_PERSISTENT, g.BATCH_ITEMS,
                   g.BATCH_ITEMS | g.BATCH_PERSISTENT, g.BATCH_ITEMS | g.BATCH_PERSISTENT | g.BATCH_OVERLAP):
            if fl == g.BATCH_DEFAULT:
                continue
            bb = g.Batch(plans, fit=g.FIT_GRID, flags=fl)
            bb.run()
            t0 = time.perf_counter()
            bb.run()
            f = forms.setdefault(fl, np.zeros(4))
            f[0] += time.perf_counter() - t0
            sf = bb.stats()
            f[1:] += (sf["tables_ms"], sf["phases_ms"], sf["fit_ms"])
            bb.close()
            same &= all(np.array_equal(p.results()["chi"], r["chi"]) for p, r in zip(plans, got))

        def seq():
            # each plan with the batch's arena as its translated-table bound,
            # released after its run so that the next plan has the room
            st4 = np.zeros(4)
            for p in plans:
                p.set_budget(arena)
                p.run(g.FIT_GRID)
                tm = p.timings()
                st4 += (tm["tables"], tm["translate"], tm["pose"], tm["fit"])
                p.set_budget(1)
            return st4
        seq()
        t0 = time.perf_counter()
        seq_stage += seq()
        plans_s += time.perf_counter() - t0
        for p, r in zip(plans, got):
            a = p.results()
            same &= all(np.array_equal(a[k], r[k]) for k in ("chi", "c1", "c2", "cell"))
            p.close()
    srv_s = None
    if not args.skip_batch_serve:
        for rep in range(2):
            srv = g.Server(max_active=args.serve_active)
            t0 = time.perf_counter()
            tickets = [srv.submit(A=d.A, B=d.B, qvals=d.q, zvals=d.z, L=d.L, a=d.a, mult=d.mult, peak=d.peak,
                                  index=d.index, c1grid=d.c1g, c2grid=d.c2g, precision=g.MIXED) for d in dims]
            for t in tickets:
                srv.wait(t)
            srv_s = time.perf_counter() - t0
            srv.close()
    hist = {}
    for d in dims:
        hist["L%d" % d.L] = hist.get("L%d" % d.L, 0) + 1
    out = {"dimers": len(dims), "poses": int(poses), "waves": len(waves), "phases": int(phases),
           "graph_kernel_launches": int(launches), "work_items": int(items),
           "graph": {"ms_per_step": graph_s * 1e3, "poses_per_s": poses / graph_s,
                     "device_ms": {"tables": dev[0], "translate_and_pose": dev[1], "fit": dev[2]}},
           "graph_forms_ms": {{0: "chunk_launches", 1: "chunk_launches+persistent", 3: "chunk_launches+persistent+overlap",
                               4: "items", 5: "items+persistent", 7: "items+persistent+overlap"}[k]:
                              {"total": v[0] * 1e3, "tables": v[1], "phases": v[2], "fit": v[3]}
                              for k, v in forms.items()},
           "graph_default_form": "chunk_launches+persistent (translation and per-pose work as single-dimer launches "
                                 "per chunk; rotations and fit as persistent work-item launches)",
           "plans_sequential": {"ms_per_step": plans_s * 1e3, "poses_per_s": poses / plans_s,
                                "device_ms": dict(zip(("tables", "translate", "pose", "fit"), seq_stage.tolist()))},
           "serving": ({"ms_per_step": srv_s * 1e3, "poses_per_s": poses / srv_s,
                        "note": "per-job plan set-up, uploads and pose decode included; %d jobs on the device"
                                % args.serve_active} if srv_s else None),
           "bitwise_equal_to_plan_runs": bool(same),
           "setup_s": {"dimers": t_build, "batch_create": create_s},
           "scenario": "%d dimers from pools of %d receptors (%d-%d atoms) and %d ligands (%d-%d atoms); L %s; "
                       "Q in {51, 101, 201}; %d-%d poses log-uniform (|t| in [25, 45] A), %d in all; grid fit 11x41; "
                       "steps: median of %d graph replays after %d"
                       % (len(dims), len(ur), min(rpool[i][0] for i in ur), max(rpool[i][0] for i in ur), len(ul),
                          min(lpool[i][0] for i in ul), max(lpool[i][0] for i in ul), json.dumps(hist),
                          min(len(d.index) for d in dims), max(len(d.index) for d in dims), poses, args.steps,
                          args.warmup)}
    return out


def run_ours(args):
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import build as libbuild
    from libfmftsaxs_gb300 import workload as wl
    if not os.path.exists(g.LIB_PATH):
        libbuild.build()
    kind = cpu_kind()          # build the CPU checker before the first GPU call
    g.init(0)
    w = wl.build(args.config, seed=args.seed)
    if args.zsub:
        w.index = w.index[wl.decode(w.index, w.L)[0] < args.zsub]
    if args.poses:
        w.index = w.index[:args.poses]
    n = len(w.index)

    # CPU baseline sample first (spawned processes, no GPU use)
    workers = max(1, min(os.cpu_count() or 1, 16))
    cs = cpu_sample(w, kind, workers) if not args.skip_cpu else None

    fp64_peak = max(g.fp64_fma_tflops() for _ in range(3))
    fp32_peak = max(g.fp32_fma_tflops() for _ in range(3))
    l2_peak = max(g.l2_read_gbs() for _ in range(3))
    head = args.precision
    prec = {"mixed": g.MIXED, "fp64": g.FP64}
    runs = {}
    for name in (["fp64", "mixed"] if head == "mixed" else ["fp64"]):
        if name == head:
            with Clocks() as clk:
                runs[name] = time_plan(g, w, prec[name], args)
            clocks = clk.summary()
        else:
            runs[name] = time_plan(g, w, prec[name], args)
    ms, stage, launches, res, nchunks = runs[head]
    value = n / (ms * 1e-3)

    # end to end through the one-shot C-ABI call from host buffers
    idx = np.ascontiguousarray(w.index, dtype=np.int64)
    e2e_s = float("nan")
    if not args.skip_e2e:
        g.score_flat(w.A, w.B, w.q, w.z, w.L, idx, w.a, w.mult, w.peak, 1, g.FIT_GRID, w.c1g, w.c2g,
                     precision=prec[head])
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g.score_flat(w.A, w.B, w.q, w.z, w.L, idx, w.a, w.mult, w.peak, 1, g.FIT_GRID, w.c1g, w.c2g,
                         precision=prec[head])
        e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = w.A.nbytes + w.B.nbytes + w.q.nbytes + w.z.nbytes + w.a.nbytes + idx.nbytes + w.c1g.nbytes + w.c2g.nbytes
    d2h = 3 * 8 * n

    pf = pose_flops(w.L, w.Q, head) * n
    achieved = pf / (stage[2] * 1e-3) / 1e12
    peak = fp32_peak if head == "mixed" else fp64_peak
    fref = reference_flops(w)
    tkey = (args.config, head)
    traffic = TRAFFIC_PER_POSE[tkey] * n / nchunks if tkey in TRAFFIC_PER_POSE else None
    out = {
        "metric": metric_name(w),
        "value": value,
        "unit": "poses/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64" if head == "mixed" else "f64",
        "data": "synthetic (seeded random-walk dimers, poses and noisy experiment)",
        "config": {"workload": "%s: receptor %d / ligand %d atoms, L=%d, Q=%d, %d poses, fit grid %dx%d"
                               % (args.config, w.rec.natoms, w.lig.natoms, w.L, w.Q, n, len(w.c1g), len(w.c2g)),
                   "precision": head, "skip": 1,
                   "l2": "inputs larger than L2 (rotation tables of ~1 GB and translated tables of several GB per step)"},
        "stages_ms": {"tables": stage[0], "translate": stage[1], "pose": stage[2], "fit": stage[3],
                      "note": "stages run in order on the plan stream; translate and pose summed over %d chunk(s)"
                              % nchunks},
        "fp64": {"value": n / (runs["fp64"][0] * 1e-3), "unit": "poses/s", "ms_per_step": runs["fp64"][0],
                 "stages_ms": dict(zip(("tables", "translate", "pose", "fit"), runs["fp64"][1][:4].tolist()))},
        "reference_flops_per_step": fref,
        "reference_equiv_tflops": fref / (ms * 1e-3) / 1e12,
        "roofline": {"bound": "fp32" if head == "mixed" else "fp64",
                     "kernel": "k_pose_cross<%s>" % ("float" if head == "mixed" else "double"),
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak > 0 else None,
                     "traffic": traffic,
                     "traffic_source": "ncu DRAM read+write per pose of the same kernel on the poses with z index < 3 "
                                       "(z index < 1 for FP64), "
                                       "scaled to the poses of one launch (%d chunk(s) per run)" % nchunks,
                     "hbm_frac": (traffic * nchunks / (stage[2] * 1e-3) / 1e9 / 6773.5) if traffic else None,
                     "peak_source": "measured in this run: register-resident %s FMA chains on every SM"
                                    % ("FP32" if head == "mixed" else "FP64")},
        "cpu_baseline": cpu_baseline_entry(w, cs, kind) if cs else None,
        "e2e": {"value": n / e2e_s, "unit": "poses/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    l2key = (args.config, head)
    if l2key in L2_TO_SM_PER_POSE and not args.zsub and not args.poses:
        # the FP32 per-pose kernel is bound by moving P and R rows from L2
        # into the SMs (L1 data path 88 % busy, FMA pipe 48 %): that is its roofline
        rl = out["roofline"]
        l2_ach = L2_TO_SM_PER_POSE[l2key] * n / (stage[2] * 1e-3) / 1e9
        rl["fp32"] = {"achieved": rl["achieved"], "peak": rl["peak"], "unit": "TFLOP/s", "frac": rl["frac"]}
        rl.update({"bound": "l2", "achieved": l2_ach, "peak": l2_peak, "unit": "GB/s",
                   "frac": l2_ach / l2_peak if l2_peak > 0 else None,
                   "l2_source": "ncu L2-to-SM read bytes per pose (618 KB) x poses / kernel time",
                   "peak_source": "measured in this run: 16-byte L2-only loads by every SM over a 32 MiB "
                                  "L2-resident buffer"})
    if head == "mixed":
        tk = None
        if n >= 100:
            tk = {}
            for name in ("fp64", "mixed"):
                p = g.Plan(w.A, w.B, w.q, w.z, w.L, w.a, w.mult, w.peak, w.c1g, w.c2g, precision=prec[name])
                p.set_poses(w.index, skip=1)
                p.run(g.FIT_GRID)
                tk[name] = p.topk(100)["pose"]
                p.close()
        out["accuracy"] = accuracy(res, runs["fp64"][3], topk=tk)
        out["accuracy"].update(iq_accuracy(g, w))
    out["expansion"] = expansion_timing(g, w, fp64_peak)
    if not args.skip_serve:
        out["serving"] = run_serving(g, args)
    if not args.skip_batch:
        out["batch"] = run_batch(g, args)
    print(json.dumps(out))


def run_reference(args):
    """The reference algorithm on the host cores: the reference's own code
    (oracle/_ref) where it was built, else the C restatement, on the same
    workload, whose inputs the oracle builds (no GPU, no product library)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from libfmftsaxs_gb300 import workload as wl
    from oracle.bind import OracleWorkload
    kind = cpu_kind()
    w = wl.build(args.config, seed=args.seed, lib=OracleWorkload())
    workers = max(1, min(os.cpu_count() or 1, 16))
    tpw = 4 if args.steps + args.warmup <= 8 else 2
    cpu_sample(w, kind, workers, triples_per_worker=1, seed=1000)   # warm-up: start-up and caches
    samples = [cpu_sample(w, kind, workers, triples_per_worker=tpw, seed=k) for k in range(args.steps)]
    n = sum(c["poses"] for c in samples)
    wall = sum(c["wall"] for c in samples)
    value = n / wall
    agg = dict(samples[0], rate=value, poses=n, wall=wall,
               per_call_s=float(np.mean([c["per_call_s"] for c in samples])),
               per_z_s=float(np.mean([c["per_z_s"] for c in samples])),
               per_triple_s=float(np.mean([c["per_triple_s"] for c in samples])))
    out = {"impl": "reference", "metric": metric_name(w), "value": value, "unit": "poses/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded random-walk dimers, poses and noisy experiment)",
           "config": {"workload": "%s: receptor %d / ligand %d atoms, L=%d, Q=%d, %d poses, fit grid %dx%d"
                                  % (args.config, w.rec.natoms, w.lig.natoms, w.L, w.Q, len(w.index), len(w.c1g),
                                     len(w.c2g)),
                      "precision": "fp64 (the reference's CPU arithmetic)", "skip": 1,
                      "sample": "each step: %d processes, each the listed poses of %d triples of one z slice"
                                % (workers, tpw)},
           "cpu_baseline": cpu_baseline_entry(w, agg, kind),
           "e2e": {"value": value, "unit": "poses/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2"])
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--poses", type=int, default=0, help="score only the first N poses (profiling cases)")
    ap.add_argument("--zsub", type=int, default=0,
                    help="score only the poses with translation z index < K: a profiling case with the whole "
                         "list's poses per translated row")
    ap.add_argument("--budget-gb", type=float, default=0.0, help="cap on the translated-table chunk (GiB)")
    ap.add_argument("--skip-cpu", action="store_true", help="no CPU baseline sample")
    ap.add_argument("--skip-e2e", action="store_true", help="no end-to-end timing")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--rotation", default="cuda", choices=["tc", "cuda"],
                    help="mixed path: rotation tables on the tcgen05 tensor cores or on CUDA cores")
    ap.add_argument("--skip-serve", action="store_true", help="no serving scenario")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="serving: mean arrivals per second")
    ap.add_argument("--serve-window", type=float, default=2.0, help="serving: seconds of arrivals")
    ap.add_argument("--serve-min-poses", type=int, default=5000)
    ap.add_argument("--serve-max-poses", type=int, default=50000)
    ap.add_argument("--serve-active", type=int, default=4, help="serving: jobs on the device at once")
    ap.add_argument("--serve-cap-gb", type=float, default=150.0, help="serving: HBM cap")
    ap.add_argument("--serve-fp64", action="store_true", help="serving: also run the FP64 path")
    ap.add_argument("--serve-fp64-window", type=float, default=0.0,
                    help="serving: seconds of arrivals for the FP64 arm (0 = --serve-window)")
    ap.add_argument("--skip-batch", action="store_true", help="no batched-dimers scenario")
    ap.add_argument("--skip-batch-serve", action="store_true", help="batched dimers: no serving comparison")
    ap.add_argument("--batch-dimers", type=int, default=64)
    ap.add_argument("--batch-max-poses", type=int, default=200000)
    ap.add_argument("--batch-lmax", type=int, default=30, help="batched dimers: only those with L up to this")
    args = ap.parse_args()
    if args.gpus > 1 and int(os.environ.get("RANK", "0")) != 0:
        return  # the path does not shard: one GPU runs, other ranks idle
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
