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
    """Score one sample of poses with a CPU implementation; returns (n, s)."""
    kind, A, B, q, z, L, idx, a, mult, peak, c1g, c2g, exp, rms = args
    from oracle import bind
    if kind == "reference":
        r = bind.Ref()
        r.score(A, B, rms[0], rms[1], rms[2], exp, q, z, L, idx[:1], 1, c1g[:1], c2g[:1])  # warm the tables
        t = time.perf_counter()
        r.score(A, B, rms[0], rms[1], rms[2], exp, q, z, L, idx, 1, c1g, c2g)
    else:
        o = bind.Oracle()
        o.score(A, B, q, z, L, idx[:1], 1, peak, a, mult, c1g[:1], c2g[:1])  # build the 3j table once
        t = time.perf_counter()
        o.score(A, B, q, z, L, idx, 1, peak, a, mult, c1g, c2g)
    return len(idx), time.perf_counter() - t


def cpu_sample(w, kind, workers, triples_per_worker=1, seed=11):
    """Each worker scores all listed poses of `triples_per_worker` distinct
    (z, beta1, beta2) triples drawn from the workload (the unit of work of
    the reference loop).  Rate = poses scored / slowest worker's time."""
    from libfmftsaxs_gb300.workload import decode, triple_counts
    L = w.L
    keys, counts = triple_counts(w.index, L)
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(keys), size=workers * triples_per_worker, replace=False)
    z, b1, b2 = decode(w.index, L)[:3]
    key = (z * (L + 1) + b1) * (L + 1) + b2
    jobs = []
    for k in range(workers):
        sel = keys[pick[k * triples_per_worker:(k + 1) * triples_per_worker]]
        idx = w.index[np.isin(key, sel)].astype(np.int32)
        jobs.append((kind, w.A, w.B, w.q, w.z, L, idx, w.a, w.mult, w.peak, w.c1g, w.c2g, w.exp,
                     (w.rmA, w.rmB, w.rm)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_worker, jobs)
    n = sum(r[0] for r in res)
    wall = max(r[1] for r in res)
    return n / wall, n, wall


def cpu_kind():
    from oracle import bind
    if os.path.isdir(bind.REF_SRC):
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
# DRAM bytes per pose of k_pose_cross from the ncu capture summarised in
# profiles/k_pose_cross_c1_fp64.md (1.228 GB read + 4 MB written for 318
# poses); the traffic of a launch scales with its pose count.
TRAFFIC_PER_POSE = {"c1": 3.873e6}


def pose_flops(L, Q):
    """Algorithmic FLOPs of the per-pose contraction for one pose: for each
    q, 9 complex multiply-adds (the 3x3 channel products) per (m, l) pair,
    (L+1)^2 pairs, 8 FLOPs per complex multiply-add."""
    return Q * (L + 1) ** 2 * 9 * 8


def reference_flops(w):
    """F_ref of the reference algorithm on this pose list: per touched
    (z, b1, b2) triple 72 Q N S(L) (sum2) + 30 Q N^3 log2 N (6-channel DFT),
    per touched (z, b2) 24 Q sum_{m,m2} sum_{l>=|m|} (K - max(|m|,|m2|,l))."""
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


def run_ours(args):
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import build as libbuild
    from libfmftsaxs_gb300 import workload as wl
    if not os.path.exists(g.LIB_PATH):
        libbuild.build()
    kind = cpu_kind()          # build the CPU checker before the first GPU call
    g.init(0)
    w = wl.build(args.config, seed=args.seed)
    if args.poses:
        w.index = w.index[:args.poses]
    n = len(w.index)

    # CPU baseline sample first (spawned processes, no GPU use)
    workers = max(1, min(os.cpu_count() or 1, 16))
    cpu_rate, cpu_n, cpu_wall = cpu_sample(w, kind, workers) if not args.skip_cpu else (None, 0, 0)

    prec = g.MIXED if args.precision == "mixed" else g.FP64
    plan = g.Plan(w.A, w.B, w.q, w.z, w.L, w.a, w.mult, w.peak, w.c1g, w.c2g, precision=prec)
    if args.budget_gb:
        plan.set_budget(int(args.budget_gb * 2 ** 30))
    plan.set_poses(w.index, skip=1)
    for _ in range(args.warmup):
        plan.run(g.FIT_GRID)
    fp64_peak = max(g.fp64_fma_tflops() for _ in range(3))
    l0 = g.launch_count()
    with Clocks() as clk:
        g.timer_start()
        stage = np.zeros(5)
        for _ in range(args.steps):
            plan.run(g.FIT_GRID)
            t = plan.timings()
            stage += np.array([t["tables"], t["translate"], t["pose"], t["fit"], t["total"]])
        ms = g.timer_stop()
    launches = g.launch_count() - l0
    clocks = clk.summary()
    value = n * args.steps / (ms * 1e-3)
    stage /= args.steps

    # end to end through the one-shot C-ABI call from host buffers
    idx = np.ascontiguousarray(w.index, dtype=np.int64)
    e2e_s = float("nan")
    if not args.skip_e2e:
        g.score_flat(w.A, w.B, w.q, w.z, w.L, idx, w.a, w.mult, w.peak, 1, g.FIT_GRID, w.c1g, w.c2g)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g.score_flat(w.A, w.B, w.q, w.z, w.L, idx, w.a, w.mult, w.peak, 1, g.FIT_GRID, w.c1g, w.c2g)
        e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = w.A.nbytes + w.B.nbytes + w.q.nbytes + w.z.nbytes + w.a.nbytes + idx.nbytes + w.c1g.nbytes + w.c2g.nbytes
    d2h = 3 * 8 * n

    pf = pose_flops(w.L, w.Q) * n
    achieved = pf / (stage[2] * 1e-3) / 1e12
    fref = reference_flops(w)
    out = {
        "metric": "poses/s @lmax=20 (FP64 plain GPU path, grid fit)",
        "value": value,
        "unit": "poses/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded random-walk dimers, poses and noisy experiment)",
        "config": {"workload": "%s: receptor %d / ligand %d atoms, L=%d, Q=%d, %d poses, fit grid %dx%d"
                               % (args.config, w.rec.natoms, w.lig.natoms, w.L, w.Q, n, len(w.c1g), len(w.c2g)),
                   "precision": "fp64", "skip": 1,
                   "l2": "inputs larger than L2 (rotation/translation tables of several GB per step)"},
        "stages_ms": {"tables": stage[0], "translate": stage[1], "pose": stage[2], "fit": stage[3]},
        "reference_flops_per_step": fref,
        "reference_equiv_tflops": fref / (ms / args.steps * 1e-3) / 1e12,
        "roofline": {"bound": "fp64", "kernel": "k_pose_cross", "achieved": achieved, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak > 0 else None,
                     "traffic": TRAFFIC_PER_POSE[args.config] * n if args.config in TRAFFIC_PER_POSE else None,
                     "traffic_source": "ncu capture of 318 poses, scaled by poses per launch",
                     "peak_source": "measured in this run: register-resident FP64 FMA chains on every SM"},
        "cpu_baseline": {"value": cpu_rate, "unit": "poses/s", "cores": workers, "kind": kind,
                         "sample": "%d poses of %d (z,beta1,beta2) triples, one triple per process, grid fit"
                                   % (cpu_n, workers)},
        "e2e": {"value": n / e2e_s, "unit": "poses/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(out))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import libfmftsaxs_gb300 as g
    from libfmftsaxs_gb300 import build as libbuild
    from libfmftsaxs_gb300 import workload as wl
    kind = cpu_kind()
    if not os.path.exists(g.LIB_PATH):
        libbuild.build()
    # the workload's inputs (expansions, experiment) come from the GPU library;
    # the timed work is the CPU implementation only
    g.init(0)
    w = wl.build(args.config, seed=args.seed)
    workers = max(1, min(os.cpu_count() or 1, 16))
    for _ in range(args.warmup):
        cpu_sample(w, kind, workers, seed=1000 + _)
    rates, ns, walls = [], [], []
    for k in range(args.steps):
        r, n, wall = cpu_sample(w, kind, workers, seed=k)
        rates.append(r); ns.append(n); walls.append(wall)
    value = sum(ns) / sum(walls)
    out = {"impl": "reference", "metric": "poses/s @lmax=20 (FP64 plain GPU path, grid fit)", "value": value,
           "unit": "poses/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * float(np.mean(walls)), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.config, "sample": "one (z,beta1,beta2) triple per host process"},
           "cpu_baseline": {"value": value, "unit": "poses/s", "cores": workers, "kind": kind,
                            "sample": "%d processes x 1 triple per step" % workers},
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
    ap.add_argument("--budget-gb", type=float, default=0.0, help="cap on the translated-table chunk (GiB)")
    ap.add_argument("--skip-cpu", action="store_true", help="no CPU baseline sample")
    ap.add_argument("--skip-e2e", action="store_true", help="no end-to-end timing")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    args = ap.parse_args()
    if args.gpus > 1 and int(os.environ.get("RANK", "0")) != 0:
        return  # the path does not shard: one GPU runs, other ranks idle
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
