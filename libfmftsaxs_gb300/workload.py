"""Seeded synthetic dimer-scoring workloads with the shapes of the benchmark
configurations, built through the library (GPU expansion, C pose
ingestion).  See synth.py for how molecules, accessible fractions and poses
are generated.

  c0  receptor 1,500 atoms (Rg 16 A), ligand 1,000 (Rg 14 A), L = 15,
      51 q on [0, 0.5], 10,000 poses with |t| in [25, 40] A
  c1  receptor 3,500 atoms (Rg 21 A), ligand 2,000 (Rg 17 A), L = 20,
      101 q on [0, 0.5], 210,000 poses in three seeded lists of 70,000,
      |t| in [30, 50] A
  c2  receptor 8,000 (Rg 28 A), ligand 4,000 (Rg 22 A), L = 30, 201 q on
      [0, 0.6], 1,000,000 poses, |t| in [40, 65] A

The "experiment" is the single-molecule intensity (sxs_profile_from_spf at
c1 = c2 = 1) of a seeded native pose of the joined complex, with 1 %
multiplicative Gaussian noise and sigma = 0.01 I.  It stays in memory at
full precision.  The fit grid is c1 in [0.95, 1.05] step 0.01 and c2 in
[0, 4] step 0.1.
"""
import numpy as np

from . import synth

CONFIGS = {
    "c0": dict(rec=(1500, 16.0), lig=(1000, 14.0), L=15, Q=51, qmax=0.5, lists=(10000,), t=(25.0, 40.0)),
    "c1": dict(rec=(3500, 21.0), lig=(2000, 17.0), L=20, Q=101, qmax=0.5, lists=(70000, 70000, 70000),
               t=(30.0, 50.0)),
    "c2": dict(rec=(8000, 28.0), lig=(4000, 22.0), L=30, Q=201, qmax=0.6, lists=(1000000,), t=(40.0, 65.0)),
}


def form_factors(lib, mol):
    vac = np.array([lib.ff_type(e)[0] for e in mol.elements])
    dum = np.array([lib.ff_type(e)[1] for e in mol.elements])
    return vac, dum


class Workload:
    pass


def config(name="c1", overrides=None):
    """The configuration dict of a named workload, with optional changes."""
    cfg = dict(CONFIGS[name])
    if overrides:
        cfg.update(overrides)
    return cfg


def molecules(cfg, seed=2026):
    """Receptor (centred at its centre of extrema) and ligand (centred at its
    centroid) of a configuration, with their accessible fractions."""
    rec = synth.make_molecule(cfg["rec"][0], cfg["rec"][1], seed)
    lig = synth.make_molecule(cfg["lig"][0], cfg["lig"][1], seed + 1)
    rec = rec.translated(-rec.center_of_extrema()).with_sasa()
    lig = lig.translated(-lig.centroid()).with_sasa()
    return rec, lig


def native_complex(rec, lig, cfg, seed=2026):
    """The seeded native pose of the joined complex (centred at its centroid,
    with accessible fractions) and the generator that then draws the
    experiment's noise."""
    rng = np.random.default_rng(seed + 7)
    Rn = synth.random_rotations(1, rng)[0]
    Tn = synth.random_translations(1, cfg["t"][0], cfg["t"][1], rng)[0]
    native = synth.join(rec, synth.Molecule(lig.xyz @ Rn.T + Tn, lig.elements))
    native = native.translated(-native.centroid()).with_sasa()
    return native, rng


def zvals(cfg):
    """Translation grid: integer z covering the configuration's |t| range."""
    t = cfg["t"]
    return np.arange(np.floor(t[0]), np.ceil(t[1]) + 1.0)


def pose_lists(cfg, seed, to_indices, z, L):
    """Packed grid indices of the configuration's seeded pose lists, in list
    order; to_indices(R, T, z, L) -> (index, keep) converts one list."""
    idx = []
    for k, n in enumerate(cfg["lists"]):
        r = np.random.default_rng(seed + 100 + k)
        R = synth.random_rotations(n, r)
        T = synth.random_translations(n, cfg["t"][0], cfg["t"][1], r)
        ii, keep = to_indices(R, T, z, L)
        idx.append(np.asarray(ii, dtype=np.int64))
    return np.concatenate(idx)


def build(name="c1", seed=2026, lib=None, expand=None, profile=None, to_indices=None, overrides=None):
    """Assemble a workload.  `lib` is the libfmftsaxs_gb300 module; the
    callables default to it (expansion on the GPU, profile and pose
    conversion in its host C)."""
    if lib is None:
        import importlib
        lib = importlib.import_module(__package__)
    cfg = config(name, overrides)
    expand = expand or lib.expand
    profile = profile or lib.profile_from_spf
    to_indices = to_indices or (lambda R, T, z, L: lib.poses_to_indices(R, T, z, L))
    L, Q = cfg["L"], cfg["Q"]
    w = Workload()
    w.name, w.L, w.Q = name, L, Q
    w.q = lib.mkarray(0.0, cfg["qmax"], Q)
    rec, lig = molecules(cfg, seed)
    water = lib.ff_water()
    vr, dr = form_factors(lib, rec)
    vl, dl = form_factors(lib, lig)
    w.A = expand(rec.xyz, vr, dr, rec.sasa, water, w.q, L)
    w.B = expand(lig.xyz, vl, dl, lig.sasa, water, w.q, L)
    w.rmA, w.rmB = float(np.mean(rec.radius)), float(np.mean(lig.radius))
    w.rm = (w.rmA * rec.natoms + w.rmB * lig.natoms) / (rec.natoms + lig.natoms)
    w.rec, w.lig = rec, lig
    # native pose and its noisy single-molecule profile
    native, rng = native_complex(rec, lig, cfg, seed)
    vn, dn = form_factors(lib, native)
    C = expand(native.xyz, vn, dn, native.sasa, water, w.q, L)
    rmC = float(np.mean(native.radius))
    I, _ = profile(C, L, w.q, rmC, 1.0, 1.0)
    w.exp = synth.noisy_experiment(w.q, I, 0.01, rng)
    w.a, w.mult, w.peak = lib.bin_experiment(w.exp[0], w.exp[1], w.exp[2], w.q, w.rm)
    # poses
    w.z = zvals(cfg)
    w.index = pose_lists(cfg, seed, to_indices, w.z, L)
    w.c1g, w.c2g = synth.C1_GRID, synth.C2_GRID
    return w


def decode(index, L):
    """(z, b1, b2, a2, g1, g2) columns of packed grid indices."""
    N, nb = 2 * L + 1, L + 1
    v = np.asarray(index, dtype=np.int64).copy()
    g2 = v % N; v //= N
    g1 = v % N; v //= N
    a2 = v % N; v //= N
    b2 = v % nb; v //= nb
    b1 = v % nb; v //= nb
    return v, b1, b2, a2, g1, g2


def triple_counts(index, L):
    z, b1, b2 = decode(index, L)[:3]
    nb = L + 1
    key = (z * nb + b1) * nb + b2
    u, c = np.unique(key, return_counts=True)
    return u, c


def batch_specs(n=64, seed=2026, min_poses=1000, max_poses=200000, pool=16):
    """Sizes of the batched workload of many uneven dimers.  A pool of
    `pool` receptors (atoms log-uniform in [500, 8000]) and `pool` ligands
    (in [300, 5000]), Rg of a compact protein of na / 8 residues, is drawn
    first; each dimer pairs one of each with L uniform in {10, 15, 20, 25,
    30}, Q in {51, 101, 201} on [0, 0.5], a pose count log-uniform in
    [min_poses, max_poses] with |t| in [25, 45] A, and the (c1, c2) of its
    experiment uniform in [0.97, 1.03] x [0, 3].  Returns (dimers, receptor
    pool, ligand pool); a pool entry is (atoms, Rg, seed)."""
    rng = np.random.default_rng(seed)

    def mol(lo, hi, k):
        na = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        return (na, 2.2 * (na / 8.0) ** 0.38, seed + 7919 * (k + 1))
    recs = [mol(500, 8000, k) for k in range(pool)]
    ligs = [mol(300, 5000, pool + k) for k in range(pool)]
    out = []
    for i in range(n):
        out.append(dict(rec=int(rng.integers(pool)), lig=int(rng.integers(pool)),
                        L=int(rng.choice((10, 15, 20, 25, 30))), Q=int(rng.choice((51, 101, 201))), qmax=0.5,
                        npose=int(np.exp(rng.uniform(np.log(min_poses), np.log(max_poses)))), t=(25.0, 45.0),
                        c1=float(rng.uniform(0.97, 1.03)), c2=float(rng.uniform(0.0, 3.0)), seed=seed + 1000 * (i + 1)))
    return out, recs, ligs


def _pool_molecule(entry):
    na, rg, seed = entry
    m = synth.make_molecule(na, rg, seed)
    return m.xyz, m.elements


def pool_molecules(entries, workers=1):
    """The molecules of pool entries (atoms, Rg, seed), built in `workers`
    spawned processes (the random walks are the slow part)."""
    if workers <= 1 or len(entries) <= 1:
        res = [_pool_molecule(e) for e in entries]
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(workers, len(entries))) as pool:
            res = pool.map(_pool_molecule, entries)
    return [synth.Molecule(x, el) for x, el in res]


def build_dimer(spec, rec, lig, lib=None):
    """One dimer of batch_specs from its pool molecules: accessible
    fractions and expansions on the GPU, the noisy profile of a seeded native
    pose at the spec's (c1, c2), poses ingested on the GPU."""
    if lib is None:
        import importlib
        lib = importlib.import_module(__package__)
    cfg = dict(spec, lists=(spec["npose"],))
    L, Q, seed = spec["L"], spec["Q"], spec["seed"]
    w = Workload()
    w.L, w.Q = L, Q
    w.q = lib.mkarray(0.0, cfg["qmax"], Q)
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    rec.sasa = lib.sasa(rec.xyz, rec.radius)
    lig.sasa = lib.sasa(lig.xyz, lig.radius)
    water = lib.ff_water()
    w.A = lib.expand(rec.xyz, *form_factors(lib, rec), rec.sasa, water, w.q, L)
    w.B = lib.expand(lig.xyz, *form_factors(lib, lig), lig.sasa, water, w.q, L)
    r = np.random.default_rng(seed + 7)
    Rn = synth.random_rotations(1, r)[0]
    Tn = synth.random_translations(1, cfg["t"][0], cfg["t"][1], r)[0]
    native = synth.join(rec, synth.Molecule(lig.xyz @ Rn.T + Tn, lig.elements))
    native = native.translated(-native.centroid())
    native.sasa = lib.sasa(native.xyz, native.radius)
    C = lib.expand(native.xyz, *form_factors(lib, native), native.sasa, water, w.q, L)
    rm = float(np.mean(native.radius))
    I, _ = lib.profile_from_spf(C, L, w.q, rm, spec["c1"], spec["c2"])
    w.exp = synth.noisy_experiment(w.q, I, 0.01, r)
    w.a, w.mult, w.peak = lib.bin_experiment(w.exp[0], w.exp[1], w.exp[2], w.q, rm)
    w.z = zvals(cfg)
    w.index = pose_lists(cfg, seed, lambda R, T, z, L: lib.poses_to_indices_gpu(R, T, z, L)[:2], w.z, L)
    w.c1g, w.c2g = synth.C1_GRID, synth.C2_GRID
    w.natoms = (rec.natoms, lig.natoms)
    return w


def plan_bytes(L, Q, npose, nz):
    """Device bytes of a mixed-precision plan of this size with its pose list
    set (rotation tables, per-z tables, outputs), for packing dimers into
    device memory."""
    K, N, NT = L + 1, 2 * L + 1, (Q + 7) // 8
    NP = K * (K + 1) // 2
    rot = 2 * NT * K * N * NP * 3 * 8 * 8
    tau = NT * nz * K ** 3 * 8 * 12 + nz * Q * N * 8
    out = npose * (6 * Q * 8 + 4 * 8 + 8 + 32 + 8)
    return rot + tau + out + 64 * Q * K * K
