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
