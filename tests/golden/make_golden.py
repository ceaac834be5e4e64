"""Generate the golden fixtures in this directory from the reference's OWN
code: oracle/_ref/libsxsref.so, built from the reference sources by
oracle/Makefile.ref (needs the reference tree, so this runs only where it
is present).  Inputs are seeded synthetic molecules and poses
(libfmftsaxs_gb300/synth.py); every expected output comes from the
reference's functions through oracle/ref_harness.c:

  expansion     atom_grp2spf_inplace      (src/pdb2spf.c:24-152)
  experiment    sxs_profile_from_spf      (src/profile.c:186-233) + noise
  fit moments   sxs_opt_params_create     (src/min_saxs.c:108-124)
  scoring       sxs_compute_saxs_scores   (src/fftsaxs.c:608-986), with the
                raw / rescaled cross terms and point_score over the fit grid
                captured at sxs_fit_params
  L-BFGS-B      chi, c1, c2 of the reference's own fit

Two kinds of fixture:
  dimer_*.npz   small dimers (L <= 10) with every input and output stored
  c0_shape.npz, c1_shape.npz
                the benchmark shapes (C0: 1,500/1,000 atoms, L = 15, 51 q,
                every pose of two z slices of the 10,000-pose list plus a
                34-pose triple; C1: 3,500/2,000 atoms, L = 20, 101 q, every
                pose of 24 triples of the 210,000-pose list plus two crafted
                triples of 40 poses).  The molecules, experiment and pose
                lists are those of libfmftsaxs_gb300/workload.py, built here
                with the reference's functions.  Atoms are stored (a test
                expands them itself) with a seeded sample of the reference's
                A_lm; per pose: the grid fit's best chi^2 and cell, I(q) at
                that cell, the reference's L-BFGS-B chi, c1, c2; raw cross
                terms and chi^2 grids for the poses of the first triples.

Usage: FMFTSAXS_REFERENCE_SRC=<reference tree> python tests/golden/make_golden.py [names...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libfmftsaxs_gb300 import synth  # noqa: E402
from oracle.bind import Ref, REF_SRC, have_ref_src  # noqa: E402

MAP = os.path.join(REF_SRC, "prms", "pdb_formfactor_mapping_clean.prm")
ELEMENT_CODE = {e: i for i, e in enumerate(synth.ELEMENTS)}


def molecule_pair(nr, na, rgr, rga, seed):
    rec = synth.make_molecule(nr, rgr, seed)
    lig = synth.make_molecule(na, rga, seed + 1)
    rec = rec.translated(-rec.center_of_extrema()).with_sasa()
    lig = lig.translated(-lig.centroid()).with_sasa()
    return rec, lig


def crafted_triple(L, z, b1, b2, n, rng):
    """n distinct cells of one (z, b1, b2) triple (so it takes the FFTW branch
    when n >= 30)."""
    N, nb = 2 * L + 1, L + 1
    cells = rng.choice(N ** 3, size=n, replace=False)
    a2, g1, g2 = cells // (N * N), (cells // N) % N, cells % N
    return ((((z * nb + b1) * nb + b2) * N + a2) * N + g1) * N + g2


def make_case(r, name, L, Q, nr, na, npose, skip, seed, crafted=(), grid_rows=48):
    rng = np.random.default_rng(seed)
    rec, lig = molecule_pair(nr, na, 9.0, 8.0, seed)
    q = r.mkarray(0.0, 0.5, Q)
    A, rmA = r.expand(rec.xyz, rec.res, rec.atom, rec.radius, rec.sasa, MAP, q, L)
    B, rmB = r.expand(lig.xyz, lig.res, lig.atom, lig.radius, lig.sasa, MAP, q, L)
    A0, _ = r.expand(rec.xyz, rec.res, rec.atom, rec.radius, None, MAP, q, L)
    rm = (rmA * rec.natoms + rmB * lig.natoms) / (rec.natoms + lig.natoms)
    Rn = synth.random_rotations(1, rng)[0]
    Tn = synth.random_translations(1, 12, 18, rng)[0]
    cplx = synth.join(rec, synth.Molecule(lig.xyz @ Rn.T + Tn, lig.elements))
    cplx = cplx.translated(-cplx.centroid()).with_sasa()
    C, rmC = r.expand(cplx.xyz, cplx.res, cplx.atom, cplx.radius, cplx.sasa, MAP, q, L)
    I, _ = r.profile_from_spf(C, L, q, rmC, 1.0, 1.0)
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = r.opt_params(eq, ei, ee, q, rm)
    z = np.arange(10.0, 21.0)
    R = synth.random_rotations(npose, rng)
    T = synth.random_translations(npose, 10.0, 20.0, rng)
    idx, _ = synth.poses_to_indices(R, T, np.zeros(3), z, L, r.ft2euler, _assemble(L))
    extra = [crafted_triple(L, *c, rng) for c in crafted]
    N, nb = 2 * L + 1, L + 1
    edge = np.array([((((0 * nb + L) * nb + L) * N + N - 1) * N + N - 1) * N + N - 1,
                     (((((len(z) - 1) * nb + 0) * nb + L) * N + 0) * N + N - 1) * N + N - 1],
                    dtype=np.int64)
    idx = np.concatenate([np.asarray(idx, dtype=np.int64)] + extra + [edge, idx[:3]]).astype(np.int32)
    c1g, c2g = synth.C1_GRID, synth.C2_GRID
    res = r.score(A, B, rmA, rmB, rm, (eq, ei, ee), q, z, L, idx, skip, c1g, c2g)
    rv, rd, h2o, _ = r.ff_lookup(MAP, rec.res, rec.atom)
    lv, ld, _, _ = r.ff_lookup(MAP, lig.res, lig.atom)
    out = dict(L=L, q=q, z=z, skip=skip, index=idx, A=A, B=B, A_nowater=A0, rmA=rmA, rmB=rmB, rm=rm,
               rec_vac=rv, rec_dum=rd, lig_vac=lv, lig_dum=ld, h2o=h2o, rec_radius=rec.radius,
               lig_radius=lig.radius,
               rec_xyz=rec.xyz, rec_el=np.array(rec.elements), rec_sasa=rec.sasa,
               lig_xyz=lig.xyz, lig_el=np.array(lig.elements), lig_sasa=lig.sasa,
               exp_q=eq, exp_i=ei, exp_err=ee, a=a, mult=mult, peak=peak, c1g=c1g, c2g=c2g,
               raw=res["raw"], scaled=res["scaled"], chi=res["chi"], c1=res["c1"], c2=res["c2"],
               branch=res["branch"], grid=res["grid"][:grid_rows], grid_rows=grid_rows)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "poses", len(idx), "fftw-branch poses", int(res["branch"].sum()))


def _assemble(L):
    from oracle.bind import Oracle
    o = Oracle()
    return o.assemble_index


def _ref_to_indices(r):
    from oracle.bind import Oracle
    o = Oracle()
    return lambda R, T, z, L: synth.poses_to_indices(R, T, np.zeros(3), z, L, r.ft2euler, o.assemble_index)


def _decode(idx, L):
    N, nb = 2 * L + 1, L + 1
    v = np.asarray(idx, dtype=np.int64)
    return v // (nb * nb * N ** 3), (v // (nb * N ** 3)) % nb, (v // N ** 3) % nb


def _crafted_in(L, z_idx, rng, n, taken):
    """n distinct cells of one (z, b1, b2) triple that the list leaves empty"""
    nb = L + 1
    while True:
        b1, b2 = int(rng.integers(0, nb)), int(rng.integers(0, nb))
        if (z_idx, b1, b2) not in taken:
            taken.add((z_idx, b1, b2))
            return crafted_triple(L, z_idx, b1, b2, n, rng)


def make_shape_case(name, cfg_name, z_pick, ntriples, crafted, seed=2026, nsample=4096, ndetail=3):
    """Benchmark-shape fixture; see the module docstring."""
    from libfmftsaxs_gb300 import workload
    from oracle.bind import Oracle
    r = Ref()
    o = Oracle()
    cfg = workload.config(cfg_name)
    L, Q = cfg["L"], cfg["Q"]
    q = r.mkarray(0.0, cfg["qmax"], Q)
    rec, lig = workload.molecules(cfg, seed)
    A, rmA = r.expand(rec.xyz, rec.res, rec.atom, rec.radius, rec.sasa, MAP, q, L)
    B, rmB = r.expand(lig.xyz, lig.res, lig.atom, lig.radius, lig.sasa, MAP, q, L)
    rm = (rmA * rec.natoms + rmB * lig.natoms) / (rec.natoms + lig.natoms)
    native, rng = workload.native_complex(rec, lig, cfg, seed)
    C, rmC = r.expand(native.xyz, native.res, native.atom, native.radius, native.sasa, MAP, q, L)
    I, _ = r.profile_from_spf(C, L, q, rmC, 1.0, 1.0)
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = r.opt_params(eq, ei, ee, q, rm)
    z = workload.zvals(cfg)
    full = workload.pose_lists(cfg, seed, _ref_to_indices(r), z, L)
    zi, b1, b2 = _decode(full, L)
    sel = np.random.default_rng(seed + 5)
    if ntriples is None:
        idx = full[np.isin(zi, z_pick)]
    else:
        # ntriples whole triples of the list at the picked z values, drawn
        # among those the reference scores with its simple_ft branch
        key = (zi * (L + 1) + b1) * (L + 1) + b2
        u, cnt = np.unique(key[np.isin(zi, z_pick)], return_counts=True)
        u = u[cnt < 30]
        chosen = sel.choice(u, size=ntriples, replace=False)
        idx = np.concatenate([full[key == k] for k in chosen])
    taken = set(zip(*[x.tolist() for x in _decode(idx, L)]))
    extra = [_crafted_in(L, int(z_pick[k % len(z_pick)]), sel, n, taken) for k, n in enumerate(crafted)]
    idx = np.concatenate([idx] + extra).astype(np.int32)
    c1g, c2g = synth.C1_GRID, synth.C2_GRID
    res = r.score(A, B, rmA, rmB, rm, (eq, ei, ee), q, z, L, idx, 1, c1g, c2g)
    grid = res["grid"].reshape(len(idx), -1)
    cell = grid.argmin(axis=1)
    best = grid[np.arange(len(idx)), cell]
    iq = np.array([o.compile_intensity(res["scaled"][i].reshape(-1), q, rm, c1g[cell[i] // len(c2g)],
                                       c2g[cell[i] % len(c2g)])[0] for i in range(len(idx))])
    # detail rows: every pose of the first ndetail triples (in list order)
    trip = (_decode(idx, L)[0] * (L + 1) + _decode(idx, L)[1]) * (L + 1) + _decode(idx, L)[2]
    first = list(dict.fromkeys(trip.tolist()))[:ndetail]
    detail = np.nonzero(np.isin(trip, first))[0]
    rs = np.random.default_rng(seed + 9)
    sa = np.sort(rs.choice(A.size, size=nsample, replace=False))
    sb = np.sort(rs.choice(B.size, size=nsample, replace=False))
    rv, rd, h2o, _ = r.ff_lookup(MAP, rec.res, rec.atom)
    lv, ld, _, _ = r.ff_lookup(MAP, lig.res, lig.atom)
    out = dict(L=L, q=q, z=z, skip=1, index=idx, config=cfg_name,
               rec_xyz=rec.xyz, rec_el=np.array([ELEMENT_CODE[e] for e in rec.elements], dtype=np.uint8),
               rec_sasa=rec.sasa, rec_vac=rv, rec_dum=rd,
               lig_xyz=lig.xyz, lig_el=np.array([ELEMENT_CODE[e] for e in lig.elements], dtype=np.uint8),
               lig_sasa=lig.sasa, lig_vac=lv, lig_dum=ld, h2o=h2o, rmA=rmA, rmB=rmB, rm=rm,
               A_at=sa.astype(np.int32), A_val=A[sa], B_at=sb.astype(np.int32), B_val=B[sb],
               exp_q=eq, exp_i=ei, exp_err=ee, a=a, mult=mult, peak=peak, c1g=c1g, c2g=c2g,
               best=best, cell=cell.astype(np.int16), iq=iq, chi=res["chi"], c1=res["c1"], c2=res["c2"],
               branch=res["branch"].astype(np.uint8), detail=detail.astype(np.int32),
               raw=res["raw"][detail], grid=res["grid"][detail])
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(name, "poses", len(idx), "fftw-branch poses", int(res["branch"].sum()), "detail", len(detail),
          "bytes", os.path.getsize(path))


CASES = {
    "dimer_l6": lambda: make_case(Ref(), "dimer_l6", L=6, Q=10, nr=120, na=80, npose=220, skip=1, seed=101,
                                  crafted=((3, 2, 4, 34), (7, 5, 1, 30))),
    "dimer_l3_skip0": lambda: make_case(Ref(), "dimer_l3_skip0", L=3, Q=6, nr=40, na=30, npose=40, skip=0,
                                        seed=202),
    "dimer_l10": lambda: make_case(Ref(), "dimer_l10", L=10, Q=16, nr=200, na=150, npose=150, skip=1, seed=303,
                                   crafted=((2, 3, 7, 31),), grid_rows=24),
    # C0: every pose of z = 30 and z = 36 (slots 5 and 11), one 34-pose triple
    "c0_shape": lambda: make_shape_case("c0_shape", "c0", z_pick=(5, 11), ntriples=None, crafted=(34,)),
    # C1: 24 triples of the list at z = 35 and z = 44 (slots 5 and 14), two 40-pose triples
    "c1_shape": lambda: make_shape_case("c1_shape", "c1", z_pick=(5, 14), ntriples=24, crafted=(40, 40)),
}


def _run(name):
    CASES[name]()
    return name


def main(names):
    if not have_ref_src():
        sys.exit("set FMFTSAXS_REFERENCE_SRC to the reference source tree")
    Ref()  # build the checker once before the workers load it
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(len(names), 4)) as pool:
        for n in pool.imap_unordered(_run, names):
            print("done", n)


if __name__ == "__main__":
    main(sys.argv[1:] or list(CASES))
