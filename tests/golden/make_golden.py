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

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libfmftsaxs_gb300 import synth  # noqa: E402
from oracle.bind import Ref, REF_SRC  # noqa: E402

MAP = os.path.join(REF_SRC, "prms", "pdb_formfactor_mapping_clean.prm")


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


def main():
    r = Ref()
    make_case(r, "dimer_l6", L=6, Q=10, nr=120, na=80, npose=220, skip=1, seed=101,
              crafted=((3, 2, 4, 34), (7, 5, 1, 30)))
    make_case(r, "dimer_l3_skip0", L=3, Q=6, nr=40, na=30, npose=40, skip=0, seed=202)
    make_case(r, "dimer_l10", L=10, Q=16, nr=200, na=150, npose=150, skip=1, seed=303, crafted=((2, 3, 7, 31),),
              grid_rows=24)


if __name__ == "__main__":
    main()
