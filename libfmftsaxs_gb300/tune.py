"""Autotuner of the mixed path's tile choices per (L, Q).

For every (L, Q) of the batched and serving workloads (L in {10, 15, 20, 25,
30}, Q in {51, 101, 201}) it builds a seeded dimer (receptor 1,500 atoms,
ligand 800, 40,000 poses with |t| in [25, 45] A), times on the GPU the
stages the choices affect, and keeps the fastest:

  tr_slices  slices of combos per block of the pipelined translation
             (k_translate_pipe): 2, 4, 8, 16; timed by the translation stage
  rot_gamma  gamma pairs per thread of the rotation (k_rotate): every
             instantiated group size that covers L + 1; timed by the table
             stage

Each candidate is run once to warm up and then three times; the median of
the stage's CUDA-event time decides.  Results never depend on the choice.
Output: a C header with the table (csrc/tiles_table.h, compiled into the
library) and a JSON file with every timing.

Usage: python -m libfmftsaxs_gb300.tune [header_path] [json_path]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LS = (10, 15, 20, 25, 30)
QS = (51, 101, 201)
GROUPS = (2, 4, 6, 8, 12, 16)
ROT_GROUPS = 4   # gamma-pair groups of a rotation block (kernels_contract.cu)


def job(g, L, Q, seed):
    from . import synth
    rng = np.random.default_rng(seed)
    rec = synth.make_molecule(1500, 16.0, seed).with_sasa()
    lig = synth.make_molecule(800, 12.0, seed + 1).with_sasa()
    rec = rec.translated(-rec.center_of_extrema())
    lig = lig.translated(-lig.centroid())
    q = g.mkarray(0.0, 0.5, Q)
    ff = lambda m: np.array([g.ff_type(e) for e in m.elements])
    fr, fl = ff(rec), ff(lig)
    A = g.expand(rec.xyz, fr[:, 0], fr[:, 1], rec.sasa, g.ff_water(), q, L)
    B = g.expand(lig.xyz, fl[:, 0], fl[:, 1], lig.sasa, g.ff_water(), q, L)
    I, _ = g.profile_from_spf(A, L, q, 1.7, 1.0, 1.0)
    eq, ei, ee = synth.noisy_experiment(q, I, 0.01, rng)
    a, mult, peak = g.bin_experiment(eq, ei, ee, q, 1.7)
    z = np.arange(25.0, 46.0)
    R = synth.random_rotations(40000, rng)
    T = synth.random_translations(40000, 25.0, 45.0, rng)
    idx, _ = g.poses_to_indices(R, T, z, L)
    return A, B, q, z, a, mult, peak, idx


def stage_ms(g, plan, key, reps=3):
    plan.run(g.FIT_NONE)
    t = []
    for _ in range(reps):
        plan.run(g.FIT_NONE)
        t.append(plan.timings()[key])
    return float(np.median(t))


def tune(g, L, Q):
    A, B, q, z, a, mult, peak, idx = job(g, L, Q, 500 + L + Q)
    p = g.Plan(A, B, q, z, L, a, mult, peak, precision=g.MIXED)
    p.set_poses(idx, skip=1)
    need = (L + 1 + ROT_GROUPS - 1) // ROT_GROUPS
    gs = [x for x in GROUPS if x >= need]
    tr = {}
    for sb in (2, 4, 8, 16):
        p.set_tiles(sb, gs[0])
        tr[sb] = stage_ms(g, p, "translate")
    best_sb = min(tr, key=tr.get)
    rot = {}
    for gg in gs:
        p.set_tiles(best_sb, gg)
        rot[gg] = stage_ms(g, p, "tables")
    best_g = min(rot, key=rot.get)
    p.close()
    return {"L": L, "Q": Q, "tr_slices": best_sb, "rot_gamma": best_g, "translate_ms": tr, "tables_ms": rot,
            "poses": int(len(idx))}


def write_header(path, rows):
    with open(path, "w") as f:
        f.write("/*\n * Tile choices per (L, Q) for the mixed-precision path: slices of combos\n"
                " * per block of the pipelined translation and gamma pairs per thread of the\n"
                " * rotation (0 = the fewest that cover L + 1).  Written by\n"
                " * libfmftsaxs_gb300/tune.py from timings on a GB300; a plan takes the entry\n"
                " * of the nearest L, then the nearest Q.\n */\n")
        f.write("#ifndef SXS_TILES_TABLE_H\n#define SXS_TILES_TABLE_H\n")
        f.write("static const struct { int L, Q, tr_slices, rot_gamma; } sxs_tiles_table[] = {\n")
        for r in rows:
            f.write("\t{%d, %d, %d, %d},\n" % (r["L"], r["Q"], r["tr_slices"], r["rot_gamma"]))
        f.write("};\n#endif\n")


def main(argv):
    import libfmftsaxs_gb300 as g
    header = argv[0] if argv else os.path.join(HERE, "csrc", "tiles_table.h")
    out_json = argv[1] if len(argv) > 1 else os.path.join(HERE, "tiles_table.json")
    g.init(0)
    rows = []
    for L in LS:
        for Q in QS:
            r = tune(g, L, Q)
            rows.append(r)
            print(json.dumps(r), flush=True)
    write_header(header, rows)
    with open(out_json, "w") as f:
        json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:])
