"""Capture the reference project's own test data (its tests/data and prms
directories) as a compact fixture, ref_4g9s.npz, so that the checks built on
it run where the reference tree is absent.

  4g9s receptor   atoms of tests/data/4g9s_r_native.pdb centred at their
                  centre of extrema as tests/saxs_test.c:59-73 does, their
                  van der Waals radii (tests/data/atoms.0.0.6.prm...) and
                  zero-angle form factors (the reference's get_ff through
                  oracle/_ref, with its mapping file)
  ref_spf         tests/data/ref_spf, the reference's A_lm of that receptor
                  (L = 15, 50 q, "% .4e"), stored as exact decimal mantissa and
                  exponent
  form factors    (vacuum, excluded volume) of the mapping's types C, N, O, S,
                  CH, CH2, CH3, H and of water, from the reference's get_ff
  mapping         the (residue, atom, type) lines of the mapping file, so a
                  test can write the same file for the drop-in default_ff_table

Usage: FMFTSAXS_REFERENCE_SRC=<reference tree> python tests/golden/make_refdata.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.bind import Ref, REF_SRC, have_ref_src  # noqa: E402

# (residue, atom) pairs of the mapping file that resolve to each type
FF_PAIRS = {"C": ("ALA", "C"), "N": ("ALA", "N"), "O": ("ALA", "O"), "S": ("MET", "SD"), "CH": ("ALA", "CA"),
            "CH3": ("ALA", "CB"), "CH2": ("ARG", "CB"), "H": ("ALA", "H")}


def read_pdb(path):
    xyz, res, atom = [], [], []
    with open(path) as f:
        for line in f:
            if line.startswith(("ATOM", "HETATM")):
                atom.append(line[12:16].strip())
                res.append(line[17:21].strip())
                xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    return np.array(xyz), res, atom


def read_prm_radii(path):
    rad = {}
    with open(path) as f:
        for line in f:
            p = line.split()
            if len(p) >= 7 and p[0] == "atom":
                rad[(p[2], p[3])] = float(p[5])
    return rad


def decimal_parts(tokens):
    """'% .4e' strings -> (mantissa * 1e4 as int32, exponent - 4 as int8):
    value = m * 10**e exactly in decimal"""
    m = np.empty(len(tokens), dtype=np.int32)
    e = np.empty(len(tokens), dtype=np.int8)
    for i, t in enumerate(tokens):
        mant, ex = t.lower().split("e")
        neg = mant.startswith("-")
        ip, fp = mant.lstrip("+-").split(".")
        v = int(ip + fp)
        m[i] = -v if neg else v
        e[i] = int(ex) - len(fp)
    return m, e


def names8(names):
    buf = np.zeros((len(names), 8), dtype=np.uint8)
    for i, s in enumerate(names):
        b = s.encode()[:7]
        buf[i, :len(b)] = np.frombuffer(b, dtype=np.uint8)
    return buf


def main():
    if not have_ref_src():
        sys.exit("set FMFTSAXS_REFERENCE_SRC to the reference source tree")
    data = os.path.join(REF_SRC, "tests", "data")
    mapping = os.path.join(data, "pdb_formfactor_mapping_clean.prm")
    r = Ref()
    xyz, res, atom = read_pdb(os.path.join(data, "4g9s_r_native.pdb"))
    rad = read_prm_radii(os.path.join(data, "atoms.0.0.6.prm.ms.3cap+0.5ace.Hr0rec"))
    vdw = np.array([rad[(a, b)] for a, b in zip(res, atom)])
    xyz = xyz - 0.5 * (xyz.min(0) + xyz.max(0))
    vac, dum, h2o, bad = r.ff_lookup(mapping, res, atom)
    assert bad == 0
    with open(os.path.join(data, "ref_spf")) as f:
        hdr = f.readline().split()
        toks = f.read().split()
    L, Q = int(hdr[0]), int(hdr[1])
    assert len(toks) == Q * (L + 1) ** 2 * 6
    m, e = decimal_parts(toks)
    mres, matom, mtype = [], [], []
    with open(mapping) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            p = line.split()
            mres.append(p[0])
            matom.append(p[1])
            mtype.append(p[2] if len(p) > 2 else "")
    ff_types = list(FF_PAIRS)
    ffv, ffd, _, _ = r.ff_lookup(mapping, [FF_PAIRS[t][0] for t in ff_types], [FF_PAIRS[t][1] for t in ff_types])
    out = dict(rec_xyz=xyz, rec_res=names8(res), rec_atom=names8(atom), rec_vdw=vdw, rec_vac=vac, rec_dum=dum,
               h2o=h2o, spf_L=L, spf_Q=Q, spf_rm_text=float(hdr[2]), spf_mant=m, spf_exp=e,
               ff_types=names8(ff_types), ff_res=names8([FF_PAIRS[t][0] for t in ff_types]),
               ff_atom=names8([FF_PAIRS[t][1] for t in ff_types]), ff_vac=ffv, ff_dum=ffd,
               map_res=names8(mres), map_atom=names8(matom), map_type=names8(mtype))
    path = os.path.join(HERE, "ref_4g9s.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes,", len(vdw), "atoms")


if __name__ == "__main__":
    main()
