"""The reference's libmol2-typed entry points (include/fmftsaxs_gb300_mol2.h,
libfmftsaxs_gb300/mol2/sxs_mol2.c) driven by C programs written against the
reference's own API and header names (include/compat/):

  tests/c/correlate_caller.c  a whole scoring run the way tools/correlate.c
                              and tests/saxs_test.c do it (molecules read,
                              centred and expanded with atom_grp2spf, the
                              experiment read, Euler file to grid indices,
                              sxs_compute_saxs_scores)
  tests/c/mol2_caller.c       default_ff_table / get_ff / average radius,
                              atom_grp2spf, sxs_ft_file2euler_file

libmol2 itself is not available here: the programs link against the
stand-in of tests/c/mol2_stub.c with the types of oracle/shim/mol2 (the
headers the reference was compiled against for the checker build).

CPU tests build and link every program and check what runs without a GPU
(form factors, radius, the FT-file conversion); GPU tests run the
expansion and the scoring.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CDIR = os.path.join(ROOT, "tests", "c")
BRIDGE = os.path.join(ROOT, "libfmftsaxs_gb300", "mol2", "sxs_mol2.c")
REF_PI = 3.14159265358  # the reference's pi under -std=c11 (src/define.h:14-16)
INC = ["-I", os.path.join(ROOT, "include", "compat"), "-I", os.path.join(ROOT, "include"), "-I", CDIR, "-I",
       os.path.join(ROOT, "oracle", "shim")]


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler on this host")
    return cc


def build(lib, out_dir, prog):
    """compile the bridge, the stand-in and one caller, link with the product"""
    out_dir = str(out_dir)
    strict = ["-std=c11", "-Wall", "-Wextra", "-Werror", "-O1"]
    objs = []
    for src, pedantic in ((BRIDGE, True), (os.path.join(CDIR, "mol2_stub.c"), False)):
        o = os.path.join(out_dir, os.path.basename(src) + ".o")
        cmd = [_cc()] + strict + (["-pedantic"] if pedantic else []) + INC + ["-c", src, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(o)
    so = lib.LIB_PATH
    exe = os.path.join(out_dir, prog)
    cmd = ([_cc()] + strict + ["-pedantic"] + INC + [os.path.join(CDIR, prog + ".c")] + objs +
           ["-o", exe, "-L", os.path.dirname(so), "-l:" + os.path.basename(so), "-Wl,-rpath," + os.path.dirname(so),
            "-lm"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _names(a):
    return [bytes(r).rstrip(b"\0").decode() for r in a]


def _atom_field(name):
    return " " + name.ljust(3) if len(name) < 4 else name[:4]


def write_pdb(path, xyz, res, atom):
    with open(path, "w") as f:
        for i, (p, r, a) in enumerate(zip(xyz, res, atom)):
            f.write("ATOM  %5d %s %3s A%4d    %r %r %r\n" % (i + 1, _atom_field(a), r, i + 1, float(p[0]),
                                                              float(p[1]), float(p[2])))


def write_prm(path, res, atom, radius):
    seen = {}
    for r, a, rad in zip(res, atom, radius):
        seen[(r, a)] = rad
    with open(path, "w") as f:
        for k, ((r, a), rad) in enumerate(sorted(seen.items())):
            f.write("atom %d %s %s X %r 0.0\n" % (k + 1, r, a, float(rad)))


def write_mapping(path, g):
    with open(path, "w") as f:
        f.write("# residue atom type\n")
        for r, a, t in zip(_names(g["map_res"]), _names(g["map_atom"]), _names(g["map_type"])):
            f.write(("%s  %s  %s\n" % (r, a, t)) if t else ("%s  %s\n" % (r, a)))


def refdata():
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "ref_4g9s.npz"), allow_pickle=False))
    L, Q = int(g["spf_L"]), int(g["spf_Q"])
    g["ref_spf"] = (g["spf_mant"].astype(np.float64) * 10.0 ** g["spf_exp"].astype(np.float64)).reshape(
        Q, (L + 1) ** 2, 6)
    return g


def write_4g9s(tmp_path, g):
    res, atom = _names(g["rec_res"]), _names(g["rec_atom"])
    pdb, prm, mp = (str(tmp_path / n) for n in ("rec.pdb", "atoms.prm", "mapping.prm"))
    write_pdb(pdb, g["rec_xyz"], res, atom)
    write_prm(prm, res, atom, g["rec_vdw"])
    write_mapping(mp, g)
    return pdb, prm, mp


def test_mol2_callers_compile_and_link(lib, tmp_path):
    """Both callers build with warnings as errors against the compat headers,
    and every reference symbol they use is defined by the bridge or the
    product library."""
    have = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True,
                          check=True).stdout
    exported = {line.split()[-1] for line in have.splitlines()}
    for prog in ("correlate_caller", "mol2_caller"):
        exe = build(lib, tmp_path, prog)
        und = subprocess.run(["nm", "-u", exe], capture_output=True, text=True, check=True).stdout
        used = {line.split()[-1] for line in und.splitlines() if line.split()[-1].startswith("sxs")}
        assert "sxs_spf_full_create" in used or "sxs_mkarray" in used
        assert not (used - exported), sorted(used - exported)


def test_form_factors_and_radius_match_reference(lib, oracle, tmp_path):
    """default_ff_table + get_ff on the reference's mapping lines give, atom
    by atom, the form factors the reference's get_ff gave for the 4g9s
    receptor (tests/golden/make_refdata.py); the average radius is the
    reference's mean of the radii."""
    g = refdata()
    exe = build(lib, tmp_path, "mol2_caller")
    pdb, prm, mp = write_4g9s(tmp_path, g)
    out = str(tmp_path / "ff.txt")
    r = subprocess.run([exe, "ff", mp, prm, pdb, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    rows = open(out).read().split("\n")
    n = len(g["rec_vdw"])
    ff = np.array([[float(x) for x in rows[i].split()] for i in range(n)])
    np.testing.assert_array_equal(ff[:, 0], g["rec_vac"])
    np.testing.assert_array_equal(ff[:, 1], g["rec_dum"])
    rm, water = (float(x) for x in rows[n].split())
    assert rm == oracle.average_radius(g["rec_vdw"])
    assert round(rm, 4) == pytest.approx(float(g["spf_rm_text"]), abs=1e-4)
    assert water == float(g["h2o"])


def test_ft_file_to_euler_file_matches_oracle(lib, oracle, tmp_path):
    """sxs_ft_file2euler_file writes, line for line, the oracle's ft2euler of
    each FT line in the reference's "% .3f" format."""
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(17)
    R = synth.random_rotations(40, rng)
    T = synth.random_translations(300, 5.0, 60.0, rng)
    rid = rng.integers(0, len(R), size=len(T))
    ref = np.array([0.75, -1.25, 2.5])
    ft, rm, eu = (str(tmp_path / n) for n in ("ft.txt", "rm.txt", "euler.txt"))
    with open(ft, "w") as f:
        for k in range(len(T)):
            f.write("%d %r %r %r 0 0 0 0 0 0\n" % (rid[k], float(T[k, 0]), float(T[k, 1]), float(T[k, 2])))
    with open(rm, "w") as f:
        for m in R:
            f.write(" ".join(repr(float(x)) for x in m.reshape(9)) + "\n")
    exe = build(lib, tmp_path, "mol2_caller")
    r = subprocess.run([exe, "ft2euler", ft, rm, eu] + [repr(float(x)) for x in ref], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    got = open(eu).read().splitlines()
    assert len(got) == len(T)
    for k in range(len(T)):
        e = oracle.ft2euler(T[k], R[rid[k]].reshape(9), ref)
        want = "%d\t" % rid[k] + "\t".join("% .3f" % v for v in e)
        assert got[k] == want


@pytest.mark.gpu
def test_dropin_atom_grp2spf_matches_reference_ref_spf(gpu, oracle, tmp_path):
    """atom_grp2spf through the drop-in (4g9s receptor, L = 15, 50 q, no
    hydration shell): V and D within 1e-4 of the reference's ref_spf (its
    "% .4e" rounding is up to 5e-5) and within 1e-12 of the oracle."""
    g = refdata()
    exe = build(gpu, tmp_path, "mol2_caller")
    pdb, prm, mp = write_4g9s(tmp_path, g)
    out = str(tmp_path / "spf.txt")
    L, Q = int(g["spf_L"]), int(g["spf_Q"])
    r = subprocess.run([exe, "expand", mp, prm, pdb, out, str(L), str(Q), "0"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    with open(out) as f:
        hdr = f.readline().split()
        got = np.loadtxt(f).reshape(Q, (L + 1) ** 2, 6)
    assert int(hdr[0]) == L and int(hdr[1]) == Q
    assert float(hdr[2]) == oracle.average_radius(g["rec_vdw"])
    gold = g["ref_spf"]
    for c in range(4):
        a, b = got[:, :, c], gold[:, :, c]
        both = (np.abs(a) > 0) & (np.abs(b) > 0)
        assert (np.abs(a[both] - b[both]) / np.abs(b[both])).max() <= 1e-4
        assert np.all(np.abs(a[~both] - b[~both]) <= 1e-6)
    assert np.all(got[:, :, 4:] == 0.0)
    q = oracle.mkarray(0.0, 0.5, Q)
    want = oracle.expand(g["rec_xyz"], g["rec_vac"], g["rec_dum"], None, float(g["h2o"]), q, L)
    want = want.reshape(3, Q, (L + 1) ** 2, 2).transpose(1, 2, 0, 3).reshape(Q, (L + 1) ** 2, 6)
    scale = np.abs(want).reshape(Q, -1).max(axis=1)[:, None, None]
    assert (np.abs(got - want) / scale).max() <= 1e-12


@pytest.mark.gpu
def test_correlate_style_caller_matches_reference_fixture(gpu, tmp_path):
    """The correlate-style program on the C0 benchmark-shape fixture (1,500 /
    1,000 atoms, L = 15, 51 q, 1,354 poses): molecules, accessible areas,
    experiment and poses written as files, read back through libmol2 (the
    stand-in) and the reference's API; chi, c1, c2 of its L-BFGS-B fit
    within 1e-8 relative and 1e-6 of the reference's."""
    from libfmftsaxs_gb300 import synth
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "c0_shape.npz"), allow_pickle=False))
    L, q, z = int(g["L"]), g["q"], g["z"]
    files = {n: str(tmp_path / n) for n in ("rec.pdb", "lig.pdb", "atoms.prm", "mapping.prm", "areas_rec",
                                             "areas_lig", "exp.dat", "euler.txt", "out.txt")}
    names = {}
    for mol in ("rec", "lig"):
        el = [synth.ELEMENTS[k] for k in g[mol + "_el"]]
        res = [synth.ELEMENT_NAMES[e][0] for e in el]
        atom = [synth.ELEMENT_NAMES[e][1] for e in el]
        rad = np.array([synth.ELEMENT_RADIUS[e] for e in el])
        write_pdb(files[mol + ".pdb"], g[mol + "_xyz"], res, atom)
        area = g[mol + "_sasa"] * (4 * REF_PI * rad * rad)
        np.savetxt(files["areas_" + mol], area, fmt="%.17g")
        names[mol] = (res, atom, rad)
    write_prm(files["atoms.prm"], names["rec"][0] + names["lig"][0], names["rec"][1] + names["lig"][1],
              np.concatenate([names["rec"][2], names["lig"][2]]))
    write_mapping(files["mapping.prm"], refdata())
    np.savetxt(files["exp.dat"], np.stack([g["exp_q"], g["exp_i"], g["exp_err"]], axis=1), fmt="%.17g")
    # Euler lines that the reading of tests/saxs_test.c:291-320 turns back
    # into the fixture's grid indices
    N, nb = 2 * L + 1, L + 1
    v = g["index"].astype(np.int64)
    g2 = v % N; v //= N
    g1 = v % N; v //= N
    a2 = v % N; v //= N
    b2 = v % nb; v //= nb
    b1 = v % nb; zi = v // nb
    bs, ast = np.pi / L, 2 * np.pi / N
    with open(files["euler.txt"], "w") as f:
        for k in range(len(v)):
            e = (z[zi[k]], b1[k] * bs, g1[k] * ast, 2 * np.pi - a2[k] * ast, b2[k] * bs, 2 * np.pi - g2[k] * ast)
            f.write("%d " % k + " ".join(repr(float(x)) for x in e) + "\n")
    exe = build(gpu, tmp_path, "correlate_caller")
    out = files["out.txt"]
    cmd = [exe, files["mapping.prm"], files["atoms.prm"], files["rec.pdb"], files["lig.pdb"], files["exp.dat"],
           files["euler.txt"], out, str(L), str(len(q)), "0.5", repr(float(z[0])), repr(float(z[-1])), "1"]
    # the stand-in's accs reads the receptor's areas, then the ligand's
    both = str(tmp_path / "areas_both")
    with open(both, "w") as f:
        f.write(open(files["areas_rec"]).read() + open(files["areas_lig"]).read())
    env = dict(os.environ, SXS_TEST_ACCS=both)
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    res = np.loadtxt(out, ndmin=2)
    assert res.shape == (len(g["index"]), 4)
    np.testing.assert_array_equal(res[:, 0], np.arange(len(g["index"])))
    np.testing.assert_allclose(res[:, 1], g["chi"], rtol=1e-8, atol=0)
    np.testing.assert_allclose(res[:, 2], g["c1"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(res[:, 3], g["c2"], rtol=0, atol=1e-6)
