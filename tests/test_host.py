"""Host-side logic of the product library (no GPU needed): the reference's
C API functions that run on the host, pose ingestion, experiment binning,
form-factor lookup, text I/O, and loud failure without a GPU."""
import ctypes as C
import glob
import os

import numpy as np
import pytest

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dimer_*.npz")))


def load(path):
    return dict(np.load(path, allow_pickle=False))


def test_mkarray_and_bessel_match_oracle(lib, oracle):
    for n, e in ((50, 0.5), (101, 0.5), (201, 0.6), (2, 1.0)):
        np.testing.assert_array_equal(lib.mkarray(0.0, e, n), oracle.mkarray(0.0, e, n))
    for l in range(0, 41, 4):
        for x in (0.0, 0.01, 1.0, 7.5, 20.0, 33.0):
            assert lib.sbessel(l, x) == oracle.sbessel(l, x)


def test_pose_ingestion_matches_oracle(lib, oracle):
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(9)
    R = synth.random_rotations(3000, rng)
    T = synth.random_translations(3000, 9.5, 30.5, rng)
    z = np.arange(10.0, 31.0)
    for L in (6, 15, 20):
        idx, keep = lib.poses_to_indices(R, T, z, L)
        idx2, keep2 = synth.poses_to_indices(R, T, np.zeros(3), z, L, oracle.ft2euler, oracle.assemble_index)
        np.testing.assert_array_equal(keep, keep2)
        np.testing.assert_array_equal(idx, idx2)
    # poses whose z falls outside the translation grid are dropped
    idx, keep = lib.poses_to_indices(R[:10], T[:10] * 10, z, 6)
    assert keep.sum() == 0 and len(idx) == 0


def test_ft2euler_matches_oracle(lib, oracle):
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(3)
    R = synth.random_rotations(200, rng)
    T = synth.random_translations(200, 5, 70, rng)
    ref = np.array([0.3, -1.2, 2.2])
    for i in range(200):
        np.testing.assert_array_equal(lib.ft2euler(T[i], R[i], ref), oracle.ft2euler(T[i], R[i].reshape(9), ref))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_bin_experiment_matches_reference(lib, path):
    g = load(path)
    a, mult, peak = lib.bin_experiment(g["exp_q"], g["exp_i"], g["exp_err"], g["q"], float(g["rm"]))
    np.testing.assert_array_equal(a, g["a"])
    assert mult == float(g["mult"]) and peak == float(g["peak"])


def test_bin_experiment_stops_at_last_point(lib, oracle):
    # experimental points beyond the model grid are ignored, no read past the end
    q = lib.mkarray(0.0, 0.5, 11)
    eq = np.linspace(0.0, 0.7, 29)
    ei = 100.0 * np.exp(-eq * 4)
    ee = 0.01 * ei
    a, mult, peak = lib.bin_experiment(eq, ei, ee, q, 1.6)
    a2, mult2, peak2 = oracle.opt_params(eq, ei, ee, q, 1.6)
    np.testing.assert_array_equal(a, a2)


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_profile_from_spf_matches_oracle(lib, oracle, path):
    g = load(path)
    L = int(g["L"])
    for c1, c2 in ((1.0, 1.0), (1.03, -1.5), (0.96, 3.9)):
        i1, e1 = lib.profile_from_spf(g["A"], L, g["q"], float(g["rmA"]), c1, c2)
        i2, e2 = oracle.profile_from_spf(g["A"], L, g["q"], float(g["rmA"]), c1, c2)
        np.testing.assert_array_equal(i1, i2)
        np.testing.assert_array_equal(e1, e2)


def test_form_factor_constants(lib):
    """Per-type constants against the reference's get_ff on its own mapping
    file (captured in tests/golden/ref_4g9s.npz by make_refdata.py)."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_4g9s.npz"), allow_pickle=False))

    def names(a):
        return [bytes(r).rstrip(b"\0").decode() for r in a]

    types, res, atom = names(g["ff_types"]), names(g["ff_res"]), names(g["ff_atom"])
    for k, t in enumerate(types):
        assert lib.ff_type(t) == (g["ff_vac"][k], g["ff_dum"][k])
    assert lib.ff_water() == float(g["h2o"])
    with pytest.raises(KeyError):
        lib.ff_type("UNOBTAINIUM")
    assert len(res) == len(atom) == len(types)


def test_ff_lookup_with_written_mapping(lib, tmp_path):
    p = tmp_path / "map.prm"
    p.write_text("# comment\n\nALA  C    C\nALA  CA   CH\nALA  CA   CH3\nXYZ  Q    NOPE\n")
    v, d, missing = lib.ff_lookup(str(p), ["ALA", "ALA", " ALA", "XYZ"], ["C", "CA", " C ", "Q"])
    assert (v[0], d[0]) == lib.ff_type("C")
    assert (v[1], d[1]) == lib.ff_type("CH3")  # later lines replace earlier ones
    assert (v[2], d[2]) == lib.ff_type("C")    # names are trimmed like get_ff does
    assert missing == 1 and np.isnan(v[3])     # a type the reference does not know


def _spf_roundtrip(lib, flat, L, Q, tmp_path):
    so = lib.load()
    so.sxs_spf_full_create.restype = C.c_void_p
    so.sxs_spf_full_read.restype = C.c_void_p
    s = so.sxs_spf_full_create(C.c_int(L), C.c_int(Q))
    assert so.sxsg_spf_from_flat(C.c_void_p(s), flat.ctypes.data_as(C.POINTER(C.c_double))) == 0
    path = str(tmp_path / "spf.txt").encode()
    so.sxs_spf_full_write(C.c_char_p(path), C.c_void_p(s))
    t = so.sxs_spf_full_read(C.c_char_p(path))
    out = np.zeros_like(flat)
    assert so.sxsg_spf_to_flat(C.c_void_p(t), out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    so.sxs_spf_full_free(C.c_void_p(s))
    so.sxs_spf_full_free(C.c_void_p(t))
    return out, open(path.decode()).readline()


def test_spf_text_format_roundtrip(lib, tmp_path):
    g = load(GOLDEN[0])
    L, Q = int(g["L"]), len(g["q"])
    out, header = _spf_roundtrip(lib, np.ascontiguousarray(g["A"]), L, Q, tmp_path)
    # "% .4e" text: 5 significant digits
    np.testing.assert_allclose(out, g["A"], rtol=6e-5, atol=1e-300)
    assert header.split()[:2] == [str(L), str(Q)]


def test_plan_fails_loudly_without_gpu(lib):
    """Without a usable GPU the library reports an error; there is no
    fallback path that would compute anything on the CPU."""
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import libfmftsaxs_gb300 as g\n"
            "try:\n    g.init(0)\nexcept g.SxsError as e:\n    print('ERR', e); sys.exit(0)\n"
            "print('GPU'); sys.exit(0)\n") % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120).stdout
    assert out.startswith("ERR") or out.startswith("GPU")
    if out.startswith("ERR"):
        with pytest.raises(lib.SxsError):
            lib.expand(np.zeros((1, 3)), [1.0], [1.0], None, 1.0, [0.0, 0.1], 2)


def test_index_helpers(lib, oracle):
    eu = np.array([12.0, 0.61, 5.9, 6.2, 2.9, 0.05])
    for L in (5, 15, 20):
        assert lib.assemble_index(eu, 3, L) == oracle.assemble_index(eu, 3, L)


def _w3j_exact(j1, j2, j3, m1, m2, m3):
    """3j symbol by the Racah sum in exact rationals, square root in 60-digit
    decimals."""
    from decimal import Decimal, getcontext
    from fractions import Fraction
    from math import factorial as f
    getcontext().prec = 60
    if m1 + m2 + m3:
        return Decimal(0)
    t1, t2, t3, t4, t5 = j2 - m1 - j3, j1 + m2 - j3, j1 + j2 - j3, j1 - m1, j2 + m2
    s = sum(Fraction((-1) ** t, f(t) * f(t - t1) * f(t - t2) * f(t3 - t) * f(t4 - t) * f(t5 - t))
            for t in range(max(0, t1, t2), min(t3, t4, t5) + 1))
    pre = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1)) \
        * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3)
    v = Decimal(s.numerator) / Decimal(s.denominator) * (Decimal(pre.numerator) / Decimal(pre.denominator)).sqrt()
    return v if (j1 - j2 - m3) % 2 == 0 else -v


def test_dsymb_table_matches_oracle_and_exact_values(lib, oracle):
    """The d_lm(l1, p) table of src/fftsaxs.c:138-174 (products of 3j symbols,
    binary128 Racah sums on the host): equal to the restatement bit for bit,
    and finite and within double rounding of exact 3j values from L = 32 on,
    where the factorial prefactors (64!^6 ~ 1e530) leave the double range."""
    from decimal import Decimal
    f = lib.load().sxs_dsymb_cached
    f.restype = C.POINTER(C.c_double)
    f.argtypes = [C.c_int]
    rng = np.random.default_rng(3)
    for L in (10, 31, 32, 40):
        n = (L + 1) ** 3 * (2 * L + 1)
        tab = np.ctypeslib.as_array(f(L), shape=(n,)).copy()
        np.testing.assert_array_equal(tab, oracle.dsymb(L))
        assert np.isfinite(tab).all()
        for _ in range(12):
            l, l1 = int(rng.integers(0, L + 1)), int(rng.integers(0, L + 1))
            p = abs(l - l1) + 2 * int(rng.integers(0, min(l, l1) + 1))
            m = int(rng.integers(-min(l, l1), min(l, l1) + 1))
            ex = float(Decimal(2 * p + 1) * Decimal((2 * l1 + 1) * (2 * l + 1)).sqrt()
                       * _w3j_exact(l, p, l1, 0, 0, 0) * _w3j_exact(l, p, l1, -m, 0, m))
            got = tab[((l * (l + 1) + m) * (L + 1) + l1) * (2 * L + 1) + p]
            assert abs(got - ex) <= 2e-15 * abs(ex) + 1e-300, (L, l, m, l1, p, got, ex)


def test_pose_ingestion_wrap_option(lib):
    """SXSG_WRAP_ANGLES (opt-in) takes the alpha/gamma digits mod N; the
    default keeps the reference's unwrapped rounding, whose digit N carries
    into the next digit of the packed index."""
    from libfmftsaxs_gb300 import synth
    from libfmftsaxs_gb300.workload import decode
    rng = np.random.default_rng(12)
    R = synth.random_rotations(20000, rng)
    T = synth.random_translations(20000, 9.5, 30.5, rng)
    z = np.arange(10.0, 31.0)
    L, N = 10, 21
    raw, keep = lib.poses_to_indices(R, T, z, L)
    wrapped, keep_w = lib.poses_to_indices(R, T, z, L, wrap=True)
    np.testing.assert_array_equal(keep, keep_w)
    diff = raw != wrapped
    assert 0.01 < diff.mean() < 0.2         # alpha2 within half a step of 0 (and the like)
    for col in decode(wrapped, L)[3:]:
        assert col.min() >= 0 and col.max() < N
    # an unwrapped digit N carried into the next digit: raw - wrapped is a
    # sum of N (gamma2), N^2 (gamma1) and N^3 (alpha2)
    d = raw[diff] - wrapped[diff]
    assert np.all(d > 0) and np.all(d % N == 0)


def test_tile_table_defaults(lib):
    """The compiled-in tile table answers every (L, Q) with valid choices."""
    for L in (5, 10, 15, 20, 25, 30, 40):
        for Q in (8, 51, 101, 201, 400):
            sb, g = lib.tiles_default(L, Q)
            assert 1 <= sb <= 64
            assert g in (0, 2, 4, 6, 8, 12, 16)


def test_batch_first_fit_packing():
    """The batch's first-fit packing of translated-table chunks into arena
    phases (sxs_pack_first_fit): every chunk in one phase, within the arena,
    no two chunks of a phase overlapping, a new phase only when no earlier
    one has room."""
    import ctypes as C
    import numpy as np
    from libfmftsaxs_gb300 import load
    lib = load()
    f = lib.sxs_pack_first_fit
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p, C.POINTER(C.c_size_t)]
    f.restype = C.c_int
    rng = np.random.default_rng(5)
    for trial in range(50):
        n = int(rng.integers(1, 300))
        cap = int(rng.integers(1000, 100000))
        sizes = np.sort(rng.integers(1, cap + 1, size=n).astype(np.uint64))[::-1].copy()
        phase = np.zeros(n, dtype=np.int32)
        off = np.zeros(n, dtype=np.uint64)
        used = C.c_size_t()
        nph = f(sizes.ctypes.data, n, cap, phase.ctypes.data, off.ctypes.data, C.byref(used))
        assert 1 <= nph <= n and phase.min() >= 0 and phase.max() == nph - 1
        fill = np.zeros(nph, dtype=np.uint64)
        for ph in range(nph):
            sel = np.where(phase == ph)[0]
            iv = sorted((int(off[k]), int(off[k] + sizes[k])) for k in sel)
            assert iv[-1][1] <= cap
            assert all(a[1] <= b[0] for a, b in zip(iv, iv[1:]))
            fill[ph] = sizes[sel].sum()
        assert int(used.value) == int(fill.max())
        for k in range(n):   # no earlier phase had room when chunk k was placed
            for ph in range(phase[k]):
                placed = sizes[(phase == ph) & (np.arange(n) < k)].sum()
                assert placed + sizes[k] > cap
