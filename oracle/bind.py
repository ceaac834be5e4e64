"""ctypes bindings for the CPU oracle (liboracle.so, a C restatement of the
reference path) and, when it was built here, the checker library
oracle/_ref/libsxsref.so (the reference's own sources compiled against the
shims in oracle/shim/).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module, and only as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsxsref.so")
# Root of the reference project's source tree (read-only), given by the
# environment; without it the checker library is only loaded if an earlier
# build left it in oracle/_ref/.
REF_SRC = os.environ.get("FMFTSAXS_REFERENCE_SRC", "")


def have_ref_src():
    """Whether the reference sources are available to build the checker."""
    return bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "src"))


def have_ref():
    """Whether the checker library exists or can be built."""
    return have_ref_src() or os.path.exists(REF_SO)


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_oracle(force=False):
    """Compile the restatement (gcc, -std=c11, no multiply-add fusion)."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-shared",
                               src, "-o", ORACLE_SO, "-lm"])
    return ORACLE_SO


def build_ref():
    """Compile the reference's own sources with the shims (needs the
    reference tree); without it, return an earlier build if there is one."""
    if not have_ref_src():
        return REF_SO if os.path.exists(REF_SO) else None
    subprocess.check_call(["make", "-s", "-f", "Makefile.ref", "REF=" + REF_SRC], cwd=HERE)
    return REF_SO


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """The C restatement.  Arrays use the flat layouts of oracle.h."""

    def __init__(self):
        self.lib = C.CDLL(build_oracle())
        L = self.lib
        L.orc_sbessel.restype = C.c_double
        L.orc_sbessel.argtypes = [C.c_int, C.c_double]
        L.orc_w3j.restype = C.c_double
        L.orc_w3j.argtypes = [C.c_int] * 6
        L.orc_best_scale.restype = C.c_double
        L.orc_point_score.restype = C.c_double
        L.orc_average_radius.restype = C.c_double
        L.orc_assemble_index.restype = C.c_int

    def sbessel(self, l, x):
        return self.lib.orc_sbessel(int(l), float(x))

    def mkarray(self, b, e, n):
        out = np.zeros(n)
        self.lib.orc_mkarray(C.c_double(b), C.c_double(e), C.c_int(n), _p(out))
        return out

    def wigner_d(self, L, beta):
        out = np.zeros((L + 1) * (2 * L + 1) ** 2)
        self.lib.orc_wigner_d(C.c_int(L), C.c_double(beta), _p(out))
        return out.reshape(L + 1, 2 * L + 1, 2 * L + 1)

    def w3j(self, *a):
        return self.lib.orc_w3j(*[int(x) for x in a])

    def dsymb(self, L):
        out = np.zeros((L + 1) ** 3 * (2 * L + 1))
        self.lib.orc_dsymb(C.c_int(L), _p(out))
        return out

    def besselj_n(self, z, q, L):
        q = np.ascontiguousarray(q, dtype=np.float64)
        out = np.zeros(len(q) * (2 * L + 1))
        self.lib.orc_besselj_n(C.c_double(z), _p(q), C.c_int(len(q)), C.c_int(L), _p(out))
        return out

    def t_matrix(self, L, bes, ds, qnum):
        K = L + 1
        tre = np.zeros(qnum * K ** 3)
        tim = np.zeros(qnum * K ** 3)
        self.lib.orc_t_matrix(C.c_int(L), C.c_int(qnum), _p(bes), _p(ds), _p(tre), _p(tim))
        return tre, tim

    def expand(self, xyz, vac, dum, sasa, h2o, q, L):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        vac = np.ascontiguousarray(vac, dtype=np.float64)
        dum = np.ascontiguousarray(dum, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = len(vac)
        out = np.zeros(3 * len(q) * (L + 1) ** 2 * 2)
        sp = None
        if sasa is not None:
            sasa = np.ascontiguousarray(sasa, dtype=np.float64)
            sp = _p(sasa)
        self.lib.orc_expand(_p(xyz), _p(vac), _p(dum), sp, C.c_double(h2o), C.c_int(n), _p(q),
                            C.c_int(len(q)), C.c_int(L), _p(out))
        return out

    def average_radius(self, vdw):
        vdw = np.ascontiguousarray(vdw, dtype=np.float64)
        return self.lib.orc_average_radius(_p(vdw), C.c_int(len(vdw)))

    def opt_params(self, eq, ei, ee, q, rm):
        eq, ei, ee, q = (np.ascontiguousarray(x, dtype=np.float64) for x in (eq, ei, ee, q))
        a = np.zeros(6 * len(q))
        mult = C.c_double()
        peak = C.c_double()
        self.lib.orc_opt_params(_p(eq), _p(ei), _p(ee), C.c_int(len(eq)), _p(q), C.c_int(len(q)),
                                C.c_double(rm), _p(a), C.byref(mult), C.byref(peak))
        return a, mult.value, peak.value

    def point_score(self, cross, q, a, mult, c1, c2):
        cross = np.ascontiguousarray(cross, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        self.lib.orc_point_score.argtypes = [_dp, _dp, C.c_int, _dp, C.c_double, C.c_double, C.c_double]
        return self.lib.orc_point_score(cross, q, len(q), a, mult, c1, c2)

    def rescale(self, cross, peak):
        cross = np.array(cross, dtype=np.float64)
        self.lib.orc_rescale(_p(cross), C.c_int(cross.size // 6), C.c_double(peak))
        return cross

    def compile_intensity(self, cross, q, rm, c1, c2, rerr=0.05):
        cross = np.ascontiguousarray(cross, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        i = np.zeros(len(q))
        e = np.zeros(len(q))
        self.lib.orc_compile_intensity(_p(cross), _p(q), C.c_int(len(q)), C.c_double(rm), C.c_double(rerr),
                                       C.c_double(c1), C.c_double(c2), _p(i), _p(e))
        return i, e

    def profile_from_spf(self, spf, L, q, rm, c1, c2):
        q = np.ascontiguousarray(q, dtype=np.float64)
        i = np.zeros(len(q))
        e = np.zeros(len(q))
        self.lib.orc_profile_from_spf(_p(np.ascontiguousarray(spf)), C.c_int(L), C.c_int(len(q)),
                                      C.c_double(rm), _p(q), C.c_double(c1), C.c_double(c2), _p(i), _p(e))
        return i, e

    def spf2cross_terms(self, spf, L, qnum):
        out = np.zeros(6 * qnum)
        self.lib.orc_spf2cross_terms(_p(np.ascontiguousarray(spf)), C.c_int(L), C.c_int(qnum), _p(out))
        return out

    def ft2euler(self, tv, rm9, ref_lig):
        tv, rm9, ref_lig = (np.ascontiguousarray(x, dtype=np.float64) for x in (tv, rm9, ref_lig))
        out = np.zeros(6)
        self.lib.orc_ft2euler(_p(tv), _p(rm9), _p(ref_lig), _p(out))
        return out

    def assemble_index(self, eu6, z_idx, L):
        eu6 = np.ascontiguousarray(eu6, dtype=np.float64)
        return self.lib.orc_assemble_index(_p(eu6), C.c_int(z_idx), C.c_int(L))

    def score(self, A, B, q, z, L, index, skip, peak, a, mult, c1g, c2g):
        q, z, c1g, c2g = (np.ascontiguousarray(x, dtype=np.float64) for x in (q, z, c1g, c2g))
        index = np.ascontiguousarray(index, dtype=np.int32)
        n = len(index)
        Q = len(q)
        raw = np.zeros((max(n, 1), 6, Q))
        scl = np.zeros((max(n, 1), 6, Q))
        grid = np.zeros((max(n, 1), len(c1g), len(c2g)))
        br = np.zeros(max(n, 1), dtype=np.int32)
        rc = self.lib.orc_score(_p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(B)), _p(q), C.c_int(Q),
                                _p(z), C.c_int(len(z)), C.c_int(L),
                                index.ctypes.data_as(C.POINTER(C.c_int)), C.c_int(n), C.c_int(skip),
                                C.c_double(peak), _p(np.ascontiguousarray(a)), C.c_double(mult),
                                _p(c1g), C.c_int(len(c1g)), _p(c2g), C.c_int(len(c2g)),
                                _p(raw), _p(scl), _p(grid), br.ctypes.data_as(C.POINTER(C.c_int)))
        if rc != 0:
            raise ValueError("oracle rejected the pose list")
        return raw[:n], scl[:n], grid[:n], br[:n]


class Ref:
    """The reference's own code (checker build).  Available only where the
    reference sources were given (FMFTSAXS_REFERENCE_SRC) or an earlier build
    of them is present; the GPU test machines have neither."""

    def __init__(self):
        so = build_ref()
        if so is None:
            raise FileNotFoundError("reference sources not present")
        self.lib = C.CDLL(so)
        self.lib.refh_sbessel.restype = C.c_double
        self.lib.refh_sbessel.argtypes = [C.c_int, C.c_double]
        self.lib.refh_w3j.restype = C.c_double
        self.lib.refh_w3j.argtypes = [C.c_int] * 7
        self.lib.refh_average_radius.restype = C.c_double
        self.lib.refh_point_score.restype = C.c_double

    def sbessel(self, l, x):
        return self.lib.refh_sbessel(int(l), float(x))

    def w3j(self, j1, j2, j3, m1, m2, m3):
        return self.lib.refh_w3j(j1, j2, j3, m1, m2, m3, j1 + j2 + j3 + 1)

    def mkarray(self, b, e, n):
        out = np.zeros(n)
        self.lib.refh_mkarray(C.c_double(b), C.c_double(e), C.c_int(n), _p(out))
        return out

    def wigner_d(self, L, beta):
        out = np.zeros((L + 1) * (2 * L + 1) ** 2)
        self.lib.refh_d_array(C.c_int(L), C.c_double(beta), _p(out))
        return out.reshape(L + 1, 2 * L + 1, 2 * L + 1)

    @staticmethod
    def _names(names):
        buf = np.zeros((len(names), 8), dtype=np.uint8)
        for i, s in enumerate(names):
            b = s.encode()[:7]
            buf[i, :len(b)] = np.frombuffer(b, dtype=np.uint8)
        return buf

    def ff_lookup(self, map_path, res, atom):
        n = len(res)
        rb, ab = self._names(res), self._names(atom)
        vac, dum = np.zeros(n), np.zeros(n)
        h2o = C.c_double()
        bad = self.lib.refh_ff_lookup(map_path.encode(), rb.ctypes.data_as(C.c_char_p), ab.ctypes.data_as(C.c_char_p),
                                      C.c_int(n), _p(vac), _p(dum), C.byref(h2o))
        return vac, dum, h2o.value, bad

    def expand(self, xyz, res, atom, vdw, sasa, map_path, q, L):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        vdw = np.ascontiguousarray(vdw, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        n = len(vdw)
        rb, ab = self._names(res), self._names(atom)
        out = np.zeros(3 * len(q) * (L + 1) ** 2 * 2)
        rm = C.c_double()
        sp = None
        if sasa is not None:
            sasa = np.ascontiguousarray(sasa, dtype=np.float64)
            sp = _p(sasa)
        self.lib.refh_expand(_p(xyz), rb.ctypes.data_as(C.c_char_p), ab.ctypes.data_as(C.c_char_p), _p(vdw), sp,
                             C.c_int(n), map_path.encode(), _p(q), C.c_int(len(q)), C.c_int(L), _p(out), C.byref(rm))
        return out, rm.value

    def profile_from_spf(self, spf, L, q, rm, c1, c2):
        q = np.ascontiguousarray(q, dtype=np.float64)
        i = np.zeros(len(q))
        e = np.zeros(len(q))
        self.lib.refh_profile_from_spf(_p(np.ascontiguousarray(spf)), C.c_int(L), C.c_int(len(q)), C.c_double(rm),
                                       _p(q), C.c_double(c1), C.c_double(c2), _p(i), _p(e))
        return i, e

    def opt_params(self, eq, ei, ee, q, rm):
        eq, ei, ee, q = (np.ascontiguousarray(x, dtype=np.float64) for x in (eq, ei, ee, q))
        a = np.zeros(6 * len(q))
        mult = C.c_double()
        peak = C.c_double()
        self.lib.refh_opt_params(_p(eq), _p(ei), _p(ee), C.c_int(len(eq)), _p(q), C.c_int(len(q)), C.c_double(rm),
                                 _p(a), C.byref(mult), C.byref(peak))
        return a, mult.value, peak.value

    def fit_cross(self, cross, eq, ei, ee, q, rm):
        """Peak rescale + L-BFGS-B of one pose: (scaled[6,Q], chi, c1, c2, scale, I[Q])."""
        cross, eq, ei, ee, q = (np.ascontiguousarray(x, dtype=np.float64) for x in (cross, eq, ei, ee, q))
        Q = len(q)
        scaled = np.zeros(6 * Q)
        res = np.zeros(5)
        inten = np.zeros(Q)
        self.lib.refh_fit_cross(_p(cross), _p(eq), _p(ei), _p(ee), C.c_int(len(eq)), _p(q), C.c_int(Q),
                                C.c_double(rm), _p(scaled), _p(res), _p(inten))
        return scaled.reshape(6, Q), res[0], res[1], res[2], res[3], inten

    def point_score(self, cross, eq, ei, ee, q, rm, c1, c2):
        cross, eq, ei, ee, q = (np.ascontiguousarray(x, dtype=np.float64) for x in (cross, eq, ei, ee, q))
        return self.lib.refh_point_score(_p(cross), _p(eq), _p(ei), _p(ee), C.c_int(len(eq)), _p(q),
                                         C.c_int(len(q)), C.c_double(rm), C.c_double(c1), C.c_double(c2))

    def score(self, A, B, rmA, rmB, rm_mean, exp, q, z, L, index, skip, c1g, c2g):
        eq, ei, ee = (np.ascontiguousarray(x, dtype=np.float64) for x in exp)
        q, z, c1g, c2g = (np.ascontiguousarray(x, dtype=np.float64) for x in (q, z, c1g, c2g))
        index = np.ascontiguousarray(index, dtype=np.int32)
        n = len(index)
        Q = len(q)
        chi, c1, c2 = np.zeros(max(n, 1)), np.zeros(max(n, 1)), np.zeros(max(n, 1))
        raw = np.zeros((max(n, 1), 6, Q))
        scl = np.zeros((max(n, 1), 6, Q))
        grid = np.zeros((max(n, 1), len(c1g), len(c2g)))
        br = np.zeros(max(n, 1), dtype=np.int32)
        rc = self.lib.refh_score(_p(np.ascontiguousarray(A)), _p(np.ascontiguousarray(B)), C.c_double(rmA),
                                 C.c_double(rmB), C.c_double(rm_mean), _p(eq), _p(ei), _p(ee), C.c_int(len(eq)),
                                 _p(q), C.c_int(Q), _p(z), C.c_int(len(z)), C.c_int(L),
                                 index.ctypes.data_as(C.POINTER(C.c_int)), C.c_int(n), C.c_int(skip),
                                 _p(c1g), C.c_int(len(c1g)), _p(c2g), C.c_int(len(c2g)),
                                 _p(chi), _p(c1), _p(c2), _p(raw), _p(scl), _p(grid),
                                 br.ctypes.data_as(C.POINTER(C.c_int)))
        if rc != 0:
            raise ValueError("reference harness rejected the pose list")
        return dict(chi=chi[:n], c1=c1[:n], c2=c2[:n], raw=raw[:n], scaled=scl[:n], grid=grid[:n], branch=br[:n])

    def ft2euler(self, tv, rm9, ref_lig):
        tv, rm9, ref_lig = (np.ascontiguousarray(x, dtype=np.float64) for x in (tv, rm9, ref_lig))
        out = np.zeros(6)
        self.lib.refh_ft2euler(_p(tv), _p(rm9), _p(ref_lig), _p(out))
        return out


class OracleWorkload:
    """The calls libfmftsaxs_gb300.workload.build makes on the product
    library, answered by the oracle on the CPU, so that a CPU baseline can
    build its inputs without loading the product.  Form factors: the
    zero-angle constants of the four types the synthetic molecules use and
    of water (src/form_factor_table.c:8-49)."""

    FF = {"C": (5.9992, 5.49096), "N": (6.9946, 0.83166), "O": (7.9994, 3.04942), "S": (15.9998, 6.63324)}
    WATER = 3.50968

    def __init__(self):
        self.o = Oracle()

    def mkarray(self, b, e, n):
        return self.o.mkarray(b, e, n)

    def ff_type(self, name):
        return self.FF[name]

    def ff_water(self):
        return self.WATER

    def expand(self, xyz, vac, dum, sasa, water, q, L):
        return self.o.expand(xyz, vac, dum, sasa, water, q, L)

    def profile_from_spf(self, spf, L, q, rm, c1, c2):
        return self.o.profile_from_spf(spf, L, q, rm, c1, c2)

    def bin_experiment(self, eq, ei, ee, q, rm):
        return self.o.opt_params(eq, ei, ee, q, rm)

    def poses_to_indices(self, R, T, z, L):
        from libfmftsaxs_gb300 import synth
        idx, keep = synth.poses_to_indices(R, T, np.zeros(3), z, L, self.o.ft2euler, self.o.assemble_index)
        return idx.astype(np.int64), keep
