"""Python mirror of the fmftsaxs-gb300 C API (ctypes over the in-tree
libfmftsaxs_gb300.so).  The library is the product: every call below runs
the sm_103a kernels through the C ABI declared in include/fmftsaxs_gb300.h.
There is no fallback: if the shared library is missing or cannot find a
GPU, calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfmftsaxs_gb300.so")

FIT_NONE, FIT_GRID, FIT_LBFGSB = 0, 1, 2
FP64 = 0
MIXED = 1
ROT_CUDA, ROT_TC = 0, 1
BATCH_PERSISTENT, BATCH_OVERLAP, BATCH_ITEMS = 1, 2, 4
FUSE_AUTO, FUSE_ON, FUSE_OFF = 0, 1, 2
BATCH_DEFAULT = BATCH_PERSISTENT

_lib = None


class SxsError(RuntimeError):
    pass


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SxsError("libfmftsaxs_gb300.so not built (run __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    lib.sxsg_last_error.restype = C.c_char_p
    lib.sxsg_launch_count.restype = C.c_longlong
    lib.sxsg_ff_water.restype = C.c_double
    lib.sxsg_assemble_index.restype = C.c_int64
    lib.sxsg_assemble_index.argtypes = [C.POINTER(C.c_double), C.c_int, C.c_int]
    lib.sxs_sbessel.restype = C.c_double
    lib.sxs_sbessel.argtypes = [C.c_int, C.c_double]
    lib.sxs_mkarray.restype = C.POINTER(C.c_double)
    lib.sxs_mkarray.argtypes = [C.c_double, C.c_double, C.c_int]
    lib.sxsg_plan_create.argtypes = [C.POINTER(C.c_void_p)] + [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_int, C.c_int,
                                     C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                     C.c_int]
    lib.sxsg_plan_set_poses.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int]
    lib.sxsg_plan_run.argtypes = [C.c_void_p, C.c_int]
    lib.sxsg_plan_results.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    lib.sxsg_plan_timings.argtypes = [C.c_void_p, C.c_void_p]
    lib.sxsg_plan_destroy.argtypes = [C.c_void_p]
    lib.sxsg_plan_destroy.restype = None
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        raise SxsError(load().sxsg_last_error().decode(errors="replace"))
    return rc


def last_error():
    return load().sxsg_last_error().decode(errors="replace")


def launch_count():
    return int(load().sxsg_launch_count())


def device_memory():
    """(free, total) bytes of the library's device."""
    f, t = C.c_size_t(), C.c_size_t()
    _check(load().sxsg_device_memory(C.byref(f), C.byref(t)))
    return int(f.value), int(t.value)


def init(device=0):
    _check(load().sxsg_init(int(device)))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def ff_type(name):
    """(vacuum_ff, dummy_ff) of a form-factor type name of the mapping file."""
    v, d = C.c_double(), C.c_double()
    if load().sxsg_ff_type(name.encode(), C.byref(v), C.byref(d)) != 0:
        raise KeyError(name)
    return v.value, d.value


def ff_water():
    return load().sxsg_ff_water()


def ff_lookup(mapping_path, res, atom):
    """(vacuum_ff[n], dummy_ff[n], n_missing) for (residue, atom) names."""
    n = len(res)
    rb = np.zeros((n, 8), dtype=np.uint8)
    ab = np.zeros((n, 8), dtype=np.uint8)
    for i in range(n):
        r, a = res[i].encode()[:8], atom[i].encode()[:8]
        rb[i, :len(r)] = np.frombuffer(r, dtype=np.uint8)
        ab[i, :len(a)] = np.frombuffer(a, dtype=np.uint8)
    vac, dum = np.zeros(n), np.zeros(n)
    rc = load().sxsg_ff_lookup(mapping_path.encode(), rb.ctypes.data_as(C.c_char_p), ab.ctypes.data_as(C.c_char_p),
                               C.c_int(n), _p(vac), _p(dum))
    if rc < 0:
        raise SxsError(last_error())
    return vac, dum, rc


def sbessel(l, x):
    return load().sxs_sbessel(int(l), float(x))


def mkarray(begin, end, n):
    lib = load()
    ptr = lib.sxs_mkarray(float(begin), float(end), int(n))
    out = np.array([ptr[i] for i in range(n)])
    C.CDLL(None).free(C.cast(ptr, C.c_void_p))
    return out


def expand(xyz, vacuum_ff, dummy_ff, sasa, water_ff, qvals, L):
    """A_lm(q) of one molecule on the GPU: flat [3][Q][(L+1)^2][2]."""
    xyz, vac, dum, q = f64(xyz), f64(vacuum_ff), f64(dummy_ff), f64(qvals)
    n = len(vac)
    out = np.zeros(3 * len(q) * (L + 1) ** 2 * 2)
    sp = None
    if sasa is not None:
        sasa = f64(sasa)
        sp = _p(sasa)
    _check(load().sxsg_expand(_p(xyz), _p(vac), _p(dum), sp, C.c_double(water_ff), C.c_int(n), _p(q),
                              C.c_int(len(q)), C.c_int(L), _p(out)))
    return out


def bin_experiment(exp_q, exp_i, exp_err, qvals, rm):
    """(a[6Q], mult, peak): the binned experiment of sxs_opt_params_create."""
    eq, ei, ee, q = f64(exp_q), f64(exp_i), f64(exp_err), f64(qvals)
    a = np.zeros(6 * len(q))
    mult, peak = C.c_double(), C.c_double()
    _check(load().sxsg_bin_experiment(_p(eq), _p(ei), _p(ee), C.c_int(len(eq)), _p(q), C.c_int(len(q)),
                                      C.c_double(rm), _p(a), C.byref(mult), C.byref(peak)))
    return a, mult.value, peak.value


def ft2euler(tv, rm9, ref_lig):
    """sxs_ft2euler on plain arrays -> (z, b1, g1, a2, b2, g2)."""
    class V3(C.Structure):
        _fields_ = [("X", C.c_double), ("Y", C.c_double), ("Z", C.c_double)]

    class M3(C.Structure):
        _fields_ = [(n, C.c_double) for n in ("m11", "m12", "m13", "m21", "m22", "m23", "m31", "m32", "m33")]

    class EU(C.Structure):
        _fields_ = [(n, C.c_double) for n in ("z", "b1", "g1", "a2", "b2", "g2")]

    t = V3(*map(float, tv))
    r = V3(*map(float, ref_lig))
    m = M3(*map(float, np.asarray(rm9).reshape(9)))
    e = EU()
    load().sxs_ft2euler(C.byref(e), C.byref(t), C.byref(m), C.byref(r))
    return np.array([e.z, e.b1, e.g1, e.a2, e.b2, e.g2])


def assemble_index(eu6, z_idx, L):
    e = f64(eu6)
    return int(load().sxsg_assemble_index(_p(e), int(z_idx), int(L)))


class Plan:
    """A device-resident scoring plan (sxsg_plan_*)."""

    def __init__(self, A, B, qvals, zvals, L, a, mult, peak, c1grid=None, c2grid=None, precision=FP64):
        lib = load()
        self.A, self.B, self.q, self.z, self.a = f64(A), f64(B), f64(qvals), f64(zvals), f64(a)
        self.c1g = f64(c1grid if c1grid is not None else np.zeros(0))
        self.c2g = f64(c2grid if c2grid is not None else np.zeros(0))
        self.L, self.Q = L, len(self.q)
        self.mult, self.peak = float(mult), float(peak)
        self.index = np.zeros(0, dtype=np.int64)
        self.h = C.c_void_p()
        _check(lib.sxsg_plan_create(C.byref(self.h), self.A.ctypes.data, self.B.ctypes.data, self.q.ctypes.data,
                                    self.Q, self.z.ctypes.data, len(self.z), L, self.a.ctypes.data, mult, peak,
                                    self.c1g.ctypes.data if len(self.c1g) else None, len(self.c1g),
                                    self.c2g.ctypes.data if len(self.c2g) else None, len(self.c2g), precision))
        self.n = 0

    def set_poses(self, index, skip=1):
        idx = np.ascontiguousarray(index, dtype=np.int64)
        self.n = len(idx)
        _check(load().sxsg_plan_set_poses(self.h, idx.ctypes.data, self.n, int(skip)))
        self.index = idx

    def set_rotation(self, engine):
        load().sxsg_plan_set_rotation.argtypes = [C.c_void_p, C.c_int]
        _check(load().sxsg_plan_set_rotation(self.h, int(engine)))

    def set_tiles(self, tr_slices=0, rot_gamma=0):
        """Tile choices (sxsg_plan_set_tiles); 0 keeps the tuned default."""
        load().sxsg_plan_set_tiles.argtypes = [C.c_void_p, C.c_int, C.c_int]
        _check(load().sxsg_plan_set_tiles(self.h, int(tr_slices), int(rot_gamma)))

    def set_fused(self, mode):
        """Translation fused with the per-pose contraction (sxsg_plan_set_fused):
        FUSE_AUTO, FUSE_ON or FUSE_OFF."""
        load().sxsg_plan_set_fused.argtypes = [C.c_void_p, C.c_int]
        _check(load().sxsg_plan_set_fused(self.h, int(mode)))

    def set_budget(self, nbytes):
        load().sxsg_plan_set_budget.argtypes = [C.c_void_p, C.c_size_t]
        _check(load().sxsg_plan_set_budget(self.h, int(nbytes)))

    def run(self, fit=FIT_GRID):
        _check(load().sxsg_plan_run(self.h, int(fit)))

    def results(self, cross=False, grid=False):
        n = self.n
        chi, c1, c2 = np.zeros(n), np.zeros(n), np.zeros(n)
        cell = np.zeros(n, dtype=np.int32)
        cr = np.zeros((n, 6, self.Q)) if cross else None
        gr = np.zeros((n, len(self.c1g), len(self.c2g))) if grid else None
        _check(load().sxsg_plan_results(self.h, chi.ctypes.data, c1.ctypes.data, c2.ctypes.data, cell.ctypes.data,
                                        cr.ctypes.data if cross else None, gr.ctypes.data if grid else None))
        out = dict(chi=chi, c1=c1, c2=c2, cell=cell)
        if cross:
            out["cross"] = cr
        if grid:
            out["grid"] = gr
        return out

    def topk(self, k):
        """The k best poses of the last fitted run, selected on the device
        (sxsg_plan_topk): dict(pose=list positions, chi, c1, c2), ascending
        chi, ties in list order."""
        lib = load()
        lib.sxsg_plan_topk.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4
        m = min(int(k), self.n)
        pose, chi, c1, c2 = np.zeros(m, dtype=np.int64), np.zeros(m), np.zeros(m), np.zeros(m)
        got = lib.sxsg_plan_topk(self.h, int(k), pose.ctypes.data, chi.ctypes.data, c1.ctypes.data, c2.ctypes.data)
        if got < 0:
            raise SxsError(last_error())
        return dict(pose=pose[:got], chi=chi[:got], c1=c1[:got], c2=c2[:got])

    def chunks(self):
        """Chunks of the translated table the last run used."""
        load().sxsg_plan_chunks.argtypes = [C.c_void_p]
        return int(load().sxsg_plan_chunks(self.h))

    def timings(self):
        ms = np.zeros(5)
        _check(load().sxsg_plan_timings(self.h, ms.ctypes.data))
        return dict(tables=ms[0], translate=ms[1], pose=ms[2], fit=ms[3], total=ms[4])

    def close(self):
        if self.h:
            load().sxsg_plan_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _BatchStats(C.Structure):
    _fields_ = [("plans", C.c_int), ("phases", C.c_int), ("launches", C.c_int), ("items", C.c_int64),
                ("poses", C.c_int64), ("arena_bytes", C.c_size_t), ("ms", C.c_double * 4)]


class Batch:
    """Many mixed-precision plans scored by one CUDA graph of persistent
    kernels (sxsg_batch_*).  The plans keep their results: read them with
    Plan.results / Plan.topk after run().  The batch holds the plans'
    device pointers: keep the plans alive and unchanged while it exists."""

    def __init__(self, plans, fit=FIT_GRID, arena_bytes=0, flags=None):
        lib = load()
        lib.sxsg_batch_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]
        if flags is None:
            flags = BATCH_DEFAULT
        lib.sxsg_batch_run.argtypes = [C.c_void_p]
        lib.sxsg_batch_stats_get.argtypes = [C.c_void_p, C.POINTER(_BatchStats)]
        lib.sxsg_batch_destroy.argtypes = [C.c_void_p]
        lib.sxsg_batch_destroy.restype = None
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[p.h.value for p in self.plans])
        self.h = C.c_void_p()
        _check(lib.sxsg_batch_create(arr, len(self.plans), int(fit), int(arena_bytes), int(flags), C.byref(self.h)))

    def run(self):
        _check(load().sxsg_batch_run(self.h))

    def stats(self):
        st = _BatchStats()
        _check(load().sxsg_batch_stats_get(self.h, C.byref(st)))
        return dict(plans=st.plans, phases=st.phases, launches=st.launches, items=int(st.items),
                    poses=int(st.poses), arena_bytes=int(st.arena_bytes), tables_ms=st.ms[0],
                    phases_ms=st.ms[1], fit_ms=st.ms[2], total_ms=st.ms[3])

    def close(self):
        if self.h:
            load().sxsg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Request(C.Structure):
    _fields_ = [("A", C.c_void_p), ("B", C.c_void_p), ("keyA", C.c_uint64), ("keyB", C.c_uint64),
                ("qvals", C.c_void_p), ("qnum", C.c_int), ("zvals", C.c_void_p), ("znum", C.c_int), ("L", C.c_int),
                ("a", C.c_void_p), ("mult", C.c_double), ("peak", C.c_double), ("c1grid", C.c_void_p),
                ("n1", C.c_int), ("c2grid", C.c_void_p), ("n2", C.c_int), ("index", C.c_void_p),
                ("n", C.c_int64), ("skip", C.c_int), ("fit_mode", C.c_int), ("precision", C.c_int)]


class Server:
    """The serving loop (sxsg_server_*): jobs are admitted in arrival order
    under an HBM cap, run concurrently on the device and keep molecule
    rotation tables cached by key."""

    def __init__(self, hbm_cap=0, max_active=4):
        lib = load()
        lib.sxsg_server_create.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_int]
        lib.sxsg_server_submit.argtypes = [C.c_void_p, C.POINTER(_Request)]
        lib.sxsg_server_submit.restype = C.c_int64
        lib.sxsg_server_poll.argtypes = [C.c_void_p, C.c_int64]
        lib.sxsg_server_wait.argtypes = [C.c_void_p, C.c_int64] + [C.c_void_p] * 4
        lib.sxsg_server_stats.argtypes = [C.c_void_p, C.c_void_p]
        lib.sxsg_server_destroy.argtypes = [C.c_void_p]
        lib.sxsg_server_destroy.restype = None
        self.h = C.c_void_p()
        _check(lib.sxsg_server_create(C.byref(self.h), int(hbm_cap), int(max_active)))
        self.sizes = {}

    def submit(self, A, B, qvals, zvals, L, a, mult, peak, index, c1grid=None, c2grid=None, skip=1, fit=FIT_GRID,
               precision=MIXED, keyA=0, keyB=0):
        A, B, q, z, a = f64(A), f64(B), f64(qvals), f64(zvals), f64(a)
        c1 = f64(c1grid if c1grid is not None else np.zeros(0))
        c2 = f64(c2grid if c2grid is not None else np.zeros(0))
        idx = np.ascontiguousarray(index, dtype=np.int64)
        r = _Request(A.ctypes.data, B.ctypes.data, int(keyA), int(keyB), q.ctypes.data, len(q), z.ctypes.data,
                     len(z), int(L), a.ctypes.data, float(mult), float(peak), c1.ctypes.data if len(c1) else None,
                     len(c1), c2.ctypes.data if len(c2) else None, len(c2), idx.ctypes.data if len(idx) else None,
                     len(idx), int(skip), int(fit), int(precision))
        t = load().sxsg_server_submit(self.h, C.byref(r))
        if t < 0:
            raise SxsError(last_error())
        self.sizes[t] = len(idx)
        return t

    def done(self, ticket):
        rc = load().sxsg_server_poll(self.h, ticket)
        if rc < 0:
            raise SxsError(last_error())
        return bool(rc)

    def wait(self, ticket):
        """dict(chi, c1, c2, queued_ms, run_ms, latency_ms)"""
        n = self.sizes.pop(ticket)
        chi, c1, c2, ms = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(3)
        _check(load().sxsg_server_wait(self.h, ticket, chi.ctypes.data, c1.ctypes.data, c2.ctypes.data,
                                       ms.ctypes.data))
        return dict(chi=chi, c1=c1, c2=c2, queued_ms=ms[0], run_ms=ms[1], latency_ms=ms[2])

    def stats(self):
        o = np.zeros(8)
        _check(load().sxsg_server_stats(self.h, o.ctypes.data))
        return dict(done=int(o[0]), poses=int(o[1]), queued=int(o[2]), running_bytes=int(o[3]),
                    cache_bytes=int(o[4]), cache_entries=int(o[5]), cache_hits=int(o[6]), cache_misses=int(o[7]))

    def close(self):
        if self.h:
            load().sxsg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def score_exact(rec_xyz, lig_xyz, vac, dum, water_w, euler, qvals, L, a, mult, cross=False):
    """Exact per-pose scoring (sxsg_score_exact): the score_ft_naive flow on
    the GPU.  euler: [n][6] (z, b1, g1, a2, b2, g2)."""
    rx, lx, v, d = f64(rec_xyz).reshape(-1, 3), f64(lig_xyz).reshape(-1, 3), f64(vac), f64(dum)
    w = f64(water_w) if water_w is not None else None
    eu, q, a = f64(euler).reshape(-1, 6), f64(qvals), f64(a)
    n = len(eu)
    chi, c1, c2 = np.zeros(n), np.zeros(n), np.zeros(n)
    cr = np.zeros((n, 6, len(q))) if cross else None
    lib = load()
    lib.sxsg_score_exact.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 4 + \
        [C.c_int64, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_double] + [C.c_void_p] * 4
    _check(lib.sxsg_score_exact(rx.ctypes.data, len(rx), lx.ctypes.data, len(lx), v.ctypes.data, d.ctypes.data,
                                w.ctypes.data if w is not None else None, eu.ctypes.data, n, q.ctypes.data, len(q),
                                int(L), a.ctypes.data, float(mult), chi.ctypes.data, c1.ctypes.data, c2.ctypes.data,
                                cr.ctypes.data if cross else None))
    out = dict(chi=chi, c1=c1, c2=c2)
    if cross:
        out["cross"] = cr
    return out


def sasa(xyz, radius, probe=1.4, npts=240, sphere=None):
    """Accessible fraction per atom on the GPU (sxsg_sasa)."""
    x, r = f64(xyz).reshape(-1, 3), f64(radius)
    out = np.zeros(len(r))
    sph = f64(sphere).reshape(-1, 3) if sphere is not None else None
    lib = load()
    lib.sxsg_sasa.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_int, C.c_void_p]
    _check(lib.sxsg_sasa(x.ctypes.data, r.ctypes.data, len(r), float(probe),
                         sph.ctypes.data if sph is not None else None, len(sph) if sph is not None else int(npts),
                         out.ctypes.data))
    return out


def profile_from_spf(spf, L, qvals, rm, c1, c2):
    """(I[Q], err[Q]) of one molecule (sxs_profile_from_spf on a flat expansion)."""
    q = f64(qvals)
    i, e = np.zeros(len(q)), np.zeros(len(q))
    _check(load().sxsg_profile_from_flat(_p(f64(spf)), C.c_int(L), C.c_int(len(q)), C.c_double(rm), _p(q),
                                         C.c_double(c1), C.c_double(c2), _p(i), _p(e)))
    return i, e


WRAP_ANGLES = 1


def poses_to_indices(rot, tr, zvals, L, ref_lig=(0.0, 0.0, 0.0), wrap=False):
    """Batch pose ingestion (ft2euler, 3-decimal round trip, index assembly).
    Returns (index[int64] of kept poses, keep mask).  wrap=True takes the
    alpha/gamma digits mod N (the reference does not wrap them)."""
    rot = f64(rot).reshape(-1, 9)
    tr = f64(tr).reshape(-1, 3)
    n = len(rot)
    idx = np.zeros(n, dtype=np.int64)
    keep = np.zeros(n, dtype=np.uint8)
    ref = f64(ref_lig)
    z = f64(zvals)
    k = load().sxsg_poses_to_indices_ex(_p(rot), _p(tr), C.c_int64(n), _p(ref), _p(z), C.c_int(len(z)), C.c_int(L),
                                        idx.ctypes.data_as(C.POINTER(C.c_int64)),
                                        keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.c_int(WRAP_ANGLES if wrap else 0))
    if k < 0:
        raise SxsError(last_error())
    return idx[keep.astype(bool)], keep.astype(bool)


def tiles_default(L, Q):
    """(slices per translation block, gamma pairs per rotation thread) of the
    library's autotuned table for (L, Q) (sxsg_tiles_default)."""
    sb, g = C.c_int(0), C.c_int(0)
    _check(load().sxsg_tiles_default(C.c_int(L), C.c_int(Q), C.byref(sb), C.byref(g)))
    return sb.value, g.value


def poses_to_indices_gpu(rot, tr, zvals, L, ref_lig=(0.0, 0.0, 0.0), wrap=False, full=False):
    """poses_to_indices on the GPU (sxsg_poses_to_indices_gpu), same results.
    Returns (index of kept poses, keep mask, poses the host redid); with
    full=True the index array covers every pose (-1 where not kept)."""
    lib = load()
    lib.sxsg_poses_to_indices_gpu.restype = C.c_int64
    rot = f64(rot).reshape(-1, 9)
    tr = f64(tr).reshape(-1, 3)
    n = len(rot)
    idx = np.zeros(n, dtype=np.int64)
    keep = np.zeros(n, dtype=np.uint8)
    ref = f64(ref_lig)
    z = f64(zvals)
    nh = C.c_int64(0)
    k = lib.sxsg_poses_to_indices_gpu(_p(rot), _p(tr), C.c_int64(n), _p(ref), _p(z), C.c_int(len(z)), C.c_int(L),
                                      idx.ctypes.data_as(C.POINTER(C.c_int64)),
                                      keep.ctypes.data_as(C.POINTER(C.c_uint8)), C.c_int(WRAP_ANGLES if wrap else 0),
                                      C.byref(nh))
    if k < 0:
        raise SxsError(last_error())
    kb = keep.astype(bool)
    return (idx if full else idx[kb]), kb, nh.value


def score_flat(A, B, qvals, zvals, L, index, a, mult, peak, skip=1, fit=FIT_GRID, c1grid=None, c2grid=None,
               cross=False, precision=FP64):
    """One-shot scoring from host buffers (sxsg_score_flat)."""
    A, B, q, z, a = f64(A), f64(B), f64(qvals), f64(zvals), f64(a)
    idx = np.ascontiguousarray(index, dtype=np.int64)
    c1g = f64(c1grid if c1grid is not None else np.zeros(0))
    c2g = f64(c2grid if c2grid is not None else np.zeros(0))
    n = len(idx)
    chi, c1, c2 = np.zeros(n), np.zeros(n), np.zeros(n)
    cr = np.zeros((n, 6, len(q))) if cross else None
    lib = load()
    lib.sxsg_score_flat.argtypes = [C.c_void_p] * 3 + [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int64,
                                    C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_int] + [C.c_void_p] * 4 + [C.c_int]
    _check(lib.sxsg_score_flat(A.ctypes.data, B.ctypes.data, q.ctypes.data, len(q), z.ctypes.data, len(z), L,
                               idx.ctypes.data, n, skip, a.ctypes.data, mult, peak, fit,
                               c1g.ctypes.data if len(c1g) else None, len(c1g),
                               c2g.ctypes.data if len(c2g) else None, len(c2g),
                               chi.ctypes.data, c1.ctypes.data, c2.ctypes.data, cr.ctypes.data if cross else None,
                               int(precision)))
    out = dict(chi=chi, c1=c1, c2=c2)
    if cross:
        out["cross"] = cr
    return out


def timer_start():
    _check(load().sxsg_timer_start())


def timer_stop():
    lib = load()
    lib.sxsg_timer_stop.restype = C.c_double
    ms = lib.sxsg_timer_stop()
    if ms < 0:
        raise SxsError("timer failed")
    return ms


def fp64_fma_tflops():
    lib = load()
    lib.sxsg_fp64_fma_tflops.restype = C.c_double
    return lib.sxsg_fp64_fma_tflops()


def fp32_fma_tflops():
    lib = load()
    lib.sxsg_fp32_fma_tflops.restype = C.c_double
    return lib.sxsg_fp32_fma_tflops()


def l2_read_gbs():
    lib = load()
    lib.sxsg_l2_read_gbs.restype = C.c_double
    return lib.sxsg_l2_read_gbs()
