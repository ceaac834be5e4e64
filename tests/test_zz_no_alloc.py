"""The allocation-free expansion entry point (sxsg_expand_noalloc) gives the
same A_lm as the regular one (sxsg_expand).

sxsg_expand_noalloc serves callers that cannot allocate device memory:
programs whose device memory all comes from a host application's pool, or
code running where a synchronising cudaMalloc is not allowed.  The caller
passes device buffers for inputs and output; the work buffers sit in a
fixed static device array shared by all calls.  This file is collected last
so that a run stopping at its first failure has run every other test; it
also passes alone in a fresh process.  Device buffers here come from torch
(plumbing only).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # channel-scaled, as in the expansion parity tests


def chan_err(x, y, Q):
    x = x.reshape(3, Q, -1)
    y = y.reshape(3, Q, -1)
    sc = np.max(np.abs(y), axis=-1, keepdims=True)
    sc[sc == 0] = 1.0
    return float(np.max(np.abs(x - y) / sc))


def _molecule(n, rg, seed):
    from libfmftsaxs_gb300 import synth
    m = synth.make_molecule(n, rg, seed).with_sasa()
    return m.translated(-m.centroid())


def _call_noalloc(gpu, torch, xyz, vac, dum, wat, q, L):
    dev = torch.device("cuda", 0)
    t = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    d_xyz, d_vac, d_dum, d_q = t(xyz), t(vac), t(dum), t(q)
    d_w = t(wat) if wat is not None else None
    out = torch.zeros(3 * len(q) * (L + 1) ** 2 * 2, dtype=torch.float64, device=dev)
    so = gpu.load()
    so.sxsg_expand_noalloc.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                          C.c_void_p]
    torch.cuda.synchronize()
    rc = so.sxsg_expand_noalloc(d_xyz.data_ptr(), d_vac.data_ptr(), d_dum.data_ptr(),
                                d_w.data_ptr() if d_w is not None else None, len(vac), d_q.data_ptr(), len(q), L,
                                out.data_ptr(), None)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_expansion_matches_regular_entry_twice(gpu):
    torch = pytest.importorskip("torch")
    L, Q = 12, 24
    q = gpu.mkarray(0.0, 0.5, Q)
    water = gpu.ff_water()
    mols = [(_molecule(300, 9.0, 11), True), (_molecule(180, 8.0, 12), False)]
    for mol, with_water in mols:  # two calls in a row share the static array
        ff = np.array([gpu.ff_type(e) for e in mol.elements])
        want = gpu.expand(mol.xyz, ff[:, 0], ff[:, 1], mol.sasa if with_water else None, water, q, L)
        wat = water * mol.sasa if with_water else None
        rc, got = _call_noalloc(gpu, torch, mol.xyz, ff[:, 0], ff[:, 1], wat, q, L)
        assert rc == 0
        assert chan_err(got, want, Q) <= TOL
        if not with_water:
            assert np.all(got.reshape(3, -1)[2] == 0.0)
    # another L next: every call rewrites the norm table it shares
    L2, Q2 = 7, 9
    q2 = gpu.mkarray(0.0, 0.4, Q2)
    mol = mols[0][0]
    ff = np.array([gpu.ff_type(e) for e in mol.elements])
    want = gpu.expand(mol.xyz, ff[:, 0], ff[:, 1], mol.sasa, water, q2, L2)
    rc, got = _call_noalloc(gpu, torch, mol.xyz, ff[:, 0], ff[:, 1], water * mol.sasa, q2, L2)
    assert rc == 0
    assert chan_err(got, want, Q2) <= TOL


def test_noalloc_rejects_requests_beyond_the_static_array(gpu):
    torch = pytest.importorskip("torch")
    L, Q = 30, 201
    n = 5000  # needs about 5000 * (2*961 + 2) doubles > 8 Mi
    xyz = np.random.default_rng(0).normal(size=(n, 3)) * 10
    rc, _ = _call_noalloc(gpu, torch, xyz, np.ones(n), np.ones(n), None, gpu.mkarray(0.0, 0.5, Q), L)
    assert rc == -3
    rc, _ = _call_noalloc(gpu, torch, xyz[:2], np.ones(2), np.ones(2), None, gpu.mkarray(0.0, 0.5, 3), 41)
    assert rc == -2
