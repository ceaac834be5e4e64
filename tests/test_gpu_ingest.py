"""Pose ingestion on the GPU (sxsg_poses_to_indices_gpu) gives, pose for
pose, the indices and keep flags of the host path (sxsg_poses_to_indices_ex,
bit-exact with the reference's ft2euler and correlate's index assembly):
random poses at the benchmark shapes, both angle options, more poses than
one device batch, and poses built to sit on the cases the device hands back
to the host (translations along z, rotations about z, Euler angles a few
ulps from a "% .3f" half-way point, a zero translation component)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host(gpu, R, T, z, L, ref, wrap):
    rot = np.ascontiguousarray(R.reshape(-1, 9), dtype=np.float64)
    idx, keep = gpu.poses_to_indices(rot, T, z, L, ref_lig=ref, wrap=wrap)
    full = np.full(len(rot), -1, dtype=np.int64)
    full[keep] = idx
    return full, keep


def _compare(gpu, R, T, z, L, ref=(0.0, 0.0, 0.0), wrap=False):
    want, wkeep = _host(gpu, R, T, z, L, ref, wrap)
    got, gkeep, nhost = gpu.poses_to_indices_gpu(R.reshape(-1, 9), T, z, L, ref_lig=ref, wrap=wrap, full=True)
    np.testing.assert_array_equal(gkeep, wkeep)
    np.testing.assert_array_equal(got, want)
    return nhost


def _euler_rot(a, b, g):
    """active z-y-z rotation R(a, b, g) (sxs_fill_active_rotation_matrix)"""
    ca, sa, cb, sb, cg, sg = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(g), np.sin(g)
    return np.array([[cg * cb * ca - sg * sa, -sg * cb * ca - cg * sa, sb * ca],
                     [cg * cb * sa + sg * ca, -sg * cb * sa + cg * ca, sb * sa],
                     [-cg * sb, sg * sb, cb]])


@pytest.mark.parametrize("L,tmin,tmax,wrap", [(15, 25.0, 40.0, False), (20, 30.0, 50.0, False),
                                             (20, 30.0, 50.0, True), (30, 40.0, 65.0, False)])
def test_random_poses_match_host(gpu, L, tmin, tmax, wrap):
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(L * 7 + wrap)
    n = 200000
    R = synth.random_rotations(n, rng)
    T = synth.random_translations(n, tmin, tmax, rng)
    z = np.arange(np.floor(tmin), np.ceil(tmax) + 1.0)
    nhost = _compare(gpu, R, T, z[::2], L, ref=(0.5, -0.25, 1.0), wrap=wrap)  # half the z values off the grid
    assert nhost < n // 100


def test_more_poses_than_one_batch(gpu):
    from libfmftsaxs_gb300 import synth
    rng = np.random.default_rng(3)
    n = (1 << 20) + 4321
    R = synth.random_rotations(n, rng)
    T = synth.random_translations(n, 30.0, 50.0, rng)
    _compare(gpu, R, T, np.arange(30.0, 51.0), 20)


def test_poses_on_the_host_fallback_cases(gpu):
    rng = np.random.default_rng(11)
    Rs, Ts = [], []
    # translations along +-z and with a zero y component
    for t in ([0, 0, 35.0], [0, 0, -35.0], [20.0, 0.0, 28.0], [0.0, 0.0, 0.0 + 40.0], [1e-12, 0, 36.0]):
        for _ in range(20):
            Rs.append(_euler_rot(*rng.uniform(0, 2 * np.pi, 3)))
            Ts.append(t)
    # identity and rotations about z (beta = 0 or pi)
    for b in (0.0, np.pi):
        for a in np.linspace(0, 2 * np.pi, 17):
            Rs.append(_euler_rot(a, b, 0.3))
            Ts.append(rng.normal(size=3) * 20 + [0, 0, 10])
    # receptor angles on a "% .3f" half-way point: place the ligand so that
    # beta_rec is k/1000 + 1/2000 to within rounding
    for k in range(200):
        b1 = 0.3 + k * 0.0137
        b1 = np.floor(b1 * 1000) / 1000 + 0.0005
        g1 = rng.uniform(0.1, 6.0)
        r = 37.0
        Ts.append([-r * np.sin(b1) * np.cos(g1), r * np.sin(b1) * np.sin(g1), r * np.cos(b1)])
        Rs.append(_euler_rot(*rng.uniform(0, 2 * np.pi, 3)))
    R, T = np.array(Rs), np.array(Ts, dtype=np.float64)
    for L in (15, 20):
        nhost = _compare(gpu, R, T, np.arange(25.0, 46.0), L)
        assert nhost >= 100   # these poses are meant for the host path
