"""Accessible fractions on the GPU (sxsg_sasa) against the Shrake-Rupley
restatement of libfmftsaxs_gb300/synth.py: identical on the same sphere
points (the same distance arithmetic, point for point); within one sphere
point per atom with the library's own golden spiral."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,seed", [(1, 1), (40, 2), (600, 3), (2500, 4)])
def test_sasa_matches_restatement(gpu, n, seed):
    from libfmftsaxs_gb300 import synth
    m = synth.make_molecule(n, 2.2 * (n / 8.0) ** 0.38 + 3.0, seed)
    sph = synth.golden_sphere(240)
    want = synth.sasa_fraction(m.xyz, m.radius, 1.4, sph=sph)
    got = gpu.sasa(m.xyz, m.radius, 1.4, sphere=sph)
    np.testing.assert_array_equal(got, want)
    own = gpu.sasa(m.xyz, m.radius, 1.4, npts=240)
    assert np.max(np.abs(own - want)) <= 1.0 / 240 + 1e-15


def test_sasa_edge_cases(gpu):
    xyz = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [50.0, 0.0, 0.0]])
    r = np.array([1.8, 0.0, 1.5])
    got = gpu.sasa(xyz, r, 1.4)
    assert got[1] == 0.0          # zero radius
    assert got[2] == 1.0          # isolated atom
    assert got[0] == 1.0          # the zero-radius neighbour's 1.4 A sphere lies inside atom 0's
    assert gpu.sasa(np.zeros((0, 3)), np.zeros(0)).shape == (0,)
