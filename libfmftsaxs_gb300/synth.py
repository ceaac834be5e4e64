"""Seeded synthetic workloads for the FFT-correlation scoring path.

The reference is measured on real complexes; here seeded stand-ins with the
same shapes are generated:

* Molecules: 3.8 A-step self-avoiding random-walk chains confined to a
  sphere whose radius gives the target radius of gyration (uniform ball:
  R = Rg * sqrt(5/3)).  Elements C/N/O/S are drawn at 63/17/19/1 % and mapped
  to the (residue, atom) names ALA C, ALA N, ALA O, MET SD, whose form-factor
  types are C, N, O, S and whose van der Waals radii in the reference's
  parameter file (prms/atoms.0.0.6.prm.ms.3cap+0.5ace.Hr0rec) are
  1.87, 1.83, 1.55 and 1.97 A.
* Solvent accessibility: the fraction of each atom's probe-expanded sphere
  (probe 1.4 A) left uncovered by its neighbours, by Shrake-Rupley sampling
  on a golden-spiral point set.  The reference obtains it from libmol2's
  accs (absent here); it is an input that both sides of every comparison
  share.
* Poses: uniform SO(3) rotations from seeded quaternions and translations
  of uniform direction with |t| uniform in a range, converted to grid
  indices the way tools/correlate.c does (ft2euler, 3-decimal round trip of
  the Euler file, index assembly).

Only numpy is used; the pose conversion and index assembly are passed in as
callables so that either the library or the oracle can do them.
"""
import numpy as np

ELEMENTS = ("C", "N", "O", "S")
ELEMENT_P = (0.63, 0.17, 0.19, 0.01)
ELEMENT_NAMES = {"C": ("ALA", "C"), "N": ("ALA", "N"), "O": ("ALA", "O"), "S": ("MET", "SD")}
ELEMENT_RADIUS = {"C": 1.87, "N": 1.83, "O": 1.55, "S": 1.97}


def random_walk_chain(n, rg, rng, step=3.8, min_sep=2.5):
    """Self-avoiding random walk of n beads, step `step`, inside a ball of
    radius rg*sqrt(5/3); beads stay at least `min_sep` apart.  A walk that
    is boxed in continues from a random earlier bead (a branch); if no bead
    can branch, the ball grows by 2 %."""
    R = rg * np.sqrt(5.0 / 3.0)
    pts = np.zeros((n, 3))
    cell = min_sep
    grid = {}

    def key(p):
        return (int(np.floor(p[0] / cell)), int(np.floor(p[1] / cell)), int(np.floor(p[2] / cell)))

    def ok(p):
        if p[0] * p[0] + p[1] * p[1] + p[2] * p[2] > R * R:
            return False
        k = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        d = pts[j] - p
                        if d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < min_sep * min_sep:
                            return False
        return True

    def add(i, p):
        pts[i] = p
        grid.setdefault(key(p), []).append(i)

    def trial(j):
        v = rng.normal(size=3)
        return pts[j] + v * (step / np.linalg.norm(v))

    add(0, np.zeros(3))
    i = 1
    while i < n:
        placed = False
        for _ in range(64):
            p = trial(i - 1)
            if ok(p):
                placed = True
                break
        if not placed:
            for _ in range(4096):
                p = trial(int(rng.integers(0, i)))
                if ok(p):
                    placed = True
                    break
        if placed:
            add(i, p)
            i += 1
        else:
            R *= 1.02
    return pts


def golden_sphere(npts):
    k = np.arange(npts) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / npts)
    theta = np.pi * (1.0 + 5 ** 0.5) * k
    return np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=1)


def sasa_fraction(xyz, radii, probe=1.4, npts=240, sph=None):
    """Shrake-Rupley accessible fraction per atom (0 for zero radius); the
    distances are summed x, y, z in that order, as the GPU kernel does."""
    n = len(xyz)
    rr = radii + probe
    sph = golden_sphere(npts) if sph is None else np.asarray(sph, dtype=np.float64)
    npts = len(sph)
    out = np.zeros(n)
    cut = 2.0 * rr.max()
    cell = {}
    keys = np.floor(xyz / cut).astype(int)
    for i, k in enumerate(map(tuple, keys)):
        cell.setdefault(k, []).append(i)
    for i in range(n):
        if radii[i] <= 0:
            continue
        k = keys[i]
        nb = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    nb.extend(cell.get((k[0] + dx, k[1] + dy, k[2] + dz), ()))
        nb = np.array([j for j in nb if j != i], dtype=int)
        p = xyz[i] + rr[i] * sph
        free = np.ones(npts, dtype=bool)
        if len(nb):
            d = xyz[nb] - xyz[i]
            dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
            close = nb[dist < rr[i] + rr[nb]]
            for j in close:
                dd = p - xyz[j]
                free &= dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1] + dd[:, 2] * dd[:, 2] >= rr[j] * rr[j]
        out[i] = free.mean()
    return out


class Molecule:
    def __init__(self, xyz, elements):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.elements = list(elements)
        self.res = [ELEMENT_NAMES[e][0] for e in self.elements]
        self.atom = [ELEMENT_NAMES[e][1] for e in self.elements]
        self.radius = np.array([ELEMENT_RADIUS[e] for e in self.elements])
        self.sasa = None

    @property
    def natoms(self):
        return len(self.elements)

    def center_of_extrema(self):
        return 0.5 * (self.xyz.min(axis=0) + self.xyz.max(axis=0))

    def centroid(self):
        return self.xyz.mean(axis=0)

    def translated(self, t):
        """A copy moved by t (accessible fractions are unchanged by a
        rigid move and are carried over)."""
        m = Molecule(self.xyz + np.asarray(t), self.elements)
        m.sasa = None if self.sasa is None else self.sasa.copy()
        return m

    def with_sasa(self, probe=1.4, npts=240):
        self.sasa = sasa_fraction(self.xyz, self.radius, probe, npts)
        return self


def make_molecule(natoms, rg, seed):
    rng = np.random.default_rng(seed)
    xyz = random_walk_chain(natoms, rg, rng)
    el = rng.choice(len(ELEMENTS), size=natoms, p=ELEMENT_P)
    return Molecule(xyz, [ELEMENTS[i] for i in el])


def join(a, b):
    m = Molecule(np.concatenate([a.xyz, b.xyz]), a.elements + b.elements)
    return m


def random_rotations(n, rng):
    """Uniform SO(3) rotation matrices (row-major 3x3) from unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def random_translations(n, tmin, tmax, rng):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.uniform(tmin, tmax, size=n)
    return d * r[:, None]


def round3(x):
    """The 3-decimal text round trip of the Euler file (index.c:114-116 writes
    "% .3f"; correlate.c:215-217 reads it back)."""
    return float("%.3f" % x)


def poses_to_indices(R, T, ref_lig, zvals, L, ft2euler, assemble_index):
    """Grid indices of poses (rotation R[i] of the ligand, translation T[i]),
    exactly as correlate does: Euler angles by ft2euler, written and read back
    with 3 decimals, z matched to zvals within 1e-3, index assembly.  Poses
    whose z is not in zvals are dropped (returned mask)."""
    idx = []
    keep = []
    zv = np.asarray(zvals)
    for i in range(len(R)):
        eu = ft2euler(T[i], R[i].reshape(9), ref_lig)
        eu = np.array([round3(v) for v in eu])
        j = np.nonzero((zv > eu[0] - 0.001) & (zv < eu[0] + 0.001))[0]
        if len(j) == 0:
            keep.append(False)
            continue
        idx.append(assemble_index(eu, int(j[0]), L))
        keep.append(True)
    return np.array(idx, dtype=np.int32), np.array(keep)


def noisy_experiment(q, intensity, rel_noise, rng):
    """I_exp = I (1 + rel_noise * N(0,1)), sigma = rel_noise * I."""
    i = intensity * (1.0 + rel_noise * rng.normal(size=len(intensity)))
    return np.array(q, dtype=np.float64), i, rel_noise * np.asarray(intensity)


def cgrid(lo, hi, n):
    """Fit-grid values lo + k*step (k = 0..n-1), step = (hi-lo)/(n-1)."""
    step = (hi - lo) / (n - 1)
    return np.array([lo + k * step for k in range(n)])


# The fit grid of the benchmark configurations: c1 in [0.95, 1.05] step 0.01,
# c2 in [0, 4] step 0.1.
C1_GRID = cgrid(0.95, 1.05, 11)
C2_GRID = cgrid(0.0, 4.0, 41)
