"""Seeded synthetic MPID systems with the shapes of the benchmark configurations.

Rigid 3-site waters (O-H 0.9572 A, H-O-H 104.52 deg) at random orientations on a
jittered cubic lattice; Z-then-X frames (O: z -> H1, x -> H2; H: z -> O, x -> the other
H); charges O -0.834, H +0.417; dipoles, quadrupoles and octopoles drawn per atom from
N(0, 0.1 / 0.05 / 0.02 e A^n) and projected traceless; isotropic polarisability 1.0 A^3
(O) and 0.3 A^3 (H); Thole width 1.3 (default width 1.3, per-atom 0.65 so that excluded
pairs also use 1.3); intramolecular 1-2 and 1-3 pairs excluded.  Units are converted to
nm / e nm^k / nm^3.  Nothing here runs on the evaluation path.
"""
import numpy as np

from .force import MPIDForce

ANG = 0.1  # nm per Angstrom


def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def traceless_quadrupole(rng, sigma, n):
    """(n, 6) in MPIDForce order XX XY YY XZ YZ ZZ."""
    a = rng.normal(0.0, sigma, size=(n, 6))
    tr = (a[:, 0] + a[:, 2] + a[:, 5]) / 3.0
    a[:, 0] -= tr
    a[:, 2] -= tr
    a[:, 5] -= tr
    return a


# MPIDForce octopole order XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ as index triples
_OCT = [(0, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (0, 0, 2), (0, 1, 2), (1, 1, 2), (0, 2, 2), (1, 2, 2), (2, 2, 2)]


def traceless_octopole(rng, sigma, n):
    """(n, 10) symmetric traceless octopoles: O' = O - (1/5)(d_ij t_k + d_ik t_j + d_jk t_i)."""
    a = rng.normal(0.0, sigma, size=(n, 10))
    full = np.zeros((n, 3, 3, 3))
    import itertools
    for c, (i, j, k) in enumerate(_OCT):
        for p in set(itertools.permutations((i, j, k))):
            full[:, p[0], p[1], p[2]] = a[:, c]
    t = np.einsum("nijj->ni", full)
    d = np.eye(3)
    corr = (np.einsum("ij,nk->nijk", d, t) + np.einsum("ik,nj->nijk", d, t) + np.einsum("jk,ni->nijk", d, t)) / 5.0
    full -= corr
    return np.stack([full[:, i, j, k] for (i, j, k) in _OCT], axis=1)


def water_box(n_waters, box_angstrom, seed=2024, lattice=None, mult_sigma=(0.1, 0.05, 0.02)):
    """Return (force, positions_nm (n,3), box_nm (3,3)) for n_waters waters."""
    rng = np.random.default_rng(seed)
    L = box_angstrom
    side = lattice or int(np.ceil(round(n_waters ** (1.0 / 3.0), 6)))
    sites = np.array([(i, j, k) for i in range(side) for j in range(side) for k in range(side)], dtype=np.float64)
    if len(sites) > n_waters:
        sites = sites[np.sort(rng.choice(len(sites), n_waters, replace=False))]
    spacing = L / side
    jitter = 0.12  # A; with >= 3.08 A spacing every O-O distance stays >= 2.6 A
    O = (sites + 0.5) * spacing + rng.uniform(-jitter, jitter, size=sites.shape)
    theta = np.deg2rad(104.52)
    roh = 0.9572
    h1 = np.array([roh * np.sin(theta / 2), 0.0, roh * np.cos(theta / 2)])
    h2 = np.array([-roh * np.sin(theta / 2), 0.0, roh * np.cos(theta / 2)])
    R = _random_rotations(rng, n_waters)
    H1 = O + R @ h1
    H2 = O + R @ h2
    pos = np.empty((3 * n_waters, 3))
    pos[0::3], pos[1::3], pos[2::3] = O, H1, H2
    pos *= ANG
    n = 3 * n_waters
    dip = rng.normal(0.0, mult_sigma[0] * ANG, size=(n, 3))
    quad = traceless_quadrupole(rng, mult_sigma[1] * ANG ** 2, n)
    octo = traceless_octopole(rng, mult_sigma[2] * ANG ** 3, n)
    f = MPIDForce()
    f.setDefaultTholeWidth(1.3)
    for w in range(n_waters):
        o, a, b = 3 * w, 3 * w + 1, 3 * w + 2
        for atom, q, z, x, alpha in ((o, -0.834, a, b, 1.0), (a, 0.417, o, b, 0.3), (b, 0.417, o, a, 0.3)):
            al = alpha * ANG ** 3
            f.addMultipole(q, dip[atom], quad[atom], octo[atom], MPIDForce.ZThenX, z, x, -1, 0.65, [al, al, al])
        f.setCovalentMap(o, MPIDForce.Covalent12, [a, b])
        f.setCovalentMap(a, MPIDForce.Covalent12, [o])
        f.setCovalentMap(a, MPIDForce.Covalent13, [b])
        f.setCovalentMap(b, MPIDForce.Covalent12, [o])
        f.setCovalentMap(b, MPIDForce.Covalent13, [a])
    box = np.diag([L * ANG] * 3)
    return f, pos, box


# Benchmark workloads (BASELINE configurations), sizes in the units above.
WORKLOADS = {
    # 216 waters, 18.64 A, cutoff 8 A, alpha 0.35 /A, 24^3 grid, order 5, mutual 1e-7 D
    "water648": dict(n_waters=216, box=18.64, cutoff=0.8, alpha=3.5, grid=24, order=5, eps=1e-7),
    # 8,000 waters, 62.14 A, cutoff 9 A, alpha 0.34 /A, 72^3 grid, order 5, mutual 1e-7 D
    "water24k": dict(n_waters=8000, box=62.14, cutoff=0.9, alpha=3.4, grid=72, order=5, eps=1e-7),
    # 96,000 waters, 142.0 A, cutoff 9 A, alpha 0.34 /A, 144^3 grid, order 5, mutual 1e-6 D
    "water288k": dict(n_waters=96000, box=142.0, cutoff=0.9, alpha=3.4, grid=144, order=5, eps=1e-6),
}


def workload(name, polarization=MPIDForce.Mutual, order=None, seed=2024, max_iter=200):
    """Configured force, positions (nm) and box (nm) of a named workload."""
    w = WORKLOADS[name]
    f, pos, box = water_box(w["n_waters"], w["box"], seed=seed)
    f.setNonbondedMethod(MPIDForce.PME)
    f.setCutoffDistance(w["cutoff"])
    f.setPMEParameters(w["alpha"], w["grid"], w["grid"], w["grid"])
    f.setPmeBSplineOrder(order or w["order"])
    f.setPolarizationType(polarization)
    f.setMutualInducedTargetEpsilon(w["eps"])
    f.setMutualInducedMaxIterations(max_iter)
    return f, pos, box
