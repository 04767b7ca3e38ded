"""Seeded synthetic MPID systems with the shapes of the benchmark configurations.

Water boxes:

Rigid 3-site waters (O-H 0.9572 A, H-O-H 104.52 deg) at random orientations on a
jittered cubic lattice; Z-then-X frames (O: z -> H1, x -> H2; H: z -> O, x -> the other
H); charges O -0.834, H +0.417; dipoles, quadrupoles and octopoles drawn per atom from
N(0, 0.1 / 0.05 / 0.02 e A^n) and projected traceless; isotropic polarisability 1.0 A^3
(O) and 0.3 A^3 (H); Thole width 1.3 (default width 1.3, per-atom 0.65 so that excluded
pairs also use 1.3); intramolecular 1-2 and 1-3 pairs excluded.

Solution (waters plus ethane-like solutes): staggered C2H6 (C-C 1.53 A, C-H 1.09 A,
tetrahedral angles) at random orientations on lattice sites whose 18 face and edge
neighbours are left empty; charges C -0.18, H +0.06; dipoles, quadrupoles and octopoles from
N(0, 0.15 / 0.08 / 0.03 e A^n); anisotropic polarisabilities with local-frame diagonal
U[0.5, 2.0] A^3 (the API takes the diagonal in the local frame); per-atom Thole widths
U[0.5, 1], so that the pair widths a_i + a_j of excluded pairs lie in U[1, 2];
1-2 and 1-3 pairs excluded, 1-4 pairs scaled by 0.5.

Units are converted to nm / e nm^k / nm^3.  Nothing here runs on the evaluation path.
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


_THETA = np.deg2rad(104.52)
_ROH = 0.9572
_H1 = np.array([_ROH * np.sin(_THETA / 2), 0.0, _ROH * np.cos(_THETA / 2)])
_H2 = np.array([-_ROH * np.sin(_THETA / 2), 0.0, _ROH * np.cos(_THETA / 2)])


def _random_waters(rng, n, L, min_oo=2.6, min_atom=1.6, batch=64, rounds=2000):
    """Random sequential placement of n rigid waters in a periodic cube of edge L (A):
    each new water (uniform O position, random orientation) is kept when its O is at least
    min_oo from every other O and all its atoms at least min_atom from every atom of the
    other waters.  Candidates are drawn `batch` at a time; the first admissible one is
    kept.  Returns O positions (n, 3) and rotations (n, 3, 3)."""
    O = np.zeros((n, 3))
    R = np.zeros((n, 3, 3))
    atoms = np.zeros((3 * n, 3))
    for w in range(n):
        for _ in range(rounds):
            o = rng.uniform(0.0, L, size=(batch, 3))
            rot = _random_rotations(rng, batch)
            if w:
                d = O[None, :w, :] - o[:, None, :]
                d -= L * np.round(d / L)
                ok = np.min(np.einsum("kij,kij->ki", d, d), axis=1) >= min_oo ** 2
                if not ok.any():
                    continue
                o, rot = o[ok], rot[ok]
                k = -1
                for c in range(len(o)):  # atom check against the waters within reach
                    d = O[:w] - o[c]
                    d -= L * np.round(d / L)
                    near = np.flatnonzero(np.einsum("ij,ij->i", d, d) < (min_atom + 2.0 * _ROH + 0.01) ** 2)
                    mine = np.stack([o[c], o[c] + rot[c] @ _H1, o[c] + rot[c] @ _H2])
                    other = atoms[(3 * near[:, None] + np.arange(3)).reshape(-1)]
                    d = other[None, :, :] - mine[:, None, :]
                    d -= L * np.round(d / L)
                    if len(other) == 0 or np.min(np.einsum("aij,aij->ai", d, d)) >= min_atom ** 2:
                        k = c
                        break
                if k < 0:
                    continue
            else:
                k = 0
            O[w], R[w] = o[k], rot[k]
            atoms[3 * w:3 * w + 3] = [o[k], o[k] + rot[k] @ _H1, o[k] + rot[k] @ _H2]
            break
        else:
            raise RuntimeError("could not place water %d of %d in a %.2f A box" % (w, n, L))
    return O, R


def water_box(n_waters, box_angstrom, seed=2024, lattice=None, mult_sigma=(0.1, 0.05, 0.02), placement="lattice"):
    """Return (force, positions_nm (n,3), box_nm (3,3)) for n_waters waters.  placement
    "lattice" puts the oxygens on a jittered cubic lattice (sites drawn at random when
    n_waters is not a cube); "random" places the waters one by one at random with minimum
    O-O (2.6 A) and atom-atom (1.6 A) distances between molecules."""
    rng = np.random.default_rng(seed)
    L = box_angstrom
    if placement == "random":
        O, R = _random_waters(rng, n_waters, L)
    else:
        side = lattice or int(np.ceil(round(n_waters ** (1.0 / 3.0), 6)))
        sites = np.array([(i, j, k) for i in range(side) for j in range(side) for k in range(side)], dtype=np.float64)
        if len(sites) > n_waters:
            sites = sites[np.sort(rng.choice(len(sites), n_waters, replace=False))]
        spacing = L / side
        jitter = 0.12  # A; with >= 3.08 A spacing every O-O distance stays >= 2.6 A
        O = (sites + 0.5) * spacing + rng.uniform(-jitter, jitter, size=sites.shape)
        R = _random_rotations(rng, n_waters)
    H1 = O + R @ _H1
    H2 = O + R @ _H2
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


def _ethane(rng):
    """Atom positions (A, 8 x 3: C1, C2, H11..H13, H21..H23) of a staggered ethane at the
    origin, randomly oriented."""
    cc, ch = 1.53, 1.09
    tet = np.deg2rad(109.47)
    c1 = np.array([0.0, 0.0, -cc / 2])
    c2 = np.array([0.0, 0.0, cc / 2])
    h = []
    for k in range(3):
        phi = 2 * np.pi * k / 3
        h.append(c1 + ch * np.array([np.sin(tet) * np.cos(phi), np.sin(tet) * np.sin(phi), np.cos(tet)]))
    for k in range(3):
        phi = 2 * np.pi * k / 3 + np.pi / 3  # staggered
        h.append(c2 + ch * np.array([np.sin(tet) * np.cos(phi), np.sin(tet) * np.sin(phi), -np.cos(tet)]))
    xyz = np.array([c1, c2] + h)
    R = _random_rotations(rng, 1)[0]
    return xyz @ R.T


def solution_box(n_waters, n_solutes, box_angstrom, seed=2024):
    """Return (force, positions_nm, box_nm) for n_waters waters and n_solutes ethanes."""
    rng = np.random.default_rng(seed)
    L = box_angstrom
    side = int(np.ceil((n_waters + 19 * n_solutes) ** (1.0 / 3.0)))
    spacing = L / side
    idx = np.arange(side ** 3)
    sites = np.stack(np.unravel_index(idx, (side, side, side)), axis=1)
    # solute sites with their 18 face and edge neighbours left empty
    taken = np.zeros(side ** 3, dtype=bool)
    solutes = []
    for cand in rng.permutation(side ** 3):
        if len(solutes) == n_solutes:
            break
        i, j, k = sites[cand]
        nb = [((i + di) % side, (j + dj) % side, (k + dk) % side)
              for di in (-1, 0, 1) for dj in (-1, 0, 1) for dk in (-1, 0, 1) if abs(di) + abs(dj) + abs(dk) <= 2]
        nbi = [np.ravel_multi_index(t, (side, side, side)) for t in nb]
        if taken[nbi].any():
            continue
        taken[nbi] = True
        solutes.append(cand)
    free = np.flatnonzero(~taken)
    water_sites = np.sort(rng.choice(free, n_waters, replace=False))
    jitter = 0.12
    fw, pw, _ = water_box(n_waters, L, seed=seed + 1)
    # move the waters of water_box onto the free sites (keep their internal geometry)
    O_old = pw[0::3] / ANG
    O_new = (sites[water_sites] + 0.5) * spacing + rng.uniform(-jitter, jitter, size=(n_waters, 3))
    shift = np.repeat(O_new - O_old, 3, axis=0)
    pos_w = pw / ANG + shift
    f = fw
    pos = [pos_w]
    nw = 3 * n_waters
    sig = (0.15, 0.08, 0.03)
    for m, site in enumerate(solutes):
        centre = (sites[site] + 0.5) * spacing
        xyz = centre + _ethane(rng)
        pos.append(xyz)
        base = nw + 8 * m
        c1, c2 = base, base + 1
        hs1, hs2 = [base + 2, base + 3, base + 4], [base + 5, base + 6, base + 7]
        dip = rng.normal(0.0, sig[0] * ANG, size=(8, 3))
        quad = traceless_quadrupole(rng, sig[1] * ANG ** 2, 8)
        octo = traceless_octopole(rng, sig[2] * ANG ** 3, 8)
        pol = rng.uniform(0.5, 2.0, size=(8, 3)) * ANG ** 3
        thole = rng.uniform(0.5, 1.0, size=8)  # per atom: pair widths a_i + a_j in U[1, 2]
        frames = [(c2, hs1[0]), (c1, hs2[0])] + [(c1, c2)] * 3 + [(c2, c1)] * 3
        charges = [-0.18, -0.18] + [0.06] * 6
        for a in range(8):
            z, x = frames[a]
            f.addMultipole(charges[a], dip[a], quad[a], octo[a], MPIDForce.ZThenX, z, x, -1, thole[a], pol[a])
        f.setCovalentMap(c1, MPIDForce.Covalent12, [c2] + hs1)
        f.setCovalentMap(c1, MPIDForce.Covalent13, hs2)
        f.setCovalentMap(c2, MPIDForce.Covalent12, [c1] + hs2)
        f.setCovalentMap(c2, MPIDForce.Covalent13, hs1)
        for hs, own, other, other_h in ((hs1, c1, c2, hs2), (hs2, c2, c1, hs1)):
            for h in hs:
                f.setCovalentMap(h, MPIDForce.Covalent12, [own])
                f.setCovalentMap(h, MPIDForce.Covalent13, [other] + [g for g in hs if g != h])
                f.setCovalentMap(h, MPIDForce.Covalent14, other_h)
    f.set14ScaleFactor(0.5)
    box = np.diag([L * ANG] * 3)
    return f, np.concatenate(pos) * ANG, box


# Benchmark workloads (BASELINE configurations), sizes in the units above.
WORKLOADS = {
    # 216 waters, 18.64 A, cutoff 8 A, alpha 0.35 /A, 24^3 grid, order 5, mutual 1e-7 D
    "water648": dict(n_waters=216, box=18.64, cutoff=0.8, alpha=3.5, grid=24, order=5, eps=1e-7),
    # 8,000 waters, 62.14 A, cutoff 9 A, alpha 0.34 /A, 72^3 grid, order 5, mutual 1e-7 D
    "water24k": dict(n_waters=8000, box=62.14, cutoff=0.9, alpha=3.4, grid=72, order=5, eps=1e-7),
    # 96,000 waters, 142.0 A, cutoff 9 A, alpha 0.34 /A, 144^3 grid, order 5, mutual 1e-6 D
    "water288k": dict(n_waters=96000, box=142.0, cutoff=0.9, alpha=3.4, grid=144, order=5, eps=1e-6),
    # 20,000 waters + 200 ethanes (61,600 atoms), 85.3 A, 96^3 grid; cutoff and alpha not
    # stated by the configuration: 9 A and 0.34 /A; order 5, mutual 1e-7 D
    "solution61k": dict(n_waters=20000, n_solutes=200, box=85.3, cutoff=0.9, alpha=3.4, grid=96, order=5, eps=1e-7),
}


def workload(name, polarization=MPIDForce.Mutual, order=None, seed=2024, max_iter=200):
    """Configured force, positions (nm) and box (nm) of a named workload."""
    w = WORKLOADS[name]
    if w.get("n_solutes"):
        f, pos, box = solution_box(w["n_waters"], w["n_solutes"], w["box"], seed=seed)
    else:
        f, pos, box = water_box(w["n_waters"], w["box"], seed=seed)
    f.setNonbondedMethod(MPIDForce.PME)
    f.setCutoffDistance(w["cutoff"])
    f.setPMEParameters(w["alpha"], w["grid"], w["grid"], w["grid"])
    f.setPmeBSplineOrder(order or w["order"])
    f.setPolarizationType(polarization)
    f.setMutualInducedTargetEpsilon(w["eps"])
    f.setMutualInducedMaxIterations(max_iter)
    return f, pos, box
