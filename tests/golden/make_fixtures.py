"""Generate reference fixtures for the GPU parity tests.

Runs the reference's own FP64 CPU force (oracle/_ref, built from the reference tree by
oracle/Makefile) on seeded synthetic systems and stores inputs and outputs as .npz:

* water648_{direct,mutual,extrapolated}.npz -- 216 rigid waters in an 18.64 A box, PME
  cutoff 0.8 nm, alpha 3.5 /nm, 24^3 grid, B-spline order 6 (the only order the
  reference implements), mutual target 1e-9 D;
* frames_{direct,mutual,extrapolated}.npz -- 40 four-atom molecules whose central atoms
  cycle through ZBisect, ThreeFold, Bisector, ZOnly and ZThenX frames with a chiral Y
  atom, anisotropic polarisabilities, 1-4 partners with scale 0.5, in a 2.2 nm box.

* properties_{water648_pme,frames_pme,frames_nocutoff}.npz -- the reference's
  getSystemMultipoleMoments and getElectrostaticPotential (64 seeded points) with
  seeded masses.

* triclinic_{direct,mutual,extrapolated}.npz -- the water box in a reduced triclinic
  cell (all three off-diagonal box entries non-zero).

* converged_water648_{full,nooctopoles}.npz -- the water box (Mutual, 1e-11 D) on a
  128^3 grid at the reference's order 6, where its PME has converged to the Ewald sum
  to ~1e-7 in forces: the target that order-5 PME must approach as its grid is refined
  (the second variant with the octopoles set to zero).

Usage:  python tests/golden/make_fixtures.py [properties | triclinic | converged]   (needs the reference tree)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import oracle as O  # noqa: E402
from mpidopenmmplugin_gb300 import MPIDForce, synthetic  # noqa: E402
import helpers  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
POL = {0: "mutual", 1: "direct", 2: "extrapolated"}


def frames_system(seed=7):
    rng = np.random.default_rng(seed)
    nmol, L = 40, 2.2
    f = MPIDForce()
    pos = []
    side = 4
    spacing = L / side
    axes = [MPIDForce.ZBisect, MPIDForce.ThreeFold, MPIDForce.Bisector, MPIDForce.ZOnly, MPIDForce.ZThenX]
    for m in range(nmol):
        c = np.array([(m // 16) % side, (m // 4) % side, m % side]) * spacing + 0.25 + rng.uniform(-0.03, 0.03, 3)
        R = synthetic._random_rotations(rng, 1)[0]
        # pyramidal X-H3 geometry, 0.1 nm bonds
        local = np.array([[0, 0, 0], [0.1, 0, 0.03], [-0.05, 0.0866, 0.03], [-0.05, -0.0866, 0.03]])
        xyz = c + local @ R.T
        base = 4 * m
        pos.extend(xyz)
        ax = axes[m % len(axes)]
        dip = rng.normal(0, 0.01, (4, 3))
        quad = synthetic.traceless_quadrupole(rng, 5e-4, 4)
        octo = synthetic.traceless_octopole(rng, 2e-5, 4)
        aniso = rng.uniform(0.5e-3, 2e-3, 3)
        z, x, y = base + 1, base + 2, base + 3
        if ax == MPIDForce.ZOnly:
            x, y = -1, -1
        elif ax in (MPIDForce.Bisector,):
            y = -1
        f.addMultipole(rng.normal(0, 0.3), dip[0], quad[0], octo[0], ax, z, x, y, 0.6, aniso)
        for h in range(1, 4):
            others = [base + k for k in range(1, 4) if k != h]
            f.addMultipole(rng.normal(0, 0.2), dip[h], quad[h], octo[h], MPIDForce.ZThenX, base, others[0],
                           others[1], 0.6, [0.4e-3] * 3)
        f.setCovalentMap(base, MPIDForce.Covalent12, [base + 1, base + 2, base + 3])
        for h in range(1, 4):
            f.setCovalentMap(base + h, MPIDForce.Covalent12, [base])
            f.setCovalentMap(base + h, MPIDForce.Covalent13, [base + k for k in range(1, 4) if k != h])
        # neighbouring molecule as 1-4 partners of the central atom
        if m + 1 < nmol:
            f.setCovalentMap(base, MPIDForce.Covalent14, [base + 4])
    f.setNonbondedMethod(MPIDForce.PME)
    f.setCutoffDistance(0.7)
    f.setPMEParameters(3.8, 24, 24, 24)
    f.setDefaultTholeWidth(1.1)
    f.set14ScaleFactor(0.5)
    return f, np.array(pos), np.diag([L, L, L])


def save(name, s, res, **extra):
    n = s.n
    offs = [0]
    idx = []
    for i in range(n):
        for t in range(8):
            lst = s.covalent[i][t] if t < len(s.covalent[i]) else []
            idx.extend(lst)
            offs.append(len(idx))
    np.savez_compressed(
        os.path.join(OUT, name), pos=s.pos, charge=s.charge, dipole=s.dipole, quadrupole=s.quadrupole,
        octopole=s.octopole, thole=s.thole, polarity=s.polarity, axis_type=s.axis_type, atom_z=s.atom_z,
        atom_x=s.atom_x, atom_y=s.atom_y, cov_offsets=np.array(offs, np.int32),
        cov_index=np.array(idx if idx else [0], np.int32), box=s.box, nonbonded_method=s.nonbonded_method,
        polarization_type=s.polarization_type, cutoff=s.cutoff, ewald_alpha=s.ewald_alpha, grid=np.array(s.grid),
        pme_order=s.pme_order, mutual_eps=s.mutual_eps, max_iter=s.max_iter,
        extrap_coeffs=np.array(s.extrap_coeffs), default_thole=s.default_thole, scale14=s.scale14,
        ref_energy=res.energy, ref_forces=res.forces, ref_induced=res.induced, ref_labdipoles=res.labdipoles,
        ref_iterations=res.iterations, **extra)
    print("wrote", name, "E =", res.energy, "iterations", res.iterations)


def main():
    O.build("ref")
    for pol in (1, 0, 2):
        f, pos, box = synthetic.workload("water648", polarization=pol, order=6)
        f.setMutualInducedTargetEpsilon(1e-9)
        s = helpers.oracle_system(f, pos, box, pme_order=6)
        save("water648_%s.npz" % POL[pol], s, O.evaluate(s, "ref", want_labdipoles=True))
        f, pos, box = frames_system()
        f.setPolarizationType(pol)
        f.setMutualInducedTargetEpsilon(1e-9)
        f.setMutualInducedMaxIterations(200)
        s = helpers.oracle_system(f, pos, box, pme_order=6)
        save("frames_%s.npz" % POL[pol], s, O.evaluate(s, "ref", want_labdipoles=True))


def make_properties():
    """properties_*.npz: the reference's getSystemMultipoleMoments and
    getElectrostaticPotential (at 64 seeded points in the box) for the water box (PME)
    and the frames system (PME and no cutoff), with seeded masses."""
    O.build("ref")
    rng = np.random.default_rng(11)
    cases = []
    f, pos, box = synthetic.workload("water648", polarization=0, order=6)
    cases.append(("water648_pme", f, pos, box, np.tile([15.999, 1.008, 1.008], f.getNumMultipoles() // 3)))
    for method, tag in ((1, "pme"), (0, "nocutoff")):
        f, pos, box = frames_system()
        f.setNonbondedMethod(method)
        f.setPolarizationType(0)
        f.setMutualInducedMaxIterations(200)
        cases.append(("frames_" + tag, f, pos, box, rng.uniform(1.0, 16.0, size=f.getNumMultipoles())))
    for name, f, pos, box, masses in cases:
        f.setMutualInducedTargetEpsilon(1e-9)
        s = helpers.oracle_system(f, pos, box, pme_order=6)
        grid = rng.uniform(0.0, 1.0, size=(64, 3)) * np.diag(box)
        moments, potential = O.properties(s, masses, grid)
        save("properties_%s.npz" % name, s, O.evaluate(s, "ref", want_labdipoles=True), masses=masses, grid_points=grid,
             ref_moments=moments, ref_potential=potential)


def triclinic_water(pol):
    """The water648 system in a reduced triclinic cell: a = (L, 0, 0), b = (0.25 L,
    0.97 L, 0), c = (-0.2 L, 0.3 L, 0.95 L), L = 1.864 nm; each oxygen keeps its
    fractional coordinates, the hydrogens their offsets from it."""
    f, pos, box = synthetic.workload("water648", polarization=pol, order=6)
    L = box[0, 0]
    cell = np.array([[L, 0, 0], [0.25 * L, 0.97 * L, 0], [-0.2 * L, 0.3 * L, 0.95 * L]])
    o = pos[0::3]
    newo = (o / L) @ cell
    out = pos.copy()
    for k in range(3):
        out[k::3] = pos[k::3] - o + newo
    return f, out, cell


def make_triclinic():
    """triclinic_{direct,mutual,extrapolated}.npz: the reference on triclinic_water."""
    O.build("ref")
    for pol in (1, 0, 2):
        f, pos, box = triclinic_water(pol)
        f.setMutualInducedTargetEpsilon(1e-9)
        s = helpers.oracle_system(f, pos, box, pme_order=6)
        save("triclinic_%s.npz" % POL[pol], s, O.evaluate(s, "ref", want_labdipoles=True))


def converged_water(variant):
    """The water648 box (Mutual) with tight solver tolerance; variant "nooctopoles" sets
    every octopole to zero."""
    f, pos, box = synthetic.workload("water648", polarization=0, order=6)
    f.setMutualInducedTargetEpsilon(1e-11)
    f.setMutualInducedMaxIterations(500)
    s = helpers.oracle_system(f, pos, box, pme_order=6)
    if variant == "nooctopoles":
        s.octopole = np.zeros_like(s.octopole)
    return s


def make_converged():
    """converged_water648_{full,nooctopoles}.npz: the reference at order 6 on 128^3."""
    O.build("ref")
    for variant in ("full", "nooctopoles"):
        s = converged_water(variant)
        s.grid = (128, 128, 128)
        save("converged_water648_%s.npz" % variant, s, O.evaluate(s, "ref", want_labdipoles=True))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "converged":
        make_converged()
    elif len(sys.argv) > 1 and sys.argv[1] == "properties":
        make_properties()
    elif len(sys.argv) > 1 and sys.argv[1] == "triclinic":
        make_triclinic()
    else:
        main()
