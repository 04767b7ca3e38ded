"""Shared test helpers: convert product-side systems to the oracle's flat form, error
metrics, and the golden fixture loader."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def oracle_system(force, pos, box, pme_order=None):
    """OracleSystem of an MPIDForce (mpidopenmmplugin_gb300.force) with positions/box in nm."""
    a = force.arrays()
    n = force.getNumMultipoles()
    cov = [force.getCovalentMaps(i) for i in range(n)]
    alpha, nx, ny, nz = force.getPMEParameters()
    return O.OracleSystem(
        pos=np.asarray(pos, dtype=np.float64), charge=a["charge"], dipole=a["dipole"], quadrupole=a["quadrupole"],
        octopole=a["octopole"], thole=a["thole"], polarity=a["polarity"], axis_type=a["axis_type"],
        atom_z=a["atom_z"], atom_x=a["atom_x"], atom_y=a["atom_y"], covalent=cov,
        box=np.asarray(box, dtype=np.float64).reshape(3, 3), nonbonded_method=force.getNonbondedMethod(),
        polarization_type=force.getPolarizationType(), cutoff=force.getCutoffDistance(), ewald_alpha=alpha,
        grid=(nx, ny, nz), pme_order=pme_order or force.getPmeBSplineOrder(),
        mutual_eps=force.getMutualInducedTargetEpsilon(), max_iter=force.getMutualInducedMaxIterations(),
        extrap_coeffs=tuple(force.getExtrapolationCoefficients()), default_thole=force.getDefaultTholeWidth(),
        scale14=force.get14ScaleFactor())


def force_from_oracle_system(s):
    """MPIDForce from an OracleSystem (for the reference's own fixtures)."""
    from mpidopenmmplugin_gb300 import MPIDForce
    f = MPIDForce()
    for i in range(s.n):
        f.addMultipole(s.charge[i], s.dipole[i], s.quadrupole[i], s.octopole[i], int(s.axis_type[i]), int(s.atom_z[i]),
                       int(s.atom_x[i]), int(s.atom_y[i]), s.thole[i], s.polarity[i])
        for t in range(8):
            if t < len(s.covalent[i]) and s.covalent[i][t]:
                f.setCovalentMap(i, t, s.covalent[i][t])
    f.setNonbondedMethod(s.nonbonded_method)
    f.setPolarizationType(s.polarization_type)
    f.setCutoffDistance(s.cutoff)
    f.setPMEParameters(s.ewald_alpha, *s.grid)
    f.setPmeBSplineOrder(s.pme_order if s.nonbonded_method == 1 else 6)
    f.setMutualInducedTargetEpsilon(s.mutual_eps)
    f.setMutualInducedMaxIterations(s.max_iter)
    f.setExtrapolationCoefficients(list(s.extrap_coeffs))
    f.setDefaultTholeWidth(s.default_thole)
    f.set14ScaleFactor(s.scale14)
    return f


def rel_rms(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))


def load_reference_tests():
    return json.load(open(os.path.join(GOLDEN_DIR, "reference_tests.json")))


def load_npz_fixture(name):
    path = os.path.join(GOLDEN_DIR, name)
    return dict(np.load(path, allow_pickle=False))


def system_from_fixture(fx):
    """OracleSystem stored in a make_fixtures.py .npz (arrays + scalar settings)."""
    n = int(fx["charge"].shape[0])
    offs = fx["cov_offsets"]
    idx = fx["cov_index"]
    cov = [[list(idx[offs[8 * i + t]:offs[8 * i + t + 1]]) for t in range(8)] for i in range(n)]
    return O.OracleSystem(
        pos=fx["pos"], charge=fx["charge"], dipole=fx["dipole"], quadrupole=fx["quadrupole"], octopole=fx["octopole"],
        thole=fx["thole"], polarity=fx["polarity"], axis_type=fx["axis_type"], atom_z=fx["atom_z"],
        atom_x=fx["atom_x"], atom_y=fx["atom_y"], covalent=cov, box=fx["box"],
        nonbonded_method=int(fx["nonbonded_method"]), polarization_type=int(fx["polarization_type"]),
        cutoff=float(fx["cutoff"]), ewald_alpha=float(fx["ewald_alpha"]), grid=tuple(int(v) for v in fx["grid"]),
        pme_order=int(fx["pme_order"]), mutual_eps=float(fx["mutual_eps"]), max_iter=int(fx["max_iter"]),
        extrap_coeffs=tuple(float(v) for v in fx["extrap_coeffs"]), default_thole=float(fx["default_thole"]),
        scale14=float(fx["scale14"]))
