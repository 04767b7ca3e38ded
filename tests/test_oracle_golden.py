"""Pin the CPU oracles to the reference's own known-answer tests.

The 18 cases (14 test functions, the two 1-4 scaling tests holding three systems each)
come from platforms/reference/tests/TestReferenceMPIDForce.cpp, extracted as text by
tests/golden/extract_reference_tests.py.  Tolerances are the ones those tests assert:
energy 1e-4 relative (1e-5 / 1e-3 absolute-or-relative for the 1-4 scaling cases) and
per-atom forces 1e-4 relative to max(|F_ref|, 1), as OpenMM's ASSERT_EQUAL_TOL/VEC do.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

import helpers

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_tests.json")))
CASES = GOLDEN["tests"]


def assert_equal_tol(expected, found, tol):
    scale = max(abs(expected), 1.0)
    assert abs(expected - found) / scale <= tol, (expected, found)


def assert_equal_vec(expected, found, tol):
    scale = max(float(np.linalg.norm(expected)), 1.0)
    assert np.all(np.abs(np.asarray(expected) - np.asarray(found)) / scale <= tol), (expected, found)


def check_case(result, case):
    assert_equal_tol(case["ref_energy"], result.energy, case["energy_tol"])
    if case["ref_forces"] is not None:
        for exp, got in zip(case["ref_forces"], result.forces):
            assert_equal_vec(exp, got, case["force_tol"])


@pytest.mark.skipif(not O.available("ref"), reason="reference oracle not built (needs the reference tree)")
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_reference_build_matches_golden(case):
    check_case(O.evaluate(O.system_from_golden(GOLDEN, case), "ref"), case)


def test_port_parameter_gradients_match_finite_differences():
    """dE/d(molecular-frame multipole parameters) of the oracle port against central
    differences of its own energy on the 160-atom frames system (every axis type,
    chirality, anisotropic polarisabilities), for each polarisation type."""
    import copy
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    rng = np.random.default_rng(3)
    for name in ("frames_direct.npz", "frames_mutual.npz", "frames_extrapolated.npz"):
        fx = helpers.load_npz_fixture(name)
        s = helpers.system_from_fixture(fx)
        s.mutual_eps, s.max_iter = 1e-11, 500
        g = O.evaluate(s, "port", want_grad=True).grad
        for _ in range(6):
            i, c = int(rng.integers(s.n)), int(rng.integers(20))
            h = 1e-6

            def energy(delta):
                t = copy.deepcopy(s)
                arr = [t.charge, t.dipole, t.quadrupole, t.octopole]
                k, off = (0, None) if c == 0 else (1, c - 1) if c < 4 else (2, c - 4) if c < 10 else (3, c - 10)
                a = np.array(arr[k], dtype=np.float64)
                if off is None:
                    a[i] += delta
                else:
                    a[i][off] += delta
                setattr(t, ["charge", "dipole", "quadrupole", "octopole"][k], a)
                return O.evaluate(t, "port").energy

            fd = (energy(h) - energy(-h)) / (2 * h)
            assert abs(fd - g[i][c]) <= 1e-6 * max(abs(fd), 1.0), (name, i, c, fd, g[i][c])


def test_port_polarization_gradients_match_finite_differences():
    """dE/d(molecular-frame polarisability X Y Z, Thole width) of the oracle port against
    central differences (h = 1e-3 relative; the energy is ~1e4 kJ/mol, so
    smaller steps are dominated by rounding) of its own energy on the 160-atom frames
    system, for every polarisation type (Extrapolated through its explicit adjoint sums)."""
    import copy
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    rng = np.random.default_rng(4)
    for name in ("frames_direct.npz", "frames_mutual.npz", "frames_extrapolated.npz"):
        fx = helpers.load_npz_fixture(name)
        s = helpers.system_from_fixture(fx)
        s.mutual_eps, s.max_iter = 1e-11, 500
        pg = O.evaluate(s, "port", want_grad=True).polgrad
        picks = [(int(rng.integers(s.n)), c) for c in range(4) for _ in range(2)]
        for i, c in picks:
            pol = np.array(s.polarity, dtype=np.float64).reshape(s.n, 3)
            base = pol[i][c] if c < 3 else float(np.asarray(s.thole)[i])
            h = 1e-3 * max(abs(base), 1e-6)

            def energy(delta):
                t = copy.deepcopy(s)
                if c < 3:
                    a = pol.copy()
                    a[i][c] += delta
                    t.polarity = a
                else:
                    a = np.array(t.thole, dtype=np.float64)
                    a[i] += delta
                    t.thole = a
                return O.evaluate(t, "port").energy

            fd = (energy(h) - energy(-h)) / (2 * h)
            assert abs(fd - pg[i][c]) <= 1e-5 * max(abs(fd), 1.0), (name, i, c, fd, pg[i][c])
