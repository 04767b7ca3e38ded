"""GPU parity: the CUDA path (through the C ABI) against the reference's FP64 CPU force.

Oracle outputs are committed fixtures (tests/golden/): the reference's 18 known-answer
cases (reference_tests.json) and reference runs on seeded systems (make_fixtures.py).

Tolerances
* FP64 path: relative RMS force error <= 1e-7, relative energy error <= 1e-8,
  induced dipoles <= 1e-6 relative RMS (the mutual fixtures converge to 1e-9 D).
* mixed path: relative RMS force error <= 5e-6 and relative energy error <= 1e-6 on the
  water box (the accuracy gates of the mixed-precision evaluation); the 4-12 atom
  known-answer cases use the reference tests' own tolerance, 1e-4 relative to
  max(|x|, 1), because their energies are small differences of large terms.
"""
import os

import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDContext, MPIDForce, synthetic

import helpers
from test_oracle_golden import assert_equal_tol, assert_equal_vec

pytestmark = pytest.mark.gpu

GOLDEN = helpers.load_reference_tests()
CASES = GOLDEN["tests"]


def run(force, pos, box, precision, **kw):
    ctx = MPIDContext(force, precision=precision, **kw)
    e, f = ctx.evaluate(pos, box)
    return ctx, e, f


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_reference_known_answers(case, precision):
    from oracle import oracle as O
    s = O.system_from_golden(GOLDEN, case)
    f = helpers.force_from_oracle_system(s)
    box = s.box if s.nonbonded_method == 1 else np.eye(3) * 10.0
    ctx, e, forces = run(f, s.pos, box, precision)
    assert_equal_tol(case["ref_energy"], e, case["energy_tol"])
    if case["ref_forces"] is not None:
        for exp, got in zip(case["ref_forces"], forces):
            assert_equal_vec(exp, got, case["force_tol"])


def _fixture_case(name):
    fx = helpers.load_npz_fixture(name)
    s = helpers.system_from_fixture(fx)
    return fx, s, helpers.force_from_oracle_system(s)


def _torque_mapped_zonly(s):
    """Atoms whose forces include a Z-only torque mapping.  The reference CPU code maps
    those through an x atom that Z-only frames do not have (undefined there), so they are
    checked against finite differences of its energy in test_zonly_matches_energy_gradient."""
    z = [i for i in range(s.n) if int(s.axis_type[i]) == MPIDForce.ZOnly]
    return set(z) | set(int(s.atom_z[i]) for i in z)


@pytest.mark.parametrize("pol", ["direct", "mutual", "extrapolated"])
@pytest.mark.parametrize("system", ["water648", "frames", "triclinic"])
def test_fixture_double(system, pol):
    fx, s, f = _fixture_case("%s_%s.npz" % (system, pol))
    ctx, e, forces = run(f, s.pos, s.box, "double")
    skip = _torque_mapped_zonly(s)
    mask = np.array([i not in skip for i in range(s.n)])
    assert abs(e - fx["ref_energy"]) / abs(fx["ref_energy"]) < 1e-8
    assert helpers.rel_rms(forces[mask], fx["ref_forces"][mask]) < 1e-7
    assert helpers.rel_rms(ctx.getInducedDipoles(), fx["ref_induced"]) < 1e-6
    assert helpers.rel_rms(ctx.getLabFramePermanentDipoles(), fx["ref_labdipoles"]) < 1e-12
    tot = ctx.getTotalDipoles()
    assert np.allclose(tot, ctx.getInducedDipoles() + ctx.getLabFramePermanentDipoles(), rtol=0, atol=1e-15)


@pytest.mark.parametrize("pol", ["direct", "mutual", "extrapolated"])
@pytest.mark.parametrize("system", ["water648", "frames", "triclinic"])
def test_fixture_mixed(system, pol):
    fx, s, f = _fixture_case("%s_%s.npz" % (system, pol))
    ctx, e, forces = run(f, s.pos, s.box, "mixed")
    skip = _torque_mapped_zonly(s)
    mask = np.array([i not in skip for i in range(s.n)])
    ferr = helpers.rel_rms(forces[mask], fx["ref_forces"][mask])
    eerr = abs(e - fx["ref_energy"]) / abs(fx["ref_energy"])
    print("%s %s mixed: energy rel err %.3e force rel RMS %.3e stats %s" % (system, pol, eerr, ferr, ctx.stats()))
    assert ferr < 5e-6
    # FP32 rounding of the real-space pair energies is random, so its relative effect on
    # the total shrinks as N^-1/2; the 1e-6 energy gate is asserted on the 24,000-atom
    # box in test_headline_accuracy_gates, the 648-atom box gets 1e-5.
    assert eerr < 1e-5
    assert helpers.rel_rms(ctx.getInducedDipoles(), fx["ref_induced"]) < 5e-6


def test_zonly_matches_energy_gradient():
    """Z-only torque mapping of the GPU path against central differences of the energy."""
    fx, s, f = _fixture_case("frames_direct.npz")
    ctx = MPIDContext(f, precision="double")
    e0, forces = ctx.evaluate(s.pos, s.box)
    # a small step keeps every pair on its side of the cutoff, where the real-space
    # energy is discontinuous; FP64 energies make the difference quotient precise
    h = 1e-5

    def energy_at(atom, c, delta):
        p = s.pos.copy()
        p[atom, c] += delta
        return ctx.evaluate(p, s.box)[0]

    for atom in sorted(_torque_mapped_zonly(s))[:6]:
        for c in range(3):
            fd = -(energy_at(atom, c, h) - energy_at(atom, c, -h)) / (2 * h)
            assert abs(fd - forces[atom, c]) < 1e-5 * max(1.0, abs(fd)), (atom, c, fd, forces[atom, c])


def test_forces_are_accumulated_and_deterministic():
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)
    ctx = MPIDContext(f, precision="mixed")
    e1, f1 = ctx.evaluate(pos, box)
    e2, f2 = ctx.evaluate(pos, box)
    assert e1 == e2
    assert np.array_equal(f1, f2)
    base = np.full_like(f1, 3.0)
    _, f3 = ctx.evaluate(pos, box, forces=base.copy())
    assert np.array_equal(f3, f1 + 3.0)


def test_mixed_against_double_order5():
    """Order-5 PME (which the reference cannot run): mixed path against the FP64 path."""
    for pol in (MPIDForce.Direct, MPIDForce.Mutual, MPIDForce.Extrapolated):
        f, pos, box = synthetic.workload("water648", polarization=pol, order=5)
        _, ed, fd = run(f, pos, box, "double")
        ctx, em, fm = run(f, pos, box, "mixed")
        assert helpers.rel_rms(fm, fd) < 5e-6, pol
        assert abs(em - ed) / abs(ed) < 1e-5, pol


@pytest.mark.parametrize("pol", [MPIDForce.Mutual, MPIDForce.Extrapolated, MPIDForce.Direct])
def test_headline_accuracy_gates(pol):
    """24,000-atom water box, order-5 PME: mixed path within 5e-6 relative RMS force and
    1e-6 relative energy of the FP64 path, induced dipoles within 5e-6."""
    f, pos, box = synthetic.workload("water24k", polarization=pol)
    cd, ed, fd = run(f, pos, box, "double")
    cm, em, fm = run(f, pos, box, "mixed")
    ferr = helpers.rel_rms(fm, fd)
    eerr = abs(em - ed) / abs(ed)
    merr = helpers.rel_rms(cm.getInducedDipoles(), cd.getInducedDipoles())
    print("water24k pol %d: energy %.3e force %.3e dipole %.3e; mixed %s; double %s" %
          (pol, eerr, ferr, merr, cm.stats(), cd.stats()))
    assert ferr < 5e-6
    assert eerr < 1e-6
    assert merr < 5e-6
    if pol == MPIDForce.Mutual:
        # the FP32 CG operator is accurate enough that one FP64 residual check confirms the
        # first inner solve (a second outer step would cost another FP64 field evaluation)
        assert cm.stats()["refinement_steps"] == 1


def test_validation_errors_on_device():
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Direct, order=5)
    ctx = MPIDContext(f, precision="mixed")
    with pytest.raises(Exception, match="twice the nonbonded cutoff"):
        ctx.evaluate(pos, np.eye(3) * 1.0)
    f.setMutualInducedMaxIterations(1)
    f.setPolarizationType(MPIDForce.Mutual)
    ctx = MPIDContext(f, precision="double")
    with pytest.raises(Exception, match="did not converge"):
        ctx.evaluate(pos, box)
    # a B-spline stencil may wrap around the grid only once
    alpha = f.getPMEParameters()[0]
    f.setPMEParameters(alpha, 24, 4, 24)
    with pytest.raises(Exception, match="at least the B-spline order"):
        MPIDContext(f, precision="mixed")


@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_preconditioned_cg_matches_plain_cg(precision):
    """The near-field preconditioner changes the path to the solution, not the solution:
    PCG and plain CG agree within the solver tolerance (1e-7 D) on the 24,000-atom box."""
    f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Mutual)
    a = MPIDContext(f, precision=precision, preconditioner=True)
    ea, fa = a.evaluate(pos, box)
    b = MPIDContext(f, precision=precision)
    eb, fb = b.evaluate(pos, box)
    sa, sb = a.stats(), b.stats()
    print("%s: PCG %d iterations (%d refinements), CG %d iterations (%d refinements)" %
          (precision, sa["solver_iterations"], sa["refinement_steps"], sb["solver_iterations"], sb["refinement_steps"]))
    assert sa["solver_residual"] < 1e-7 and sb["solver_residual"] < 1e-7
    assert abs(ea - eb) / abs(eb) < 1e-7
    assert helpers.rel_rms(fa, fb) < 2e-6
    assert helpers.rel_rms(a.getInducedDipoles(), b.getInducedDipoles()) < 2e-6


@pytest.mark.parametrize("pol", [MPIDForce.Direct, MPIDForce.Mutual, MPIDForce.Extrapolated])
def test_solution61k_gates(pol):
    """61,600-atom solution (20,000 waters + 200 ethanes with anisotropic polarisabilities,
    Thole widths U[1, 2], 1-4 scaling 0.5), 96^3 grid: mixed path against the FP64 path
    for each polarisation type within the accuracy gates (force 5e-6, energy 1e-6,
    induced dipoles 5e-6)."""
    f, pos, box = synthetic.workload("solution61k", polarization=pol)
    cd, ed, fd = run(f, pos, box, "double")
    cm, em, fm = run(f, pos, box, "mixed")
    ferr = helpers.rel_rms(fm, fd)
    eerr = abs(em - ed) / abs(ed)
    merr = helpers.rel_rms(cm.getInducedDipoles(), cd.getInducedDipoles())
    print("solution61k pol %d: energy %.3e force %.3e dipole %.3e; iterations %d / %d" %
          (pol, eerr, ferr, merr, cm.stats()["solver_iterations"], cd.stats()["solver_iterations"]))
    assert ferr < 5e-6
    assert eerr < 1e-6
    assert merr < 5e-6


@pytest.mark.parametrize("pol", [MPIDForce.Mutual, MPIDForce.Extrapolated])
def test_water288k_gates(pol):
    """288,000-atom water box, 144^3 grid, Mutual to 1e-6 D and OPT extrapolation: mixed
    path against the FP64 path within the accuracy gates."""
    f, pos, box = synthetic.workload("water288k", polarization=pol)
    cd, ed, fd = run(f, pos, box, "double")
    cm, em, fm = run(f, pos, box, "mixed")
    ferr = helpers.rel_rms(fm, fd)
    eerr = abs(em - ed) / abs(ed)
    merr = helpers.rel_rms(cm.getInducedDipoles(), cd.getInducedDipoles())
    print("water288k pol %d: energy %.3e force %.3e dipole %.3e; mixed %.1f ms, double %.1f ms" %
          (pol, eerr, ferr, merr, cm.stats()["ms_total"], cd.stats()["ms_total"]))
    assert ferr < 5e-6
    assert eerr < 1e-6
    assert merr < 5e-6


def test_solution61k_double_matches_oracle():
    """FP64 path against the oracle port (pinned to the reference) on the 61,600-atom
    solution, mutual polarisation: anisotropic polarisabilities, 1-4 scaling and per-atom
    Thole widths at full size."""
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    f, pos, box = synthetic.workload("solution61k", polarization=MPIDForce.Mutual)
    f.setMutualInducedTargetEpsilon(1e-9)
    ctx, e, forces = run(f, pos, box, "double")
    ref = O.evaluate(helpers.oracle_system(f, pos, box), "port")
    eerr = abs(e - ref.energy) / abs(ref.energy)
    ferr = helpers.rel_rms(forces, ref.forces)
    print("solution61k double vs oracle: energy %.3e force %.3e" % (eerr, ferr))
    assert eerr < 1e-8
    assert ferr < 1e-7


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("case", ["water648_pme", "frames_pme", "frames_nocutoff"])
def test_system_moments_and_potential_match_reference(case, precision):
    """getSystemMultipoleMoments and getElectrostaticPotential against the reference's own
    outputs (tests/golden/properties_*.npz, from MPIDReferenceForce.cpp:2349-2528)."""
    fx = helpers.load_npz_fixture("properties_%s.npz" % case)
    s = helpers.system_from_fixture(fx)
    f = helpers.force_from_oracle_system(s)
    ctx = MPIDContext(f, precision=precision)
    box = s.box if s.nonbonded_method == 1 else np.eye(3) * 10.0
    mom = ctx.getSystemMultipoleMoments(s.pos, box, fx["masses"])
    pot = ctx.getElectrostaticPotential(fx["grid_points"], s.pos, box)
    ref_m, ref_p = fx["ref_moments"], fx["ref_potential"]
    tol = 1e-8 if precision == "double" else 2e-6
    scale_m = np.abs(ref_m).max()
    assert np.abs(mom - ref_m).max() <= tol * scale_m + 1e-12, (mom, ref_m)
    assert helpers.rel_rms(pot, ref_p) <= tol


@pytest.mark.parametrize("precision", ["double", "mixed"])
@pytest.mark.parametrize("name", ["frames_direct.npz", "frames_mutual.npz", "frames_extrapolated.npz",
                                  "water648_mutual.npz"])
def test_parameter_gradients_match_oracle(name, precision):
    """dE/d(molecular-frame multipole parameters) against the oracle port's gradients
    (checked there against central differences): FP64 to 1e-9, mixed to 1e-5 (relative
    RMS over all atoms and components)."""
    from oracle import oracle as O
    if not O.available("port"):
        O.build("port")
    fx = helpers.load_npz_fixture(name)
    s = helpers.system_from_fixture(fx)
    s.mutual_eps, s.max_iter = 1e-10, 500
    f = helpers.force_from_oracle_system(s)
    ctx = MPIDContext(f, precision=precision)
    g = ctx.getParameterGradients(s.pos, s.box)
    ref = O.evaluate(s, "port", want_grad=True).grad
    err = helpers.rel_rms(g, ref)
    worst = np.unravel_index(np.argmax(np.abs(g - ref)), g.shape)
    print("%s %s: gradient rel RMS %.3e; largest difference at atom %d component %d (axis %d): %.6e vs %.6e" %
          (name, precision, err, worst[0], worst[1], int(s.axis_type[worst[0]]), g[worst], ref[worst]))
    assert err < (1e-8 if precision == "double" else 1e-5)


def test_parameter_gradients_finite_differences_on_device():
    """FP64 path: the gradient along random admissible parameter directions (charges,
    dipoles, traceless quadrupoles and octopoles of a few atoms) against central
    differences of the device energy, to 1e-6 relative."""
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)
    f.setMutualInducedTargetEpsilon(1e-10)
    ctx = MPIDContext(f, precision="double")
    g = ctx.getParameterGradients(pos, box)
    rng = np.random.default_rng(5)
    for trial in range(4):
        atoms = rng.choice(f.getNumMultipoles(), 3, replace=False)
        v = np.zeros((f.getNumMultipoles(), 20))
        for a in atoms:
            v[a, 0] = rng.normal()
            v[a, 1:4] = rng.normal(size=3) * 0.01
            v[a, 4:10] = synthetic.traceless_quadrupole(rng, 0.001, 1)[0]
            v[a, 10:20] = synthetic.traceless_octopole(rng, 1e-4, 1)[0]
        h = 1e-4

        def energy(sign):
            f2 = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)[0]
            f2.setMutualInducedTargetEpsilon(1e-10)
            for a in atoms:
                p = list(f2.getMultipoleParameters(int(a)))
                p[0] += sign * h * v[a, 0]
                p[1] = list(np.asarray(p[1]) + sign * h * v[a, 1:4])
                p[2] = list(np.asarray(p[2]) + sign * h * v[a, 4:10])
                p[3] = list(np.asarray(p[3]) + sign * h * v[a, 10:20])
                f2.setMultipoleParameters(int(a), *p)
            c2 = MPIDContext(f2, precision="double")
            return c2.evaluate(pos, box)[0]

        fd = (energy(1) - energy(-1)) / (2 * h)
        an = float((g * v).sum())
        print("direction %d: analytic %.10e fd %.10e" % (trial, an, fd))
        assert abs(an - fd) <= 1e-6 * max(abs(fd), 1.0)


def test_automatic_pme_parameters_and_force_side_queries():
    """PME parameters left at 0 are chosen from the Ewald error tolerance (OpenMM's rule,
    as the reference kernel does); the force's context queries of the reference API
    (getInducedDipoles(context), getPMEParametersInContext(context), ...) answer through
    an MPIDContext."""
    from mpidopenmmplugin_gb300.forcefield import pme_parameters
    f, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)
    f.setPMEParameters(0.0, 0, 0, 0)
    f.setEwaldErrorTolerance(5e-4)
    with pytest.raises(Exception, match="PME parameters are 0"):
        MPIDContext(f, precision="double")
    masses = np.tile([15.999, 1.008, 1.008], f.getNumMultipoles() // 3)
    ctx = MPIDContext(f, precision="double", box=box, masses=masses)
    alpha, grid = pme_parameters(f.getCutoffDistance(), np.diag(box), 5e-4, minimum=5)
    assert f.getPMEParametersInContext(ctx) == (alpha, grid[0], grid[1], grid[2])
    e, forces = ctx.evaluate(pos, box)
    f2 = synthetic.workload("water648", polarization=MPIDForce.Mutual, order=5)[0]
    f2.setPMEParameters(alpha, *grid)
    e2, forces2 = MPIDContext(f2, precision="double").evaluate(pos, box)
    assert abs(e - e2) <= 1e-12 * abs(e2) and helpers.rel_rms(forces, forces2) < 1e-12
    assert np.array_equal(f.getInducedDipoles(ctx), ctx.getInducedDipoles())
    assert np.array_equal(f.getTotalDipoles(ctx), ctx.getTotalDipoles())
    assert np.array_equal(f.getLabFramePermanentDipoles(ctx), ctx.getLabFramePermanentDipoles())
    m = f.getSystemMultipoleMoments(ctx)
    assert np.allclose(m, ctx.getSystemMultipoleMoments(pos, box, masses), rtol=1e-12, atol=1e-12)
    grid_pts = np.random.default_rng(2).uniform(0, box[0, 0], size=(5, 3))
    assert np.allclose(f.getElectrostaticPotential(grid_pts, ctx), ctx.getElectrostaticPotential(grid_pts, pos, box),
                       rtol=1e-12, atol=1e-12)
    # updateParametersInContext: a changed charge reaches the context
    p = list(f.getMultipoleParameters(0))
    p[0] += 0.01
    f.setMultipoleParameters(0, *p)
    f.updateParametersInContext(ctx)
    assert ctx.evaluate(pos, box)[0] != e


_PORT_CACHE = {}


def _port_water24k(eps):
    """The oracle port's FP64 evaluation of the 24,000-atom box (order 5, Mutual) at
    solver tolerance eps, once per process."""
    from oracle import oracle as O
    if eps not in _PORT_CACHE:
        if not O.available("port"):
            O.build("port")
        f, pos, box = synthetic.workload("water24k", polarization=MPIDForce.Mutual)
        f.setMutualInducedTargetEpsilon(eps)
        _PORT_CACHE[eps] = (f, pos, box, O.evaluate(helpers.oracle_system(f, pos, box), "port"))
    return _PORT_CACHE[eps]


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_water24k_order5_against_oracle(precision):
    """The headline box (24,000 atoms, 72^3 grid, order-5 PME, Mutual) against the oracle
    port's FP64 evaluation of the same inputs.  FP64 path (both solves to 1e-9 D):
    energy 1e-8, forces 1e-7, induced dipoles 1e-6 relative.  Mixed path (1e-7 D, the
    workload's tolerance, as is the port): the accuracy gates, energy 1e-6, forces 5e-6,
    induced dipoles 5e-6."""
    eps = 1e-9 if precision == "double" else 1e-7
    f, pos, box, ref = _port_water24k(eps)
    ctx, e, forces = run(f, pos, box, precision)
    eerr = abs(e - ref.energy) / abs(ref.energy)
    ferr = helpers.rel_rms(forces, ref.forces)
    merr = helpers.rel_rms(ctx.getInducedDipoles(), ref.induced)
    print("water24k %s vs oracle: energy %.3e force %.3e dipole %.3e" % (precision, eerr, ferr, merr))
    if precision == "double":
        assert eerr < 1e-8 and ferr < 1e-7 and merr < 1e-6
    else:
        assert eerr < 1e-6 and ferr < 5e-6 and merr < 5e-6
