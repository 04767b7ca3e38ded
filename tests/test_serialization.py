"""XML serialization in the reference's format (serialization/src/MPIDForceProxy.cpp),
checked as the reference's own TestSerializeMPIDForce.cpp does: a force with every
setting changed from its default, 3 multipoles with Bisector frames and all eight
covalent maps, written and read back, every field equal."""
import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDError, MPIDForce, serialization, synthetic


def _force():
    f = MPIDForce()
    f.setForceGroup(3)
    f.setNonbondedMethod(MPIDForce.NoCutoff)
    f.setCutoffDistance(0.9)
    f.setAEwald(0.544)
    f.setPmeGridDimensions([64, 63, 61])
    f.setMutualInducedMaxIterations(200)
    f.setMutualInducedTargetEpsilon(1.0e-05)
    f.setEwaldErrorTolerance(1.0e-05)
    f.set14ScaleFactor(0.4)
    f.setExtrapolationCoefficients([0.1, 0.2, 0.3])
    f.setDefaultTholeWidth(2.5)
    rng = np.random.default_rng(1)
    for i in range(3):
        f.addMultipole(float(i + 1), rng.normal(size=3), rng.normal(size=6), rng.normal(size=10), MPIDForce.Bisector,
                       i + 1, i + 2, i + 3, 0.1 * (i + 1), list(rng.uniform(0.5, 2, size=3)))
        for t in range(MPIDForce.CovalentEnd):
            f.setCovalentMap(i, t, list(range(t + 1)))
    return f


def _assert_same(a, b):
    assert a.getForceGroup() == b.getForceGroup()
    assert a.getCutoffDistance() == b.getCutoffDistance()
    assert a.getNonbondedMethod() == b.getNonbondedMethod()
    assert a.getPolarizationType() == b.getPolarizationType()
    assert a.getAEwald() == b.getAEwald()
    assert a.getPmeGridDimensions() == b.getPmeGridDimensions()
    assert a.getMutualInducedMaxIterations() == b.getMutualInducedMaxIterations()
    assert a.getMutualInducedTargetEpsilon() == b.getMutualInducedTargetEpsilon()
    assert a.getEwaldErrorTolerance() == b.getEwaldErrorTolerance()
    assert a.get14ScaleFactor() == b.get14ScaleFactor()
    assert a.getDefaultTholeWidth() == b.getDefaultTholeWidth()
    assert a.getPmeBSplineOrder() == b.getPmeBSplineOrder()
    assert a.getExtrapolationCoefficients() == b.getExtrapolationCoefficients()
    assert a.getNumMultipoles() == b.getNumMultipoles()
    for i in range(a.getNumMultipoles()):
        pa, pb = a.getMultipoleParameters(i), b.getMultipoleParameters(i)
        for x, y in zip(pa, pb):
            assert x == y
        for t in range(MPIDForce.CovalentEnd):
            assert a.getCovalentMap(i, t) == b.getCovalentMap(i, t)


def test_round_trip_every_field():
    f1 = _force()
    f2 = serialization.deserialize(serialization.serialize(f1))
    _assert_same(f1, f2)


def test_round_trip_workload():
    f1, pos, box = synthetic.workload("water648", polarization=MPIDForce.Mutual)
    f2 = serialization.deserialize(serialization.serialize(f1))
    _assert_same(f1, f2)
    assert (f1.arrays()["cov_index"] == f2.arrays()["cov_index"]).all()


def test_reads_version_0_without_the_extra_attributes():
    """A file as the reference writes it (no defaultTholeWidth / pmeBSplineOrder): those
    two keep their defaults, everything else is read."""
    text = serialization.serialize(_force())
    text = text.replace(' defaultTholeWidth="2.5"', "").replace(' pmeBSplineOrder="6"', "")
    f = serialization.deserialize(text)
    assert f.getDefaultTholeWidth() == MPIDForce().getDefaultTholeWidth()
    assert f.getPmeBSplineOrder() == 6
    assert f.getNumMultipoles() == 3 and f.getForceGroup() == 3


def test_rejects_other_versions():
    text = serialization.serialize(_force()).replace('version="0"', 'version="1"')
    with pytest.raises(MPIDError, match="Unsupported version number"):
        serialization.deserialize(text)


def test_document_shape():
    import xml.etree.ElementTree as ET
    root = ET.fromstring(serialization.serialize(_force()))
    assert root.tag == "Force" and root.get("type") == "MPIDForce" and root.get("version") == "0"
    p = root.find("MultipoleParticles").findall("Particle")[1]
    assert [c.tag for c in p] == ["Dipole", "Quadrupole", "Octopole"] + serialization.COVALENT_TYPES
    assert [int(cv.get("v")) for cv in p.find("Covalent14")] == [0, 1, 2]
    assert root.find("ExtrapolationCoefficients").get("c2") == "0.3"
