"""Force-field XML -> MPIDForce builder (mpidopenmmplugin_gb300.forcefield), the
restatement of the reference's MPIDGenerator (python/mpidplugin.i:538-1055).

The test force field below is written for these tests (not a published model): a
water with a bisector-frame oxygen and Z-then-X hydrogens whose x atom is two bonds away,
an ammonia whose nitrogen has a three-fold frame, a Z-bisect example, a Z-only hydrogen
and a frameless ion.  CPU tests check the frames, parameters and covalent maps it
assigns; where the reference tree is present, its own water models (swm4.xml, swm6.xml)
are read as well.  The GPU test evaluates a water box built by the builder against the
oracle port.
"""
import os

import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDForce
from mpidopenmmplugin_gb300.forcefield import ForceField, Topology, axis_type, pme_parameters

TEST_FF = """
<ForceField>
 <AtomTypes>
  <Type name="W-O" class="OW" element="O" mass="15.999"/>
  <Type name="W-H" class="HW" element="H" mass="1.008"/>
  <Type name="A-N" class="N3" element="N" mass="14.007"/>
  <Type name="A-H" class="HN" element="H" mass="1.008"/>
  <Type name="Z-C" class="CZ" element="C" mass="12.011"/>
  <Type name="Z-H" class="HZ" element="H" mass="1.008"/>
  <Type name="Z-X" class="XZ" element="Cl" mass="35.45"/>
  <Type name="ION" class="IO" element="Na" mass="22.99"/>
 </AtomTypes>
 <Residues>
  <Residue name="WAT">
   <Atom name="O" type="W-O"/><Atom name="H1" type="W-H"/><Atom name="H2" type="W-H"/>
   <Bond from="0" to="1"/><Bond from="0" to="2"/>
  </Residue>
  <Residue name="AMM">
   <Atom name="N" type="A-N"/><Atom name="H1" type="A-H"/><Atom name="H2" type="A-H"/><Atom name="H3" type="A-H"/>
   <Bond atomName1="N" atomName2="H1"/><Bond atomName1="N" atomName2="H2"/><Bond atomName1="N" atomName2="H3"/>
  </Residue>
  <Residue name="ZBS">
   <Atom name="C" type="Z-C"/><Atom name="X" type="Z-X"/><Atom name="H1" type="Z-H"/><Atom name="H2" type="Z-H"/>
   <Bond from="0" to="1"/><Bond from="0" to="2"/><Bond from="0" to="3"/>
  </Residue>
  <Residue name="ION"><Atom name="NA" type="ION"/></Residue>
 </Residues>
 <MPIDForce coulomb14scale="0.5" defaultTholeWidth="1.3">
  <Multipole type="W-O" kz="-W-H" kx="-W-H" c0="-0.834" dZ="-0.0051" qXX="0.0002" qYY="-0.0001" qZZ="-0.0001"
             oXXZ="0.00001" oYYZ="-0.00002" oZZZ="0.00001"/>
  <Multipole type="W-H" kz="W-O" kx="W-H" c0="0.417" dX="0.0012" dZ="-0.0021"/>
  <Multipole type="A-N" kz="-A-H" kx="-A-H" ky="-A-H" c0="-0.9" dZ="0.004"/>
  <Multipole type="A-H" kz="A-N" c0="0.3" dZ="-0.001"/>
  <Multipole type="Z-C" kz="Z-X" kx="-Z-H" ky="-Z-H" c0="0.1" dZ="0.002" qXX="0.0001" qYY="0.0001" qZZ="-0.0002"/>
  <Multipole type="Z-X" kz="Z-C" c0="-0.2"/>
  <Multipole type="Z-H" kz="Z-C" kx="Z-X" c0="0.05"/>
  <Multipole class="IO" c0="1.0"/>
  <Polarize type="W-O" polarizabilityXX="0.0011" polarizabilityYY="0.0010" polarizabilityZZ="0.0009" thole="0.7"/>
  <Polarize type="W-H" polarizabilityXX="0.0003" polarizabilityYY="0.0003" polarizabilityZZ="0.0003" thole="0.6"/>
  <Polarize type="A-N" polarizabilityXX="0.0012" polarizabilityYY="0.0012" polarizabilityZZ="0.0012" thole="0.65"/>
 </MPIDForce>
</ForceField>
"""


def test_axis_type_rules():
    assert axis_type("", "", "") == MPIDForce.NoAxisType
    assert axis_type("A", "", "") == MPIDForce.ZOnly
    assert axis_type("A", "B", "") == MPIDForce.ZThenX
    assert axis_type("A", "B", "C") == MPIDForce.ZThenX
    assert axis_type("-A", "B", "") == MPIDForce.Bisector
    assert axis_type("A", "-B", "") == MPIDForce.Bisector
    assert axis_type("A", "-B", "-C") == MPIDForce.ZBisect
    assert axis_type("-A", "-B", "-C") == MPIDForce.ThreeFold


def _topology():
    top = Topology()
    top.addResidue("WAT", ["O", "H1", "H2"])        # 0 1 2
    top.addResidue("AMM", ["N", "H1", "H2", "H3"])  # 3 4 5 6
    top.addResidue("ZBS", ["C", "X", "H1", "H2"])   # 7 8 9 10
    top.addResidue("ION", ["NA"])                   # 11
    top.addResidue("WAT", ["H1", "O", "H2"])        # 12 13 14 (atom order differs from the template)
    return top


def test_frames_parameters_and_covalent_maps():
    ff = ForceField(TEST_FF)
    f = ff.createForce(_topology(), MPIDForce.PME, 0.8, polarization="mutual", aEwald=3.0, pmeGridDimensions=[20, 20, 20])
    assert f.getNumMultipoles() == 15
    assert f.getPolarizationType() == MPIDForce.Mutual
    assert f.get14ScaleFactor() == 0.5 and f.getDefaultTholeWidth() == 1.3
    assert f.getPMEParameters() == (3.0, 20, 20, 20)
    expect = {  # atom: (axis type, z, x, y)
        0: (MPIDForce.Bisector, 1, 2, -1),
        1: (MPIDForce.ZThenX, 0, 2, -1),     # x is the other hydrogen, two bonds away
        2: (MPIDForce.ZThenX, 0, 1, -1),
        3: (MPIDForce.ThreeFold, 4, 5, 6),
        4: (MPIDForce.ZOnly, 3, -1, -1),
        7: (MPIDForce.ZBisect, 8, 9, 10),
        8: (MPIDForce.ZOnly, 7, -1, -1),
        9: (MPIDForce.ZThenX, 7, 8, -1),
        11: (MPIDForce.NoAxisType, -1, -1, -1),
        13: (MPIDForce.Bisector, 12, 14, -1),
        12: (MPIDForce.ZThenX, 13, 14, -1),
    }
    for i, (ax, z, x, y) in expect.items():
        p = f.getMultipoleParameters(i)
        assert (p[4], p[5], p[6], p[7]) == (ax, z, x, y), (i, p[4:8])
    q, d, Q, O, _, _, _, _, thole, pol = f.getMultipoleParameters(0)
    assert q == -0.834 and d == [0.0, 0.0, -0.0051] and Q == [0.0002, 0.0, -0.0001, 0.0, 0.0, -0.0001]
    assert O == [0.0, 0.0, 0.0, 0.0, 0.00001, 0.0, -0.00002, 0.0, 0.0, 0.00001]
    assert thole == 0.7 and pol == [0.0011, 0.0010, 0.0009]
    # no Polarize entry: polarisability and Thole width 0
    assert f.getMultipoleParameters(4)[8:] == (0.0, [0.0, 0.0, 0.0])
    assert f.getMultipoleParameters(11)[0] == 1.0
    assert f.getCovalentMap(0, MPIDForce.Covalent12) == [1, 2]
    assert f.getCovalentMap(1, MPIDForce.Covalent13) == [2]
    assert f.getCovalentMap(4, MPIDForce.Covalent13) == [5, 6]
    assert f.getCovalentMap(8, MPIDForce.Covalent13) == [9, 10]
    assert all(f.getCovalentMap(i, MPIDForce.Covalent14) == [] for i in range(15))
    assert f.getCovalentMap(11, MPIDForce.Covalent12) == []


def test_covalent_14_and_explicit_bonds():
    ff = ForceField(TEST_FF)
    top = Topology()
    # a chain of two "waters" bonded O-O across residues: H1-O-O'-H1' is 1-4
    a = top.addResidue("WAT", ["O", "H1", "H2"], bonds=[(0, 1), (0, 2)])
    b = top.addResidue("WAT", ["O", "H1", "H2"], bonds=[(0, 1), (0, 2)])
    top.addBond(a[0], b[0])
    f = ff.createForce(top, MPIDForce.NoCutoff, 1.0)
    assert f.getPolarizationType() == MPIDForce.Extrapolated
    assert f.getCovalentMap(a[1], MPIDForce.Covalent14) == [b[1], b[2]]
    assert f.getCovalentMap(a[0], MPIDForce.Covalent13) == [b[1], b[2]]


def test_errors_and_conflicts():
    ff = ForceField(TEST_FF)
    top = Topology()
    top.addResidue("XXX", ["A"])
    with pytest.raises(ValueError, match="No template"):
        ff.createForce(top)
    with pytest.raises(ValueError, match="invalide polarization"):
        ff.createForce(_topology(), polarization="bogus")
    bad = TEST_FF.replace('<Polarize type="A-N"', '<Polarize type="Z-Y"').replace(
        '<Type name="ION"', '<Type name="Z-Y" class="ZY" element="C" mass="1"/><Type name="ION"')
    with pytest.raises(ValueError, match="polarize type not present"):
        ForceField(bad)
    second = "<ForceField><MPIDForce coulomb14scale=\"0.8\" defaultTholeWidth=\"1.3\"/></ForceField>"
    with pytest.raises(ValueError, match="coulomb14scale"):
        ForceField(TEST_FF, second)
    with pytest.warns(UserWarning, match="Conflicting coulomb14scale"):
        f = ForceField(TEST_FF).createForce(_topology(), coulomb14scale=0.4)
    assert f.get14ScaleFactor() == 0.4
    # an atom whose type has no entry that can be placed
    lone = Topology()
    lone.addResidue("WAT", ["O", "H1", "H2"], bonds=[(0, 1)])  # H2 has no bonds
    with pytest.raises(ValueError, match="was not assigned"):
        ff.createForce(lone)


def test_pme_parameters_rule():
    alpha, grid = pme_parameters(0.9, [6.214, 6.214, 3.0], 5e-4)
    assert abs(alpha - np.sqrt(-np.log(1e-3)) / 0.9) < 1e-12
    raw = [int(np.ceil(2 * alpha * L / (3 * 5e-4 ** 0.2))) for L in (6.214, 6.214, 3.0)]
    for n, r in zip(grid, raw):
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        assert m == 1 and n >= r and n - r < 8


# the reference tree, where it is present (read only by these CPU tests)
REF_PARAMS = os.path.join(os.environ.get("MPID_REFERENCE_ROOT", "/root/reference"), "examples", "parameters")


@pytest.mark.skipif(not os.path.isdir(REF_PARAMS), reason="reference tree absent")
@pytest.mark.parametrize("name", ["swm4.xml", "swm6.xml"])
def test_reference_water_models(name):
    """The reference's own MPID water models read and assigned: bisector oxygen with its
    polarisability and Thole width, Z-then-X hydrogens; values as written in the file."""
    import xml.etree.ElementTree as ET
    path = os.path.join(REF_PARAMS, name)
    root = ET.parse(path).getroot()
    ff = ForceField(path)
    top = Topology()
    for _ in range(4):
        top.addResidue("HOH", ["H1", "H2", "O"])
    f = ff.createForce(top, MPIDForce.PME, 0.8, aEwald=3.5, pmeGridDimensions=[24, 24, 24])
    mult = {m.get("type"): m.attrib for m in root.findall("MPIDForce/Multipole")}
    polz = {p.get("type"): p.attrib for p in root.findall("MPIDForce/Polarize")}
    for w in range(4):
        h1, h2, o = 3 * w, 3 * w + 1, 3 * w + 2
        po = f.getMultipoleParameters(o)
        assert po[4:8] == (MPIDForce.Bisector, h1, h2, -1)
        assert po[0] == float(mult["OT"]["c0"]) and po[1][2] == float(mult["OT"]["dZ"])
        assert po[8] == float(polz["OT"]["thole"]) and po[9][0] == float(polz["OT"]["polarizabilityXX"])
        assert f.getMultipoleParameters(h1)[4:8] == (MPIDForce.ZThenX, o, h2, -1)
        assert f.getMultipoleParameters(h2)[4:8] == (MPIDForce.ZThenX, o, h1, -1)
        assert f.getMultipoleParameters(h1)[0] == float(mult["HT"]["c0"])


@pytest.mark.gpu
def test_builder_water_box_matches_oracle():
    """A 216-water box built from the test force field (residue atom order O, H1, H2),
    evaluated through the C ABI in FP64 and against the oracle port."""
    import helpers
    from oracle import oracle as O
    from mpidopenmmplugin_gb300 import MPIDContext, synthetic
    if not O.available("port"):
        O.build("port")
    _, pos, box = synthetic.water_box(216, 18.64, seed=9)
    top = Topology()
    for _ in range(216):
        top.addResidue("WAT", ["O", "H1", "H2"])
    ff = ForceField(TEST_FF)
    for pol in ("mutual", "direct", "extrapolated"):
        f = ff.createForce(top, MPIDForce.PME, 0.8, polarization=pol, aEwald=3.5, pmeGridDimensions=[24, 24, 24],
                           mutualInducedTargetEpsilon=1e-9)
        f.setPmeBSplineOrder(5)
        ctx = MPIDContext(f, precision="double")
        e, forces = ctx.evaluate(pos, box)
        ref = O.evaluate(helpers.oracle_system(f, pos, box), "port")
        assert abs(e - ref.energy) <= 1e-8 * abs(ref.energy), (pol, e, ref.energy)
        assert helpers.rel_rms(forces, ref.forces) < 1e-7, pol
