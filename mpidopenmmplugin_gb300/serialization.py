"""XML serialization of an MPIDForce in the reference's format (version 0).

The element and attribute names, their meaning and the version number follow the
reference's serialization proxy (serialization/src/MPIDForceProxy.cpp:70-245), as
OpenMM's XmlSerializer writes it: a root <Force type="MPIDForce" version="0" ...> with
the force-wide settings as attributes, <MultipoleParticleGridDimension d0 d1 d2>,
<ExtrapolationCoefficients c0 c1 ...>, and <MultipoleParticles> holding one <Particle>
per atom with <Dipole>, <Quadrupole>, <Octopole> and the eight covalent maps
(<Covalent12> ... <PolarizationCovalent14>, each a list of <Cv v="index"/>).

Two details differ from the reference and are harmless to its reader: the "damp"
attribute (written from an uninitialised variable there) holds the damping factor
(mean polarisability)^(1/6) used by the kernels, and the default Thole width and PME
B-spline order, which version 0 does not carry, are added as extra attributes that the
reference's reader ignores.  Reading a reference-written file leaves those two at their
defaults, as the reference does.
"""
import xml.etree.ElementTree as ET

from .force import MPIDError, MPIDForce

VERSION = 0
COVALENT_TYPES = ["Covalent12", "Covalent13", "Covalent14", "Covalent15", "PolarizationCovalent11",
                  "PolarizationCovalent12", "PolarizationCovalent13", "PolarizationCovalent14"]
_QUAD = ["qXX", "qXY", "qYY", "qXZ", "qYZ", "qZZ"]
_OCT = ["oXXX", "oXXY", "oXYY", "oYYY", "oXXZ", "oXYZ", "oYYZ", "oXZZ", "oYZZ", "oZZZ"]


def _f(x):
    return repr(float(x))


def serialize(force: MPIDForce) -> str:
    """XML text of `force` (MPIDForceProxy::serialize, MPIDForceProxy.cpp:70-160)."""
    alpha, nx, ny, nz = force.getPMEParameters()
    root = ET.Element("Force", {
        "type": "MPIDForce", "version": str(VERSION), "forceGroup": str(getattr(force, "forceGroup", 0)),
        "nonbondedMethod": str(force.getNonbondedMethod()), "polarizationType": str(force.getPolarizationType()),
        "mutualInducedMaxIterations": str(force.getMutualInducedMaxIterations()),
        "cutoffDistance": _f(force.getCutoffDistance()), "aEwald": _f(alpha),
        "mutualInducedTargetEpsilon": _f(force.getMutualInducedTargetEpsilon()),
        "ewaldErrorTolerance": _f(force.getEwaldErrorTolerance()), "scaleFactor14": _f(force.get14ScaleFactor()),
        "defaultTholeWidth": _f(force.getDefaultTholeWidth()), "pmeBSplineOrder": str(force.getPmeBSplineOrder()),
    })
    ET.SubElement(root, "MultipoleParticleGridDimension", {"d0": str(nx), "d1": str(ny), "d2": str(nz)})
    ET.SubElement(root, "ExtrapolationCoefficients",
                  {"c%d" % i: _f(c) for i, c in enumerate(force.getExtrapolationCoefficients())})
    particles = ET.SubElement(root, "MultipoleParticles")
    for i in range(force.getNumMultipoles()):
        q, d, Q, O, axis, z, x, y, thole, pol = force.getMultipoleParameters(i)
        damp = (sum(pol) / 3.0) ** (1.0 / 6.0) if sum(pol) > 0 else 0.0
        p = ET.SubElement(particles, "Particle", {
            "axisType": str(axis), "multipoleAtomZ": str(z), "multipoleAtomX": str(x), "multipoleAtomY": str(y),
            "charge": _f(q), "thole": _f(thole), "damp": _f(damp), "polarizabilityXX": _f(pol[0]),
            "polarizabilityYY": _f(pol[1]), "polarizabilityZZ": _f(pol[2])})
        ET.SubElement(p, "Dipole", {"dX": _f(d[0]), "dY": _f(d[1]), "dZ": _f(d[2])})
        ET.SubElement(p, "Quadrupole", {k: _f(v) for k, v in zip(_QUAD, Q)})
        ET.SubElement(p, "Octopole", {k: _f(v) for k, v in zip(_OCT, O)})
        for t, name in enumerate(COVALENT_TYPES):
            m = ET.SubElement(p, name)
            for a in force.getCovalentMap(i, t):
                ET.SubElement(m, "Cv", {"v": str(a)})
    ET.indent(root)
    return '<?xml version="1.0" ?>\n' + ET.tostring(root, encoding="unicode") + "\n"


def deserialize(text: str) -> MPIDForce:
    """MPIDForce from XML text (MPIDForceProxy::deserialize, MPIDForceProxy.cpp:162-245):
    rejects versions other than 0 with the reference's message."""
    root = ET.fromstring(text)
    if root.tag != "Force" or root.get("type", "MPIDForce") != "MPIDForce":
        raise MPIDError("not a serialized MPIDForce")
    version = int(root.get("version", "-1"))
    if version < 0 or version > VERSION:
        raise MPIDError("Unsupported version number")
    f = MPIDForce()
    f.forceGroup = int(root.get("forceGroup", "0"))
    f.setNonbondedMethod(int(root.get("nonbondedMethod")))
    f.setPolarizationType(int(root.get("polarizationType")))
    f.setMutualInducedMaxIterations(int(root.get("mutualInducedMaxIterations")))
    f.setCutoffDistance(float(root.get("cutoffDistance")))
    f.setMutualInducedTargetEpsilon(float(root.get("mutualInducedTargetEpsilon")))
    f.setEwaldErrorTolerance(float(root.get("ewaldErrorTolerance")))
    f.set14ScaleFactor(float(root.get("scaleFactor14")))
    if root.get("defaultTholeWidth") is not None:
        f.setDefaultTholeWidth(float(root.get("defaultTholeWidth")))
    if root.get("pmeBSplineOrder") is not None:
        f.setPmeBSplineOrder(int(root.get("pmeBSplineOrder")))
    g = root.find("MultipoleParticleGridDimension")
    f.setPMEParameters(float(root.get("aEwald")), int(g.get("d0")), int(g.get("d1")), int(g.get("d2")))
    c = root.find("ExtrapolationCoefficients")
    coeff = []
    while c is not None and c.get("c%d" % len(coeff)) is not None:
        coeff.append(float(c.get("c%d" % len(coeff))))
    f.setExtrapolationCoefficients(coeff)
    for i, p in enumerate(root.find("MultipoleParticles").findall("Particle")):
        d = p.find("Dipole")
        Q = p.find("Quadrupole")
        O = p.find("Octopole")
        f.addMultipole(float(p.get("charge")), [float(d.get(k)) for k in ("dX", "dY", "dZ")],
                       [float(Q.get(k)) for k in _QUAD], [float(O.get(k)) for k in _OCT], int(p.get("axisType")),
                       int(p.get("multipoleAtomZ")), int(p.get("multipoleAtomX")), int(p.get("multipoleAtomY")),
                       float(p.get("thole")),
                       [float(p.get(k)) for k in ("polarizabilityXX", "polarizabilityYY", "polarizabilityZZ")])
        for t, name in enumerate(COVALENT_TYPES):
            m = p.find(name)
            f.setCovalentMap(i, t, [int(cv.get("v")) for cv in m.findall("Cv")] if m is not None else [])
    return f
