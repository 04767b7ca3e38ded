"""Build an MPIDForce from a force-field XML file and a topology.

This restates, without OpenMM, what the reference's `MPIDGenerator` does inside OpenMM's
`ForceField` (python/mpidplugin.i:538-1055):

* `<MPIDForce coulomb14scale=".." defaultTholeWidth="..">` holds `<Multipole>` entries
  (the atom type, the axis-defining types kz / kx / ky, charge c0, dipole dX dY dZ,
  quadrupole qXX qXY qYY qXZ qYZ qZZ and octopole oXXX .. oZZZ in the molecular frame,
  nm units) and `<Polarize>` entries (polarizabilityXX / YY / ZZ in nm^3, thole).  Missing
  multipole components are 0.  A leading '-' on kz / kx / ky marks bisecting axes: the
  axis type follows from which of them are present and signed (`axis_type`).
* `<AtomTypes>` names the types (and their classes); `<Residues>` gives each residue
  template's atoms (name, type) and bonds.
* Each atom of the topology takes the first `<Multipole>` entry of its type whose axis
  atoms can be found, searching in this order: z and x (and y) among its bonded (1-2)
  partners; z a partner and x (and y) a 1-3 atom bonded to z; z a partner and no x; no
  axis atoms.  Ties between candidate atoms go to the lowest index.  Atoms without a
  matching entry are an error.
* Covalent maps 1-2, 1-3 and 1-4 come from the bonds; polarisation defaults to
  Extrapolated, as in the reference generator.

`Topology` is the minimal stand-in for OpenMM's: residues with named atoms and bonds
(bonds not given are taken from the residue templates).
"""
import math
import warnings
import xml.etree.ElementTree as ET

from .force import MPIDForce

_QUAD = ("qXX", "qXY", "qYY", "qXZ", "qYZ", "qZZ")
_OCT = ("oXXX", "oXXY", "oXYY", "oYYY", "oXXZ", "oXYZ", "oYYZ", "oXZZ", "oYZZ", "oZZZ")


def axis_type(kz, kx, ky):
    """Axis type from the (possibly '-'-prefixed) axis-type strings ('' when absent):
    no z -> NoAxisType; z without x -> ZOnly; otherwise ZThenX, or Bisector if z or x is
    signed, ZBisect if x and y are signed, ThreeFold if all three are."""
    zn, xn, yn = kz.startswith("-"), kx.startswith("-"), ky.startswith("-")
    t = MPIDForce.ZThenX
    if not kz:
        t = MPIDForce.NoAxisType
    if kz and not kx:
        t = MPIDForce.ZOnly
    if (kz and zn) or (kx and xn):
        t = MPIDForce.Bisector
    if kx and xn and ky and yn:
        t = MPIDForce.ZBisect
    if kz and zn and kx and xn and ky and yn:
        t = MPIDForce.ThreeFold
    return t


class Topology:
    """Residues of named atoms and the bonds between atoms (global indices)."""

    def __init__(self):
        self.atoms = []      # (atom name, residue index)
        self.residues = []   # (residue name, [atom indices])
        self.bonds = []      # (i, j)
        self._bonded_residues = set()

    def addResidue(self, name, atom_names, bonds=None):
        """Add a residue; `bonds` are (i, j) pairs of indices within the residue (None:
        take them from the force field's template).  Returns the atoms' global indices."""
        first = len(self.atoms)
        idx = list(range(first, first + len(atom_names)))
        r = len(self.residues)
        self.residues.append((name, idx))
        self.atoms.extend((a, r) for a in atom_names)
        if bonds is not None:
            self._bonded_residues.add(r)
            for i, j in bonds:
                self.bonds.append((first + i, first + j))
        return idx

    def addBond(self, i, j):
        """A bond between two atoms (e.g. across residues)."""
        self.bonds.append((int(i), int(j)))
        self._bonded_residues.add(self.atoms[i][1])
        self._bonded_residues.add(self.atoms[j][1])

    def getNumAtoms(self):
        return len(self.atoms)


class ForceField:
    """The parts of an OpenMM force-field XML that define an MPIDForce.  `files` are
    paths or XML strings; several files merge, as OpenMM's ForceField does."""

    def __init__(self, *files):
        self.types = {}       # type name -> {"class", "element", "mass"}
        self.templates = {}   # residue name -> {"atoms": [(name, type)], "bonds": [(i, j)]}
        self.type_map = {}    # type name -> [multipole entries, file order]
        self.scale14 = None
        self.default_thole = None
        self._seen_mpid = False
        for f in files:
            self.load(f)

    def load(self, f):
        root = ET.fromstring(f) if f.lstrip().startswith("<") else ET.parse(f).getroot()
        for t in root.findall("AtomTypes/Type"):
            self.types[t.get("name")] = {"class": t.get("class"), "element": t.get("element"),
                                         "mass": float(t.get("mass", 0.0))}
        for r in root.findall("Residues/Residue"):
            atoms = [(a.get("name"), a.get("type")) for a in r.findall("Atom")]
            names = [a[0] for a in atoms]
            bonds = []
            for b in r.findall("Bond"):
                if b.get("from") is not None:
                    bonds.append((int(b.get("from")), int(b.get("to"))))
                else:
                    bonds.append((names.index(b.get("atomName1")), names.index(b.get("atomName2"))))
            self.templates[r.get("name")] = {"atoms": atoms, "bonds": bonds}
        for el in root.findall("MPIDForce"):
            self._parse_mpid(el)

    def _types_of(self, attrib):
        """Atom types an entry applies to: its `type`, or every type of its `class`."""
        if "type" in attrib:
            if attrib["type"] not in self.types:
                raise ValueError("MPIDGenerator: unknown atom type %s" % attrib["type"])
            return [attrib["type"]]
        if "class" in attrib:
            ts = [n for n, t in self.types.items() if t["class"] == attrib["class"]]
            if ts:
                return ts
            raise ValueError("MPIDGenerator: error getting type for multipole: %s" % attrib["class"])
        raise ValueError("MPIDGenerator: an entry needs a type or class")

    def _parse_mpid(self, el):
        s14, dtw = el.get("coulomb14scale"), el.get("defaultTholeWidth")
        if self._seen_mpid:
            if s14 != self.scale14:
                raise ValueError("Found multiple MPIDForce tags with different coulomb14scale arguments")
            if dtw != self.default_thole:
                raise ValueError("Found multiple MPIDForce tags with different defaultTholeWidth arguments")
        self._seen_mpid = True
        self.scale14, self.default_thole = s14, dtw
        for m in el.findall("Multipole"):
            a = m.attrib
            key = a.get("type", a.get("class"))
            # the axis strings present, in the order kz, kx, ky, fill the z, x, y slots
            raw = [a[k] for k in ("kz", "kx", "ky") if a.get(k)]
            raw += [""] * (3 - len(raw))
            entry = {
                "key": key,
                "axis_type": axis_type(*raw),
                "kz": raw[0].lstrip("-"), "kx": raw[1].lstrip("-"), "ky": raw[2].lstrip("-"),
                "charge": float(a.get("c0")),
                "dipole": [float(a.get(k, 0.0)) for k in ("dX", "dY", "dZ")],
                "quadrupole": [float(a.get(k, 0.0)) for k in _QUAD],
                "octopole": [float(a.get(k, 0.0)) for k in _OCT],
                "polarizability": [0.0, 0.0, 0.0],
                "thole": 0.0,
            }
            for t in self._types_of(a):
                self.type_map.setdefault(t, []).append(dict(entry))
        for p in el.findall("Polarize"):
            a = p.attrib
            key = a.get("type", a.get("class"))
            pol = [float(a["polarizabilityXX"]), float(a["polarizabilityYY"]), float(a["polarizabilityZZ"])]
            thole = float(a["thole"])
            for t in self._types_of(a):
                if t not in self.type_map:
                    raise ValueError("MPIDGenerator: polarize type not present: %s" % key)
                hits = [e for e in self.type_map[t] if e["key"] == key]
                if not hits:
                    raise ValueError("MPIDGenerator: error getting type for polarize: %s not in multipole list?" % key)
                for e in hits:
                    e["polarizability"] = list(pol)
                    e["thole"] = thole

    # ------------------------------------------------------------------ topology

    def atom_types(self, topology):
        """Type of every atom, from its residue template (matched by residue name, then by
        atom name)."""
        out = [None] * topology.getNumAtoms()
        for rname, idx in topology.residues:
            tpl = self.templates.get(rname)
            if tpl is None:
                raise ValueError("No template found for residue %s" % rname)
            bytype = dict(tpl["atoms"])
            for i in idx:
                name = topology.atoms[i][0]
                if name not in bytype:
                    raise ValueError("Atom %s of residue %s is not in its template" % (name, rname))
                out[i] = bytype[name]
        return out

    def bonds(self, topology):
        """The topology's bonds, plus template bonds of residues added without any."""
        bonds = list(topology.bonds)
        for r, (rname, idx) in enumerate(topology.residues):
            if r in topology._bonded_residues:
                continue
            tpl = self.templates[rname]
            names = [topology.atoms[i][0] for i in idx]
            tnames = [a[0] for a in tpl["atoms"]]
            for i, j in tpl["bonds"]:
                bonds.append((idx[names.index(tnames[i])], idx[names.index(tnames[j])]))
        return bonds

    @staticmethod
    def bonded_sets(n, bonds):
        """1-2, 1-3 and 1-4 sets of every atom."""
        b12 = [set() for _ in range(n)]
        for i, j in bonds:
            b12[i].add(j)
            b12[j].add(i)
        b13 = []
        for i in range(n):
            s = set()
            for j in b12[i]:
                s |= b12[j]
            b13.append(s - b12[i] - {i})
        b14 = []
        for i in range(n):
            s = set()
            for j in b13[i]:
                s |= b12[j]
            b14.append(s - b12[i] - b13[i] - {i})
        return b12, b13, b14

    @staticmethod
    def _axis_atoms(entries, types, i, b12, b13):
        """(entry, z, x, y) for atom i: the first entry, pass by pass, whose axis types
        are found among i's bonded atoms (see the module docstring); None if none is."""
        p12 = sorted(b12[i])
        p13 = sorted(b13[i])
        # pass 1: z, x (and y) all bonded to i
        for e in entries:
            kz, kx, ky = e["kz"], e["kx"], e["ky"]
            if not kz or not kx:
                continue
            for z in p12:
                if types[z] != kz:
                    continue
                for x in p12:
                    if x == z or types[x] != kx:
                        continue
                    if not ky:
                        if types[x] == types[z] and x < z:
                            return e, x, z, -1
                        xs = [c for c in p12 if types[c] == kx and c != z]
                        return e, z, min(xs), -1
                    for y in p12:
                        if y in (z, x) or types[y] != ky:
                            continue
                        return e, z, x, y
        # pass 2: z bonded to i; x (and y) bonded to z, two bonds from i
        for e in entries:
            kz, kx, ky = e["kz"], e["kx"], e["ky"]
            if not kz or not kx:
                continue
            for z in p12:
                if types[z] != kz:
                    continue
                for x in p13:
                    if x == z or types[x] != kx or z not in b12[x]:
                        continue
                    if not ky:
                        xs = [c for c in p13 if types[c] == kx and c != z and z in b12[c]]
                        return e, z, min(xs), -1
                    for y in p13:
                        if y in (z, x) or types[y] != ky or z not in b12[y]:
                            continue
                        return e, z, x, y
        # pass 3: z only
        for e in entries:
            if e["kz"] and not e["kx"]:
                for z in p12:
                    if types[z] == e["kz"]:
                        return e, z, -1, -1
        # pass 4: no axis atoms
        for e in entries:
            if not e["kz"]:
                return e, -1, -1, -1
        return None

    def createForce(self, topology, nonbondedMethod=MPIDForce.PME, nonbondedCutoff=1.0, **args):
        """MPIDForce for `topology` (the arguments of the reference generator's
        createForce: polarization ('direct' | 'mutual' | 'extrapolated', default
        extrapolated), coulomb14scale, defaultTholeWidth, aEwald, pmeGridDimensions,
        mutualInducedMaxIterations, mutualInducedTargetEpsilon, ewaldErrorTolerance)."""
        force = MPIDForce()
        if nonbondedMethod not in (MPIDForce.NoCutoff, MPIDForce.PME):
            raise ValueError("MPIDForce: input cutoff method not available.")
        force.setNonbondedMethod(nonbondedMethod)
        force.setCutoffDistance(nonbondedCutoff)
        if "ewaldErrorTolerance" in args:
            force.setEwaldErrorTolerance(float(args["ewaldErrorTolerance"]))
        force.setPolarizationType(MPIDForce.Extrapolated)
        if "polarization" in args:
            p = str(args["polarization"]).lower()
            kinds = {"direct": MPIDForce.Direct, "mutual": MPIDForce.Mutual, "extrapolated": MPIDForce.Extrapolated}
            if p not in kinds:
                raise ValueError("MPIDForce: invalide polarization type: " + str(args["polarization"]))
            force.setPolarizationType(kinds[p])
        for key, mine, setter in (("coulomb14scale", self.scale14, force.set14ScaleFactor),
                                  ("defaultTholeWidth", self.default_thole, force.setDefaultTholeWidth)):
            argval = float(args[key]) if key in args else None
            myval = float(mine) if mine else None
            if argval is not None:
                if myval is not None and myval != argval:
                    warnings.warn("Conflicting %s values found in forcefield file (%s) and createSystem args (%s).  "
                                  "Using the value from createSystem's arguments" % (key, myval, argval))
                setter(argval)
            elif myval is not None:
                setter(myval)
        if "aEwald" in args:
            force.setAEwald(float(args["aEwald"]))
        if "pmeGridDimensions" in args:
            force.setPmeGridDimensions(list(args["pmeGridDimensions"]))
        if "mutualInducedMaxIterations" in args:
            force.setMutualInducedMaxIterations(int(args["mutualInducedMaxIterations"]))
        if "mutualInducedTargetEpsilon" in args:
            force.setMutualInducedTargetEpsilon(float(args["mutualInducedTargetEpsilon"]))

        types = self.atom_types(topology)
        n = len(types)
        b12, b13, b14 = self.bonded_sets(n, self.bonds(topology))
        for i in range(n):
            name, r = topology.atoms[i]
            where = "%s of %s %d" % (name, topology.residues[r][0], r)
            if types[i] not in self.type_map:
                raise ValueError("No multipole type for atom " + where)
            hit = self._axis_atoms(self.type_map[types[i]], types, i, b12, b13)
            if hit is None:
                raise ValueError("Atom %s was not assigned." % where)
            e, z, x, y = hit
            force.addMultipole(e["charge"], e["dipole"], e["quadrupole"], e["octopole"], e["axis_type"], z, x, y,
                               e["thole"], e["polarizability"])
            force.setCovalentMap(i, MPIDForce.Covalent12, sorted(b12[i]))
            force.setCovalentMap(i, MPIDForce.Covalent13, sorted(b13[i]))
            force.setCovalentMap(i, MPIDForce.Covalent14, sorted(b14[i]))
        return force


def pme_parameters(cutoff, box, tolerance=5e-4, minimum=5):
    """Ewald alpha (1/nm) and grid for a cutoff (nm), box edges (nm) and error tolerance,
    by the published rule OpenMM documents for its PME: alpha = sqrt(-ln(2 tol)) / cutoff,
    n_k = ceil(2 alpha L_k / (3 tol^(1/5))) rounded up to a product of 2, 3, 5 and 7 (at
    least `minimum`, the B-spline order)."""
    alpha = math.sqrt(-math.log(2.0 * tolerance)) / cutoff

    def smooth(n):
        while True:
            m = n
            for f in (2, 3, 5, 7):
                while m % f == 0:
                    m //= f
            if m == 1:
                return n
            n += 1

    grid = [smooth(max(minimum, int(math.ceil(2.0 * alpha * L / (3.0 * tolerance ** 0.2))))) for L in box]
    return alpha, grid
