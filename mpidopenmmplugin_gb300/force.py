"""MPIDForce parameter container (host side).

Mirrors the reference's C++/SWIG class `MPIDForce`
(openmmapi/include/openmm/MPIDForce.h:54-489, defaults openmmapi/src/MPIDForce.cpp:43-50):
same method names, argument meaning, parameter orders and validation errors
(openmmapi/src/MPIDForceImpl.cpp:56-150).  A force is evaluated on the GPU through
`mpidopenmmplugin_gb300.MPIDContext`, which plays the part of an OpenMM Context
holding the CalcMPIDForce kernel.
"""
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np


class MPIDError(RuntimeError):
    """Raised where the reference throws OpenMMException."""


@dataclass
class _Multipole:
    charge: float
    dipole: List[float]
    quadrupole: List[float]
    octopole: List[float]
    axis_type: int
    atom_z: int
    atom_x: int
    atom_y: int
    thole: float
    polarity: List[float]
    covalent: List[List[int]] = field(default_factory=lambda: [[] for _ in range(8)])


class MPIDForce:
    # NonbondedMethod (MPIDForce.h:58-71)
    NoCutoff = 0
    PME = 1
    # PolarizationType (MPIDForce.h:73-94)
    Mutual = 0
    Direct = 1
    Extrapolated = 2
    # MultipoleAxisTypes (MPIDForce.h:97)
    ZThenX, Bisector, ZBisect, ThreeFold, ZOnly, NoAxisType, LastAxisTypeIndex = range(7)
    # CovalentType (MPIDForce.h:99-101)
    Covalent12, Covalent13, Covalent14, Covalent15 = 0, 1, 2, 3
    PolarizationCovalent11, PolarizationCovalent12, PolarizationCovalent13, PolarizationCovalent14 = 4, 5, 6, 7
    CovalentEnd = 8

    def __init__(self):
        self._nonbonded = MPIDForce.NoCutoff
        self._polarization = MPIDForce.Extrapolated
        self._pme_order = 6
        self._cutoff = 1.0
        self._ewald_tol = 5e-4
        self._max_iter = 60
        self._target_eps = 1.0e-5
        self._electric = 138.9354558456
        self._default_thole = 5.0
        self._alpha = 0.0
        self._grid = [0, 0, 0]
        self._scale14 = 1.0
        self._extrap = [-0.154, 0.017, 0.658, 0.474]
        self._multipoles: List[_Multipole] = []
        self.forceGroup = 0

    # ---- force-wide settings
    def getForceGroup(self):
        return self.forceGroup

    def setForceGroup(self, group):
        if not 0 <= int(group) <= 31:
            raise MPIDError("Force group must be between 0 and 31")
        self.forceGroup = int(group)

    def getNumMultipoles(self):
        return len(self._multipoles)

    def getNonbondedMethod(self):
        return self._nonbonded

    def setNonbondedMethod(self, method):
        if method not in (0, 1):
            raise MPIDError("MPIDForce: Illegal value for nonbonded method")
        self._nonbonded = int(method)

    def getPolarizationType(self):
        return self._polarization

    def setPolarizationType(self, t):
        self._polarization = int(t)

    def setExtrapolationCoefficients(self, coefficients: Sequence[float]):
        self._extrap = [float(c) for c in coefficients]

    def getExtrapolationCoefficients(self):
        return list(self._extrap)

    def getCutoffDistance(self):
        return self._cutoff

    def setCutoffDistance(self, distance):
        self._cutoff = float(distance)

    def getPMEParameters(self):
        return (self._alpha, self._grid[0], self._grid[1], self._grid[2])

    def setPMEParameters(self, alpha, nx, ny, nz):
        self._alpha = float(alpha)
        self._grid = [int(nx), int(ny), int(nz)]

    def getAEwald(self):
        return self._alpha

    def setAEwald(self, alpha):
        self._alpha = float(alpha)

    def getPmeBSplineOrder(self):
        return self._pme_order

    def setPmeBSplineOrder(self, order):
        """Not in the reference (which fixes order 6); the GB300 kernels support 5 and 6."""
        if order not in (5, 6):
            raise MPIDError("MPIDForce: PME B-spline order must be 5 or 6")
        self._pme_order = int(order)

    def getPmeGridDimensions(self):
        return list(self._grid)

    def setPmeGridDimensions(self, dims):
        self._grid = [int(dims[0]), int(dims[1]), int(dims[2])]

    def getMutualInducedMaxIterations(self):
        return self._max_iter

    def setMutualInducedMaxIterations(self, n):
        self._max_iter = int(n)

    def getMutualInducedTargetEpsilon(self):
        return self._target_eps

    def setMutualInducedTargetEpsilon(self, eps):
        self._target_eps = float(eps)

    def getEwaldErrorTolerance(self):
        return self._ewald_tol

    def setEwaldErrorTolerance(self, tol):
        self._ewald_tol = float(tol)

    def setDefaultTholeWidth(self, val):
        self._default_thole = float(val)

    def getDefaultTholeWidth(self):
        return self._default_thole

    def set14ScaleFactor(self, f):
        self._scale14 = float(f)

    def get14ScaleFactor(self):
        return self._scale14

    def usesPeriodicBoundaryConditions(self):
        return self._nonbonded == MPIDForce.PME

    # ---- per-particle parameters (MPIDForce.h:245-308)
    def addMultipole(self, charge, molecularDipole, molecularQuadrupole, molecularOctopole, axisType,
                     multipoleAtomZ, multipoleAtomX, multipoleAtomY, thole, alphas):
        self._multipoles.append(_Multipole(float(charge), [float(v) for v in molecularDipole],
                                           [float(v) for v in molecularQuadrupole],
                                           [float(v) for v in molecularOctopole], int(axisType), int(multipoleAtomZ),
                                           int(multipoleAtomX), int(multipoleAtomY), float(thole),
                                           [float(v) for v in alphas]))
        m = self._multipoles[-1]
        if len(m.dipole) != 3 or len(m.quadrupole) != 6 or len(m.octopole) != 10 or len(m.polarity) != 3:
            self._multipoles.pop()
            raise MPIDError("MPIDForce: wrong number of multipole components")
        return len(self._multipoles) - 1

    def getMultipoleParameters(self, index):
        m = self._multipoles[index]
        return (m.charge, list(m.dipole), list(m.quadrupole), list(m.octopole), m.axis_type, m.atom_z, m.atom_x,
                m.atom_y, m.thole, list(m.polarity))

    def setMultipoleParameters(self, index, charge, molecularDipole, molecularQuadrupole, molecularOctopole,
                               axisType, multipoleAtomZ, multipoleAtomX, multipoleAtomY, thole, alphas):
        cov = self._multipoles[index].covalent
        self._multipoles[index] = _Multipole(float(charge), [float(v) for v in molecularDipole],
                                             [float(v) for v in molecularQuadrupole],
                                             [float(v) for v in molecularOctopole], int(axisType), int(multipoleAtomZ),
                                             int(multipoleAtomX), int(multipoleAtomY), float(thole),
                                             [float(v) for v in alphas], cov)

    def setCovalentMap(self, index, typeId, covalentAtoms):
        self._multipoles[index].covalent[int(typeId)] = [int(a) for a in covalentAtoms]

    def getCovalentMap(self, index, typeId):
        return list(self._multipoles[index].covalent[int(typeId)])

    def getCovalentMaps(self, index):
        return [list(l) for l in self._multipoles[index].covalent]

    # ---- flat arrays for the C ABI
    def arrays(self):
        ms = self._multipoles
        n = len(ms)
        offs = [0]
        idx = []
        for m in ms:
            for t in range(8):
                idx.extend(m.covalent[t])
                offs.append(len(idx))
        return dict(
            charge=np.array([m.charge for m in ms], dtype=np.float64),
            dipole=np.array([m.dipole for m in ms], dtype=np.float64).reshape(n, 3),
            quadrupole=np.array([m.quadrupole for m in ms], dtype=np.float64).reshape(n, 6),
            octopole=np.array([m.octopole for m in ms], dtype=np.float64).reshape(n, 10),
            axis_type=np.array([m.axis_type for m in ms], dtype=np.int32),
            atom_z=np.array([m.atom_z for m in ms], dtype=np.int32),
            atom_x=np.array([m.atom_x for m in ms], dtype=np.int32),
            atom_y=np.array([m.atom_y for m in ms], dtype=np.int32),
            thole=np.array([m.thole for m in ms], dtype=np.float64),
            polarity=np.array([m.polarity for m in ms], dtype=np.float64).reshape(n, 3),
            cov_offsets=np.array(offs, dtype=np.int32),
            cov_index=np.array(idx if idx else [0], dtype=np.int32),
        )

    # ---- validation of MPIDForceImpl::initialize (MPIDForceImpl.cpp:56-150)
    # Context-side queries of the reference's MPIDForce (MPIDForce.h:228, 379-435), taking
    # an MPIDContext in place of an OpenMM Context.
    def getPMEParametersInContext(self, context):
        return context.getPMEParametersInContext()

    def getLabFramePermanentDipoles(self, context):
        return context.getLabFramePermanentDipoles()

    def getInducedDipoles(self, context):
        return context.getInducedDipoles()

    def getTotalDipoles(self, context):
        return context.getTotalDipoles()

    def getElectrostaticPotential(self, inputGrid, context):
        """At the context's last positions (those of its last evaluate call)."""
        if context.last_positions is None:
            raise MPIDError("getElectrostaticPotential: the context has no positions yet")
        return context.getElectrostaticPotential(inputGrid, context.last_positions, context.last_box)

    def getSystemMultipoleMoments(self, context):
        """At the context's last positions, with the masses the context was created with."""
        if context.last_positions is None or context.masses is None:
            raise MPIDError("getSystemMultipoleMoments: the context needs masses and positions")
        return context.getSystemMultipoleMoments(context.last_positions, context.last_box, context.masses)

    def updateParametersInContext(self, context):
        context.update_parameters(self)

    def validate(self, num_particles, box=None):
        if self.getNumMultipoles() != num_particles:
            raise MPIDError("MPIDForce must have exactly as many particles as the System it belongs to.")
        if self._nonbonded == MPIDForce.PME and box is not None:
            b = np.asarray(box, dtype=np.float64).reshape(3, 3)
            if self._cutoff > 0.5 * b[0, 0] or self._cutoff > 0.5 * b[1, 1] or self._cutoff > 0.5 * b[2, 2]:
                raise MPIDError("MPIDForce: The cutoff distance cannot be greater than half the periodic box size.")
        tol = 1.0e-5
        for i, m in enumerate(self._multipoles):
            q = m.quadrupole
            tr = abs(q[0] + q[2] + q[5])
            if tr > tol:
                raise MPIDError("MPIDForce: quadrupole for particle=%d has nonzero trace: %g; MPID plugin assumes "
                                "traceless quadrupole." % (i, tr))
            o = m.octopole
            for (a, b, c), name in (((0, 2, 7), "(XXX,XYY,XZZ)"), ((1, 3, 8), "(YXX,YYY,YZZ)"),
                                    ((4, 6, 9), "(ZXX,ZYY,ZZZ)")):
                tr = abs(o[a] + o[b] + o[c])
                if tr > tol:
                    raise MPIDError("MPIDForce: %s octopole for particle=%d has nonzero trace: %g; MPID plugin "
                                    "assumes traceless octopoles." % (name, i, tr))
            if m.axis_type not in range(6):
                raise MPIDError("MPIDForce: axis type=%d not currently handled" % m.axis_type)
            if m.axis_type != MPIDForce.NoAxisType and not (0 <= m.atom_z < num_particles):
                raise MPIDError("MPIDForce: invalid z axis particle: %d" % m.atom_z)
            if m.axis_type not in (MPIDForce.NoAxisType, MPIDForce.ZOnly) and not (0 <= m.atom_x < num_particles):
                raise MPIDError("MPIDForce: invalid x axis particle: %d" % m.atom_x)
            if m.axis_type in (MPIDForce.ZBisect, MPIDForce.ThreeFold) and not (0 <= m.atom_y < num_particles):
                raise MPIDError("MPIDForce: invalid y axis particle: %d" % m.atom_y)
