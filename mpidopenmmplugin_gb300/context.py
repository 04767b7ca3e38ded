"""GPU evaluation of an MPIDForce through the C ABI of libmpid_gb300.so.

`MPIDContext(force, num_particles)` creates the device context (the part of an OpenMM
Context that owns the CalcMPIDForce kernel, MPIDCudaKernels.cpp:210-662) and
`evaluate(positions, box)` runs CalcMPIDForceKernel::execute (mpidKernels.h:77).
There is no CPU fallback: without the library or a CUDA device the calls raise.
"""
import ctypes
import os

import numpy as np

from . import _build
from .force import MPIDError, MPIDForce

MPID_PRECISION_MIXED = 0
MPID_PRECISION_DOUBLE = 1
MPID_FLAG_EXACT_ANISO_TORQUE = 1
MPID_FLAG_NEAR_FIELD_PCG = 2
MPID_FLAG_GRAPH_SOLVER = 4
MPID_FLAG_SERIAL_STAGES = 8

# Entry points declared in include/mpid_gb300.h
C_API = ["mpid_default_settings", "mpid_create", "mpid_destroy", "mpid_set_multipoles", "mpid_set_covalent",
         "mpid_evaluate", "mpid_evaluate_device", "mpid_evaluate_device_noalloc", "mpid_get_dipoles",
         "mpid_get_pme_parameters", "mpid_get_stats", "mpid_last_error", "mpid_get_system_multipole_moments",
         "mpid_get_electrostatic_potential", "mpid_get_parameter_gradients", "mpid_evaluate_with_gradients",
         "mpid_evaluate_batch", "mpid_set_work_split", "mpid_set_atom_types"]


class Settings(ctypes.Structure):
    _fields_ = [
        ("num_atoms", ctypes.c_int),
        ("nonbonded_method", ctypes.c_int),
        ("polarization_type", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("ewald_alpha", ctypes.c_double),
        ("grid", ctypes.c_int * 3),
        ("pme_order", ctypes.c_int),
        ("mutual_eps", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("n_extrap", ctypes.c_int),
        ("extrap_coeffs", ctypes.c_double * 8),
        ("default_thole", ctypes.c_double),
        ("scale14", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("flags", ctypes.c_uint),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("solver_iterations", ctypes.c_int),
        ("refinement_steps", ctypes.c_int),
        ("solver_residual", ctypes.c_double),
        ("max_neighbours", ctypes.c_int),
        ("ms_total", ctypes.c_double),
        ("ms_stage", ctypes.c_double * 8),
        ("stage_launches", ctypes.c_int * 8),
        ("energy_parts", ctypes.c_double * 3),
        ("kernel_launches", ctypes.c_int),
        ("library_calls", ctypes.c_int),
        ("graph_captures", ctypes.c_int),
        ("graph_replays", ctypes.c_int),
        ("device_allocations", ctypes.c_longlong),
    ]


STAGES = ["setup", "fixed_field_pairs", "pme", "dipole_field_pairs", "cufft", "pair_kernel", "recip_self_torque",
          "refinement_field_pairs"]


_LIB = None


def library_path():
    return _build.LIB


def load_library(build=True):
    """Load libmpid_gb300.so (building it in place when missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise MPIDError("libmpid_gb300.so is not built; run mpidopenmmplugin_gb300._build.build()")
    lib = ctypes.CDLL(_build.LIB)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    lib.mpid_default_settings.argtypes = [ctypes.POINTER(Settings), ctypes.c_int]
    lib.mpid_default_settings.restype = None
    lib.mpid_create.argtypes = [ctypes.POINTER(Settings), ctypes.c_int, ctypes.POINTER(vp)]
    lib.mpid_destroy.argtypes = [vp]
    lib.mpid_destroy.restype = None
    lib.mpid_set_multipoles.argtypes = [vp, dp, dp, dp, dp, ip, ip, ip, ip, dp, dp]
    lib.mpid_set_covalent.argtypes = [vp, ip, ip]
    lib.mpid_evaluate.argtypes = [vp, dp, dp, dp, dp]
    lib.mpid_evaluate_device.argtypes = [vp, vp, dp, vp, vp, vp]
    lib.mpid_evaluate_device_noalloc.argtypes = [vp, vp, dp, vp, vp, vp]
    lib.mpid_get_dipoles.argtypes = [vp, ctypes.c_int, dp]
    lib.mpid_get_pme_parameters.argtypes = [vp, dp, ip, ip, ip]
    lib.mpid_get_system_multipole_moments.argtypes = [vp, dp, dp, dp, dp]
    lib.mpid_get_electrostatic_potential.argtypes = [vp, dp, dp, dp, ctypes.c_int, dp]
    lib.mpid_get_parameter_gradients.argtypes = [vp, dp, dp, dp]
    lib.mpid_evaluate_with_gradients.argtypes = [vp, dp, dp, dp, dp, dp, dp]
    pp = ctypes.POINTER(ctypes.c_void_p)
    lib.mpid_evaluate_batch.argtypes = [pp, ctypes.c_int, pp, pp, pp, dp, pp, pp, dp, ctypes.c_int]
    lib.mpid_set_work_split.argtypes = [vp, ctypes.c_int]
    lib.mpid_set_atom_types.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.mpid_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    lib.mpid_last_error.argtypes = []
    lib.mpid_last_error.restype = ctypes.c_char_p
    for name in C_API:
        if name not in ("mpid_default_settings", "mpid_destroy", "mpid_last_error"):
            getattr(lib, name).restype = ctypes.c_int
    _LIB = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class MPIDContext:
    """One MPIDForce on one GPU.

    precision: "mixed" (FP32 pair/PME/solver, 64-bit fixed-point forces, FP64 energy and
    FP64 residual refinement) or "double" (FP64 throughout).
    """

    def __init__(self, force: MPIDForce, num_particles=None, device=0, precision="mixed",
                 exact_aniso_torque=False, box=None, preconditioner=False, masses=None, solver_graphs=True,
                 serial_stages=False):
        """masses: per-atom masses for getSystemMultipoleMoments through the force's
        context methods (the System's masses in the reference).  box: the periodic box,
        needed when the force's PME parameters are 0 (chosen from its Ewald error
        tolerance, as the reference kernel does through OpenMM).  solver_graphs: under PME,
        replay the evaluation's launches (set-up, solver start, solver iterations,
        force/energy phase, gradient passes) from CUDA graphs captured on first use; calls
        on the legacy default stream (device pointers with stream 0) launch directly.
        serial_stages: profiling; the side streams fold onto the calling stream so that the
        stage times of stats() add up to the evaluation's device time, with the cuFFT
        executions as their own stage ("cufft")."""
        self.lib = load_library()
        n = force.getNumMultipoles() if num_particles is None else int(num_particles)
        force.validate(n, box)
        s = Settings()
        self.lib.mpid_default_settings(ctypes.byref(s), n)
        s.nonbonded_method = force.getNonbondedMethod()
        s.polarization_type = force.getPolarizationType()
        s.cutoff = force.getCutoffDistance()
        alpha, nx, ny, nz = force.getPMEParameters()
        if force.getNonbondedMethod() == MPIDForce.PME and (alpha == 0.0 or 0 in (nx, ny, nz)):
            # the automatic choice of MPIDCudaKernels.cpp:440-449 (OpenMM's rule)
            if box is None:
                raise MPIDError("MPIDForce: PME parameters are 0; give the periodic box to choose them from the "
                                "Ewald error tolerance")
            from .forcefield import pme_parameters
            b = np.asarray(box, dtype=np.float64).reshape(3, 3)
            alpha, (nx, ny, nz) = pme_parameters(force.getCutoffDistance(), [b[0, 0], b[1, 1], b[2, 2]],
                                                 force.getEwaldErrorTolerance(), minimum=force.getPmeBSplineOrder())
        self.masses = None if masses is None else np.asarray(masses, dtype=np.float64).reshape(n)
        self.last_positions = None
        self.last_box = None
        s.ewald_alpha = alpha
        s.grid[0], s.grid[1], s.grid[2] = nx, ny, nz
        s.pme_order = force.getPmeBSplineOrder()
        s.mutual_eps = force.getMutualInducedTargetEpsilon()
        s.max_iter = force.getMutualInducedMaxIterations()
        c = force.getExtrapolationCoefficients()
        if len(c) > 8:
            raise MPIDError("at most 8 extrapolation coefficients are supported")
        s.n_extrap = len(c)
        for i, v in enumerate(c):
            s.extrap_coeffs[i] = v
        s.default_thole = force.getDefaultTholeWidth()
        s.scale14 = force.get14ScaleFactor()
        s.precision = {"mixed": MPID_PRECISION_MIXED, "double": MPID_PRECISION_DOUBLE}[precision]
        s.flags = ((MPID_FLAG_EXACT_ANISO_TORQUE if exact_aniso_torque else 0) |
                   (MPID_FLAG_NEAR_FIELD_PCG if preconditioner else 0) |
                   (MPID_FLAG_GRAPH_SOLVER if solver_graphs else 0) |
                   (MPID_FLAG_SERIAL_STAGES if serial_stages else 0))
        self.n = n
        self.precision = precision
        self.device = int(device)
        self._h = ctypes.c_void_p()
        self._check(self.lib.mpid_create(ctypes.byref(s), int(device), ctypes.byref(self._h)))
        self.update_parameters(force)

    def _check(self, rc):
        if rc != 0:
            raise MPIDError(self.lib.mpid_last_error().decode(errors="replace"))

    def update_parameters(self, force: MPIDForce):
        """updateParametersInContext (MPIDForce.h:435): copy multipoles and covalent maps."""
        if force.getNumMultipoles() != self.n:
            raise MPIDError("updateParametersInContext: The number of multipoles has changed")
        a = force.arrays()
        self._arrays = a  # keep alive
        self._check(self.lib.mpid_set_multipoles(self._h, _dp(a["charge"]), _dp(a["dipole"]), _dp(a["quadrupole"]),
                                                 _dp(a["octopole"]), _ip(a["axis_type"]), _ip(a["atom_z"]),
                                                 _ip(a["atom_x"]), _ip(a["atom_y"]), _dp(a["thole"]),
                                                 _dp(a["polarity"])))
        self._check(self.lib.mpid_set_covalent(self._h, _ip(a["cov_offsets"]), _ip(a["cov_index"])))

    def evaluate(self, positions, box, forces=None):
        """Energy (kJ/mol) and forces (n, 3) (kJ/mol/nm); forces are ADDED to `forces` if given."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(self.n, 3)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self.last_positions, self.last_box = pos.copy(), b.copy()
        f = np.zeros((self.n, 3)) if forces is None else np.ascontiguousarray(forces, dtype=np.float64)
        e = ctypes.c_double(0.0)
        self._check(self.lib.mpid_evaluate(self._h, _dp(pos), _dp(b), _dp(f), ctypes.byref(e)))
        return e.value, f

    def evaluate_device(self, d_positions, box, d_forces, d_energy=0, stream=0):
        """Device-pointer evaluation (integers are raw CUDA addresses)."""
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self._check(self.lib.mpid_evaluate_device(self._h, ctypes.c_void_p(d_positions), _dp(b),
                                                  ctypes.c_void_p(d_forces), ctypes.c_void_p(d_energy),
                                                  ctypes.c_void_p(stream)))

    def evaluate_device_noalloc(self, d_positions, box, d_forces, d_energy=0, stream=0):
        """evaluate_device through the allocation-free entry point (PME, small systems)."""
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        self._check(self.lib.mpid_evaluate_device_noalloc(self._h, ctypes.c_void_p(d_positions), _dp(b),
                                                          ctypes.c_void_p(d_forces), ctypes.c_void_p(d_energy),
                                                          ctypes.c_void_p(stream)))

    def _dipoles(self, which):
        out = np.zeros((self.n, 3))
        self._check(self.lib.mpid_get_dipoles(self._h, int(which), _dp(out)))
        return out

    def getInducedDipoles(self):
        return self._dipoles(0)

    def getLabFramePermanentDipoles(self):
        return self._dipoles(1)

    def getTotalDipoles(self):
        return self._dipoles(2)

    def getPermanentField(self):
        """Permanent electric field at each atom (e/nm^2) of the last evaluation."""
        return self._dipoles(3)

    def getSystemMultipoleMoments(self, positions, box, masses):
        """MPIDForce::getSystemMultipoleMoments (MPIDForce.h:423): 13 values at `positions`."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(self.n, 3)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        m = np.ascontiguousarray(masses, dtype=np.float64).reshape(self.n)
        out = np.zeros(13)
        self._check(self.lib.mpid_get_system_multipole_moments(self._h, _dp(pos), _dp(b), _dp(m), _dp(out)))
        return out

    def getElectrostaticPotential(self, grid, positions, box):
        """MPIDForce::getElectrostaticPotential (MPIDForce.h:404): potential (kJ/mol/e) at
        the (k, 3) grid points, with the induced dipoles at `positions`."""
        g = np.ascontiguousarray(grid, dtype=np.float64).reshape(-1, 3)
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(self.n, 3)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        out = np.zeros(len(g))
        self._check(self.lib.mpid_get_electrostatic_potential(self._h, _dp(pos), _dp(b), _dp(g), len(g), _dp(out)))
        return out

    def getParameterGradients(self, positions, box):
        """dE/d(molecular-frame multipole parameters) at `positions`, shape (n, 20): charge,
        dipole X Y Z, quadrupole XX XY YY XZ YZ ZZ, octopole XXX ... ZZZ."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(self.n, 3)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        out = np.zeros((self.n, 20))
        self._check(self.lib.mpid_get_parameter_gradients(self._h, _dp(pos), _dp(b), _dp(out)))
        return out

    def evaluateWithGradients(self, positions, box, forces=True, multipole=True, polarization=True):
        """One evaluation returning (energy, forces (n, 3) or None, multipole-parameter
        gradients (n, 20) or None, polarisation gradients (n, 4) or None).  The
        polarisation gradients are dE/d(molecular-frame polarisability X Y Z) and
        dE/d(Thole width)."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(self.n, 3)
        b = np.ascontiguousarray(box, dtype=np.float64).reshape(9)
        f = np.zeros((self.n, 3)) if forces else None
        gm = np.zeros((self.n, 20)) if multipole else None
        gp = np.zeros((self.n, 4)) if polarization else None
        e = ctypes.c_double(0.0)
        null = ctypes.POINTER(ctypes.c_double)()
        self._check(self.lib.mpid_evaluate_with_gradients(
            self._h, _dp(pos), _dp(b), null if f is None else _dp(f), ctypes.byref(e),
            null if gm is None else _dp(gm), null if gp is None else _dp(gp)))
        return e.value, f, gm, gp

    def setAtomTypes(self, types, ntypes):
        """Parameter types of the atoms (0 .. ntypes-1, ntypes <= 16) for the per-type
        gradient sums of evaluate_batch(type_grad=True) (mpid_set_atom_types)."""
        t = np.ascontiguousarray(types, dtype=np.int32).reshape(self.n)
        self._check(self.lib.mpid_set_atom_types(self._h, t.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(ntypes)))
        self.ntypes = int(ntypes)

    def setWorkSplit(self, max_split):
        """Upper bound (power of two up to 32, 0 = automatic) of the warps each pair-kernel
        work item is cut into (mpid_set_work_split)."""
        self._check(self.lib.mpid_set_work_split(self._h, int(max_split)))

    def getPMEParametersInContext(self):
        a = ctypes.c_double()
        nx, ny, nz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.mpid_get_pme_parameters(self._h, ctypes.byref(a), ctypes.byref(nx), ctypes.byref(ny),
                                                     ctypes.byref(nz)))
        return a.value, nx.value, ny.value, nz.value

    def stats(self):
        s = Stats()
        self._check(self.lib.mpid_get_stats(self._h, ctypes.byref(s)))
        return dict(solver_iterations=s.solver_iterations, refinement_steps=s.refinement_steps,
                    solver_residual=s.solver_residual, max_neighbours=s.max_neighbours, ms_total=s.ms_total,
                    ms_stage={STAGES[k]: s.ms_stage[k] for k in range(len(STAGES))},
                    stage_launches={STAGES[k]: s.stage_launches[k] for k in range(len(STAGES))},
                    energy_parts=dict(recip_self=s.energy_parts[0], real_space=s.energy_parts[1],
                                      scaled_pairs=s.energy_parts[2]),
                    kernel_launches=s.kernel_launches, library_calls=s.library_calls,
                    graph_captures=s.graph_captures, graph_replays=s.graph_replays,
                    device_allocations=s.device_allocations)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self.lib.mpid_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def evaluate_batch(contexts, positions, boxes, forces=True, multipole=True, polarization=True, launch=0, flat=False,
                   type_grad=False):
    """mpid_evaluate_batch over MPIDContexts of PME systems on one device.  launch 0
    (fused): one kernel launch per operation for all boxes (each box's evaluation recorded
    once, operation i of every box launched together, FFTs batched per grid size; boxes of
    at most 4096 atoms); -1: each box's evaluation as a graph, all in one parent graph;
    k > 0: each box's graph on one of k streams.  The first call of a context, and any
    context whose list shape or solver length changed, takes the ordinary evaluation.
    Returns (energies (k,), forces [(n, 3)] or None, multipole gradients [(n, 20)] or
    None, polarisation gradients [(n, 4)] or None); the per-box arrays are consecutive
    rows of one array per quantity, which flat=True returns instead ((sum n, 3), ...).
    type_grad=True (every context with setAtomTypes) appends the (ntypes, 24) per-type
    sums of the 20 multipole and 4 polarisation gradient components over all boxes,
    summed on the device per box."""
    k = len(contexts)
    if k == 0:
        return np.zeros(0), None, None, None
    lib = contexts[0].lib
    keep = []

    sizes = [c.n for c in contexts]
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)

    def rows(width):
        whole = np.zeros((int(offsets[-1]), width))
        keep.append(whole)
        return whole, [whole[offsets[i]:offsets[i + 1]] for i in range(k)]

    def ptrs(arrays):
        out = (ctypes.c_void_p * k)(*[None if a is None else a.ctypes.data for a in arrays])
        return ctypes.cast(out, ctypes.POINTER(ctypes.c_void_p)), out

    pos = [np.ascontiguousarray(p, dtype=np.float64).reshape(c.n, 3) for c, p in zip(contexts, positions)]
    bx = [np.ascontiguousarray(b, dtype=np.float64).reshape(9) for b in boxes]
    fo_all, fo = rows(3) if forces else (None, None)
    gm_all, gm = rows(20) if multipole else (None, None)
    gp_all, gp = rows(4) if polarization else (None, None)
    e = np.zeros(k)
    cp, cbuf = ptrs([None] * k)
    for i, c in enumerate(contexts):
        cbuf[i] = c._h.value
    pp, pbuf = ptrs(pos)
    bp, bbuf = ptrs(bx)
    null = ctypes.POINTER(ctypes.c_void_p)()
    fp = ptrs(fo) if fo is not None else (null, None)
    mp = ptrs(gm) if gm is not None else (null, None)
    qp = ptrs(gp) if gp is not None else (null, None)
    tg = np.zeros((getattr(contexts[0], "ntypes", 0), 24)) if type_grad else None
    tgp = _dp(tg) if type_grad else ctypes.POINTER(ctypes.c_double)()
    contexts[0]._check(lib.mpid_evaluate_batch(cp, k, pp, bp, fp[0], _dp(e), mp[0], qp[0], tgp, int(launch)))
    for c, p, b in zip(contexts, pos, bx):
        c.last_positions, c.last_box = p.copy(), b.copy()
    out = (e, fo_all, gm_all, gp_all) if flat else (e, fo, gm, gp)
    return out + (tg,) if type_grad else out
