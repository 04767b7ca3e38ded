"""Python access to the two CPU oracles (test infrastructure only).

* ``ref``  -- the reference's own FP64 CPU force (MPIDReferenceForce.cpp), compiled in
  place by ``make -C oracle ref`` into oracle/_ref/libmpidref.so.  Present only where
  the reference tree is available.
* ``port`` -- this directory's C restatement (mpid_port.c), built by
  ``make -C oracle port`` into oracle/libmpidport.so.  Builds anywhere.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may import this
module; the product never does.
"""
import ctypes
import os
import subprocess
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libmpidref.so")
PORT_LIB = os.path.join(HERE, "libmpidport.so")


@dataclass
class OracleSystem:
    """Flat MPIDForce description (units nm, e, kJ/mol; orders as MPIDForce::addMultipole)."""
    pos: np.ndarray                 # (n, 3)
    charge: np.ndarray              # (n,)
    dipole: np.ndarray              # (n, 3)
    quadrupole: np.ndarray          # (n, 6)  XX XY YY XZ YZ ZZ
    octopole: np.ndarray            # (n, 10) XXX XXY XYY YYY XXZ XYZ YYZ XZZ YZZ ZZZ
    thole: np.ndarray               # (n,)
    polarity: np.ndarray            # (n, 3)
    axis_type: np.ndarray           # (n,)
    atom_z: np.ndarray
    atom_x: np.ndarray
    atom_y: np.ndarray
    covalent: List[List[List[int]]]  # [atom][type 0..7] -> partner list
    box: np.ndarray                 # (3, 3) row vectors
    nonbonded_method: int = 1       # 0 NoCutoff, 1 PME
    polarization_type: int = 0      # 0 Mutual, 1 Direct, 2 Extrapolated
    cutoff: float = 1.0
    ewald_alpha: float = 0.0
    grid: tuple = (0, 0, 0)
    pme_order: int = 6
    mutual_eps: float = 1e-5
    max_iter: int = 60
    extrap_coeffs: tuple = (-0.154, 0.017, 0.658, 0.474)
    default_thole: float = 5.0
    scale14: float = 1.0

    @property
    def n(self):
        return int(self.pos.shape[0])


@dataclass
class OracleResult:
    energy: float
    forces: np.ndarray
    induced: np.ndarray
    labdipoles: Optional[np.ndarray]
    iterations: int
    epsilon: float
    converged: bool
    grad: Optional[np.ndarray] = None  # (n, 20) molecular-frame parameter gradients (port)
    polgrad: Optional[np.ndarray] = None  # (n, 4) polarisability X Y Z and Thole gradients (port)


class _In(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("pos", ctypes.POINTER(ctypes.c_double)),
        ("charge", ctypes.POINTER(ctypes.c_double)),
        ("dipole", ctypes.POINTER(ctypes.c_double)),
        ("quadrupole", ctypes.POINTER(ctypes.c_double)),
        ("octopole", ctypes.POINTER(ctypes.c_double)),
        ("thole", ctypes.POINTER(ctypes.c_double)),
        ("polarity", ctypes.POINTER(ctypes.c_double)),
        ("axis_type", ctypes.POINTER(ctypes.c_int)),
        ("atom_z", ctypes.POINTER(ctypes.c_int)),
        ("atom_x", ctypes.POINTER(ctypes.c_int)),
        ("atom_y", ctypes.POINTER(ctypes.c_int)),
        ("cov_offsets", ctypes.POINTER(ctypes.c_int)),
        ("cov_index", ctypes.POINTER(ctypes.c_int)),
        ("nonbonded_method", ctypes.c_int),
        ("polarization_type", ctypes.c_int),
        ("cutoff", ctypes.c_double),
        ("ewald_alpha", ctypes.c_double),
        ("grid", ctypes.c_int * 3),
        ("pme_order", ctypes.c_int),
        ("box", ctypes.c_double * 9),
        ("mutual_eps", ctypes.c_double),
        ("max_iter", ctypes.c_int),
        ("n_extrap", ctypes.c_int),
        ("extrap_coeffs", ctypes.POINTER(ctypes.c_double)),
        ("default_thole", ctypes.c_double),
        ("scale14", ctypes.c_double),
    ]


class _Out(ctypes.Structure):
    _fields_ = [
        ("energy", ctypes.c_double),
        ("forces", ctypes.POINTER(ctypes.c_double)),
        ("induced", ctypes.POINTER(ctypes.c_double)),
        ("labdipoles", ctypes.POINTER(ctypes.c_double)),
        ("iterations", ctypes.c_int),
        ("epsilon", ctypes.c_double),
        ("converged", ctypes.c_int),
        ("message", ctypes.c_char * 512),
        ("grad", ctypes.POINTER(ctypes.c_double)),
        ("polgrad", ctypes.POINTER(ctypes.c_double)),
    ]


class OracleError(RuntimeError):
    pass


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


_LIBS = {}


def build(which="port"):
    """Build an oracle library with the committed Makefile; returns its path or None."""
    target = {"port": "port", "ref": "ref"}[which]
    if which == "ref" and not os.path.isdir(os.environ.get("MPID_REFERENCE_ROOT", "/root/reference")):
        return None
    env = dict(os.environ)
    if "MPID_REFERENCE_ROOT" in os.environ:
        env["REF"] = os.environ["MPID_REFERENCE_ROOT"]
    subprocess.run(["make", "-s", "-C", HERE, target], check=True, env=env)
    return REF_LIB if which == "ref" else PORT_LIB


def available(which):
    return os.path.exists(REF_LIB if which == "ref" else PORT_LIB)


def _lib(which):
    if which not in _LIBS:
        path = REF_LIB if which == "ref" else PORT_LIB
        if not os.path.exists(path):
            raise OracleError("oracle library %s is not built (make -C oracle %s)" % (path, which))
        lib = ctypes.CDLL(path)
        fn = getattr(lib, "mpidref_evaluate" if which == "ref" else "mpidport_evaluate")
        fn.argtypes = [ctypes.POINTER(_In), ctypes.POINTER(_Out)]
        fn.restype = ctypes.c_int
        _LIBS[which] = fn
    return _LIBS[which]


def _input(sys_: OracleSystem):
    """Flat _In structure for sys_ and the arrays it points into (kept alive together)."""
    n = sys_.n
    pos = np.ascontiguousarray(sys_.pos, dtype=np.float64).reshape(-1)
    arrs = dict(
        charge=np.ascontiguousarray(sys_.charge, dtype=np.float64),
        dipole=np.ascontiguousarray(sys_.dipole, dtype=np.float64).reshape(-1),
        quadrupole=np.ascontiguousarray(sys_.quadrupole, dtype=np.float64).reshape(-1),
        octopole=np.ascontiguousarray(sys_.octopole, dtype=np.float64).reshape(-1),
        thole=np.ascontiguousarray(sys_.thole, dtype=np.float64),
        polarity=np.ascontiguousarray(sys_.polarity, dtype=np.float64).reshape(-1),
    )
    iarrs = dict(
        axis_type=np.ascontiguousarray(sys_.axis_type, dtype=np.int32),
        atom_z=np.ascontiguousarray(sys_.atom_z, dtype=np.int32),
        atom_x=np.ascontiguousarray(sys_.atom_x, dtype=np.int32),
        atom_y=np.ascontiguousarray(sys_.atom_y, dtype=np.int32),
    )
    offs = [0]
    idx = []
    for a in range(n):
        lists = sys_.covalent[a] if a < len(sys_.covalent) else []
        for t in range(8):
            lst = lists[t] if t < len(lists) else []
            idx.extend(int(v) for v in lst)
            offs.append(len(idx))
    offs = np.asarray(offs, dtype=np.int32)
    idx = np.asarray(idx if idx else [0], dtype=np.int32)
    coeffs = np.asarray(sys_.extrap_coeffs, dtype=np.float64)
    inp = _In()
    inp.n = n
    inp.pos = _dp(pos)
    for k, v in arrs.items():
        setattr(inp, k, _dp(v))
    for k, v in iarrs.items():
        setattr(inp, k, _ip(v))
    inp.cov_offsets = _ip(offs)
    inp.cov_index = _ip(idx)
    inp.nonbonded_method = int(sys_.nonbonded_method)
    inp.polarization_type = int(sys_.polarization_type)
    inp.cutoff = float(sys_.cutoff)
    inp.ewald_alpha = float(sys_.ewald_alpha)
    for k in range(3):
        inp.grid[k] = int(sys_.grid[k])
    inp.pme_order = int(sys_.pme_order)
    box = np.asarray(sys_.box, dtype=np.float64).reshape(-1)
    for k in range(9):
        inp.box[k] = box[k]
    inp.mutual_eps = float(sys_.mutual_eps)
    inp.max_iter = int(sys_.max_iter)
    inp.n_extrap = len(coeffs)
    inp.extrap_coeffs = _dp(coeffs)
    inp.default_thole = float(sys_.default_thole)
    inp.scale14 = float(sys_.scale14)
    return inp, (pos, arrs, iarrs, offs, idx, coeffs, box)


def evaluate(sys_: OracleSystem, which="ref", want_labdipoles=False, want_grad=False) -> OracleResult:
    n = sys_.n
    inp, keep = _input(sys_)
    forces = np.zeros(3 * n)
    induced = np.zeros(3 * n)
    lab = np.zeros(3 * n) if want_labdipoles else None
    out = _Out()
    out.forces = _dp(forces)
    out.induced = _dp(induced)
    out.labdipoles = _dp(lab) if lab is not None else None
    grad = None
    if want_grad:
        if which != "port":
            raise OracleError("parameter gradients come from the port")
        grad = np.zeros(20 * n)
        out.grad = _dp(grad)
    else:
        out.grad = None
    polgrad = None
    if want_grad:
        polgrad = np.zeros(4 * n)
        out.polgrad = _dp(polgrad)
    else:
        out.polgrad = None
    rc = _lib(which)(ctypes.byref(inp), ctypes.byref(out))
    if rc != 0:
        raise OracleError(out.message.decode(errors="replace"))
    return OracleResult(energy=out.energy, forces=forces.reshape(n, 3), induced=induced.reshape(n, 3),
                        labdipoles=None if lab is None else lab.reshape(n, 3), iterations=out.iterations,
                        epsilon=out.epsilon, converged=bool(out.converged),
                        grad=None if grad is None else grad.reshape(n, 20),
                        polgrad=None if polgrad is None else polgrad.reshape(n, 4))


def properties(sys_: OracleSystem, masses, grid):
    """The reference's getSystemMultipoleMoments (13 values) and getElectrostaticPotential
    at the (k, 3) grid points (MPIDReferenceKernels.cpp:302-341); reference build only."""
    inp, keep = _input(sys_)
    lib = ctypes.CDLL(REF_LIB) if os.path.exists(REF_LIB) else None
    if lib is None:
        raise OracleError("oracle library %s is not built (make -C oracle ref)" % REF_LIB)
    fn = lib.mpidref_properties
    fn.argtypes = [ctypes.POINTER(_In), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_char_p]
    fn.restype = ctypes.c_int
    m = np.ascontiguousarray(masses, dtype=np.float64)
    g = np.ascontiguousarray(grid, dtype=np.float64).reshape(-1, 3)
    moments = np.zeros(13)
    potential = np.zeros(len(g))
    msg = ctypes.create_string_buffer(512)
    rc = fn(ctypes.byref(inp), _dp(m), _dp(g), len(g), _dp(moments), _dp(potential), msg)
    if rc != 0:
        raise OracleError(msg.value.decode(errors="replace"))
    return moments, potential


def system_from_golden(golden: dict, test: dict) -> OracleSystem:
    """Build an OracleSystem for one entry of tests/golden/reference_tests.json."""
    atoms = golden["systems"][test["system"]]
    n = len(atoms)
    cov = []
    for a in atoms:
        lists = [[] for _ in range(8)]
        for t, lst in a["covalent"].items():
            lists[int(t)] = list(lst)
        cov.append(lists)
    L = test["box"]
    return OracleSystem(
        pos=np.array([a["pos"] for a in atoms]),
        charge=np.array([a["charge"] for a in atoms]),
        dipole=np.array([a["dipole"] for a in atoms]),
        quadrupole=np.array([a["quadrupole"] for a in atoms]),
        octopole=np.array([a["octopole"] for a in atoms]),
        thole=np.array([a["thole"] for a in atoms]),
        polarity=np.array([a["polarity"] for a in atoms]),
        axis_type=np.array([a["axis_type"] for a in atoms]),
        atom_z=np.array([a["atom_z"] for a in atoms]),
        atom_x=np.array([a["atom_x"] for a in atoms]),
        atom_y=np.array([a["atom_y"] for a in atoms]),
        covalent=cov,
        box=np.diag([L, L, L]),
        nonbonded_method=test["nonbonded_method"],
        polarization_type=test["polarization_type"],
        cutoff=test["cutoff"],
        ewald_alpha=test.get("ewald_alpha", 0.0),
        grid=tuple(test.get("grid", (0, 0, 0))),
        pme_order=6,
        mutual_eps=test["mutual_eps"],
        max_iter=test["max_iter"],
        extrap_coeffs=tuple(test["extrap_coeffs"]),
        default_thole=test["default_thole"],
        scale14=test["scale14"],
    )
