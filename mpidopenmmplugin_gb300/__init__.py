"""GB300-native MPIDForce energy/force evaluation.

`MPIDForce` mirrors the reference's force class (parameters, covalent maps, PME and
solver settings); `MPIDContext` evaluates it on one GPU through the C ABI of
libmpid_gb300.so (include/mpid_gb300.h); `serialization` reads and writes the
reference's XML format; `forcefield` builds an MPIDForce from a force-field XML and a
topology; `fitting` evaluates batches of boxes with per-type parameter gradients.
"""
from .force import MPIDError, MPIDForce
from .context import MPIDContext, load_library, library_path
from . import serialization, forcefield, fitting

__all__ = ["MPIDForce", "MPIDContext", "MPIDError", "load_library", "library_path", "serialization", "forcefield",
           "fitting"]
