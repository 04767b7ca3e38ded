"""In-tree build of libmpid_gb300.so for sm_103a (nvcc, no cmake)."""
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libmpid_gb300.so")
SOURCES = ["mpid_context.cu"]
DEPS = ["mpid_context.cu", "mpid_kernels.cuh", "mpid_math.cuh", "qi_tables.cuh", "pme_host.h", "df64.cuh",
        "radial_tables.h", "cg_radial.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmpid_gb300.so")


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, d) for d in DEPS] + [os.path.join(ROOT, "include", "mpid_gb300.h")]
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force=False, verbose=False):
    """Compile the CUDA library in place; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-std=c++17", "-O3", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-shared",
           "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    cmd += [os.path.join(CSRC, s) for s in SOURCES]
    cmd += ["-o", tmp, "-lcufft"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB
