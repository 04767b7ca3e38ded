"""CPU tests: host-side API, C ABI exports, synthetic inputs, and the oracle port pinned
to the reference's known answers and to reference runs (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from mpidopenmmplugin_gb300 import MPIDError, MPIDForce, synthetic
from mpidopenmmplugin_gb300 import _build, context
from oracle import oracle as O

import helpers
from test_oracle_golden import CASES, GOLDEN, check_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def port():
    O.build("port")
    return True


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_port_matches_golden(port, case):
    check_case(O.evaluate(O.system_from_golden(GOLDEN, case), "port"), case)


@pytest.mark.parametrize("name", ["water648_direct", "water648_mutual", "water648_extrapolated", "frames_direct",
                                  "frames_mutual", "frames_extrapolated", "triclinic_direct", "triclinic_mutual",
                                  "triclinic_extrapolated"])
def test_port_matches_reference_fixtures(port, name):
    fx = helpers.load_npz_fixture(name + ".npz")
    s = helpers.system_from_fixture(fx)
    p = O.evaluate(s, "port")
    z = [i for i in range(s.n) if int(s.axis_type[i]) == MPIDForce.ZOnly]
    skip = set(z) | set(int(s.atom_z[i]) for i in z)
    mask = np.array([i not in skip for i in range(s.n)])
    assert abs(p.energy - fx["ref_energy"]) / abs(fx["ref_energy"]) < 1e-10
    assert helpers.rel_rms(p.forces[mask], fx["ref_forces"][mask]) < 1e-9
    assert helpers.rel_rms(p.induced, fx["ref_induced"]) < 1e-8


def test_library_exports_every_declared_symbol():
    """libmpid_gb300.so loads without a GPU and exports each function in include/*.h."""
    lib = _build.build()
    decl = open(os.path.join(ROOT, "include", "mpid_gb300.h")).read()
    names = set(re.findall(r"\b(mpid_[a-z_]+)\s*\(", decl))
    assert names == set(context.C_API)
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if l.strip())
    assert names <= exported, names - exported
    import ctypes
    ctypes.CDLL(lib)


def test_force_api_mirrors_reference_defaults():
    f = MPIDForce()
    assert f.getNonbondedMethod() == MPIDForce.NoCutoff
    assert f.getPolarizationType() == MPIDForce.Extrapolated
    assert f.getPmeBSplineOrder() == 6
    assert f.getMutualInducedMaxIterations() == 60
    assert f.getMutualInducedTargetEpsilon() == 1e-5
    assert f.getDefaultTholeWidth() == 5.0
    assert f.getExtrapolationCoefficients() == [-0.154, 0.017, 0.658, 0.474]
    i = f.addMultipole(1.0, [0, 0, 0.1], [0] * 6, [0] * 10, MPIDForce.NoAxisType, -1, -1, -1, 0.3, [1e-3] * 3)
    assert i == 0 and f.getNumMultipoles() == 1
    f.setCovalentMap(0, MPIDForce.Covalent13, [4, 5])
    assert f.getCovalentMap(0, MPIDForce.Covalent13) == [4, 5]
    assert f.getCovalentMaps(0)[MPIDForce.Covalent13] == [4, 5]
    with pytest.raises(MPIDError):
        f.setNonbondedMethod(7)


@pytest.mark.parametrize("bad,match", [
    (dict(quadrupole=[1e-3, 0, 0, 0, 0, 0]), "nonzero trace"),
    (dict(octopole=[1e-3] + [0] * 9), "octopole for particle"),
    (dict(axis=9), "axis type"),
    (dict(z=5), "invalid z axis"),
    (dict(x=-1), "invalid x axis"),
])
def test_validation_rules(bad, match):
    f = MPIDForce()
    q = bad.get("quadrupole", [0] * 6)
    o = bad.get("octopole", [0] * 10)
    f.addMultipole(0.5, [0, 0, 0], q, o, bad.get("axis", MPIDForce.ZThenX), bad.get("z", 1), bad.get("x", 1), -1,
                   0.3, [1e-3] * 3)
    f.addMultipole(-0.5, [0, 0, 0], [0] * 6, [0] * 10, MPIDForce.NoAxisType, -1, -1, -1, 0.3, [1e-3] * 3)
    with pytest.raises(MPIDError, match=match):
        f.validate(2)


def test_cutoff_against_box():
    f, pos, box = synthetic.workload("water648", order=5)
    f.validate(f.getNumMultipoles(), box)
    with pytest.raises(MPIDError, match="half the periodic box"):
        f.validate(f.getNumMultipoles(), np.eye(3) * 1.0)


def test_synthetic_multipoles_are_traceless():
    rng = np.random.default_rng(0)
    q = synthetic.traceless_quadrupole(rng, 1.0, 50)
    assert np.abs(q[:, 0] + q[:, 2] + q[:, 5]).max() < 1e-12
    o = synthetic.traceless_octopole(rng, 1.0, 50)
    for a, b, c in ((0, 2, 7), (1, 3, 8), (4, 6, 9)):
        assert np.abs(o[:, a] + o[:, b] + o[:, c]).max() < 1e-12
    f, pos, box = synthetic.workload("water648")
    assert f.getNumMultipoles() == 648
    d = pos[0::3, None, :] - pos[None, 0::3, :]
    d -= box[0, 0] * np.round(d / box[0, 0])
    r = np.sqrt((d ** 2).sum(-1))
    np.fill_diagonal(r, 10)
    assert r.min() >= 0.26 - 1e-9


@pytest.mark.parametrize("alpha,cutoff", [(3.4, 0.9), (3.5, 0.8), (4.0, 0.7)])
def test_double_float_residual_arithmetic(tmp_path, alpha, cutoff):
    """The df arithmetic and Ewald tables of the residual field (df64.cuh,
    radial_tables.h) against long double: tables, exp(-s), division and square root
    to ~1e-14 relative."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    csrc = os.path.join(ROOT, "mpidopenmmplugin_gb300", "csrc")
    exe = str(tmp_path / "df_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", csrc, os.path.join(ROOT, "tests", "native", "df_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, str(alpha), str(cutoff)], check=True, capture_output=True, text=True).stdout
    errs = {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert set(errs) == {"erfc_table", "erf_table", "exp_neg", "div", "sqrt"}
    for name, e in errs.items():
        assert e < 1e-13, (name, e)


def test_solution_workload_geometry():
    """61,600-atom solution: 20,000 waters + 200 neutral ethanes, solutes away from waters,
    anisotropic polarisabilities and 1-4 partners on the solutes."""
    from scipy.spatial import cKDTree
    f, pos, box = synthetic.workload("solution61k")
    n = f.getNumMultipoles()
    assert n == 61600 and pos.shape == (n, 3)
    assert abs(sum(f.getMultipoleParameters(i)[0] for i in range(n))) < 1e-9
    L = box[0, 0]
    w = pos - L * np.floor(pos / L)
    pairs = cKDTree(w, boxsize=L).query_pairs(0.2, output_type="ndarray")
    mol = np.concatenate([np.repeat(np.arange(20000), 3), 20000 + np.repeat(np.arange(200), 8)])
    inter = pairs[mol[pairs[:, 0]] != mol[pairs[:, 1]]]
    assert not (inter >= 60000).any()  # no solute atom within 2 A of another molecule
    p = f.getMultipoleParameters(60000)
    assert len(set(p[-1])) == 3  # anisotropic
    assert f.getCovalentMap(60002, MPIDForce.Covalent14)
    f.validate(n, box)


def test_radial_functions_against_long_double(tmp_path):
    """Ewald radial functions of the pair kernels (tests/native/radial_check.cpp) against long double:
    FP64 to 1e-14; FP32 to a few ulp with no systematic bias in the erfc recursion."""
    import shutil
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    csrc = os.path.join(ROOT, "mpidopenmmplugin_gb300", "csrc")
    exe = str(tmp_path / "radial_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", csrc, os.path.join(ROOT, "tests", "native", "radial_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "3.4", "0.9"], check=True, capture_output=True, text=True).stdout
    res = {k: (float(a), float(b)) for k, a, b in (line.split() for line in out.strip().splitlines())}
    assert res["erf_double"][0] < 1e-14 and res["erfc_double"][0] < 1e-14
    assert res["erf_float"][0] < 2e-6 and res["erfc_float"][0] < 4e-6
    assert abs(res["erfc_float"][1]) < 2e-8
    assert abs(res["erf_float"][1]) < 1e-7


def test_openmm_adapter_compiles_against_interface_stubs():
    """The OpenMM CUDA-platform adapter (mpidopenmmplugin_gb300/openmm) compiles for
    sm_103a against stand-in headers that declare the OpenMM and MPIDForce interfaces it
    calls (tests/openmm_stub).  OpenMM itself is not installed here, so this checks the
    adapter's code against those declarations only; it does not link or run it."""
    import shutil
    import subprocess
    import tempfile
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    stub = os.path.join(root, "tests", "openmm_stub", "include")
    src = os.path.join(root, "mpidopenmmplugin_gb300", "openmm")
    inc = os.path.join(root, "include")
    with tempfile.TemporaryDirectory() as tmp:
        for f in ("GB300MPIDKernels.cu", "GB300MPIDKernelFactory.cpp"):
            r = subprocess.run([nvcc, "-std=c++17", "-c", "-gencode", "arch=compute_103a,code=sm_103a", "-I", stub,
                                "-I", inc, os.path.join(src, f), "-o", os.path.join(tmp, f + ".o")],
                               capture_output=True, text=True)
            assert r.returncode == 0, r.stderr[-2000:]


def test_bench_reference_arm_json_line():
    """`bench.py --impl reference` (the CPU arm the GPU line is compared with) prints one
    JSON line with the GPU arm's metric and unit, the cpu_baseline and e2e objects, and a
    time bound: here the three warm-up evaluations asked for and one timed evaluation of
    the 24,000-atom box."""
    import json
    import sys
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, check=True, cwd=ROOT).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "evals/s" and d["higher_is_better"] is True
    assert d["metric"].startswith("force+energy evals/s")
    assert d["steps"] == 1 and d["warmup"] == 3 and d["steps_requested"] == 1 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of mpid_settings and mpid_stats have the header's size and field
    offsets (checked against a C program compiled from include/mpid_gb300.h)."""
    import shutil
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not available")
    structs = {"mpid_settings": context.Settings, "mpid_stats": context.Stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "mpid_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_flop_counts_match_bench_constants(tmp_path):
    """bench.py's FLOP/pair figures (the roofline numerator) are the counts that
    tests/native/flop_count.cpp takes from the pair kernels' own per-pair mathematics."""
    import shutil
    import sys
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "flop_count")
    subprocess.run([cxx, "-O0", "-std=c++17", "-I", os.path.join(ROOT, "mpidopenmmplugin_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "flop_count.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    mean = {}
    for line in out.splitlines():
        m = re.match(r"(k_\w+(?: mut)?)\s.*mean\s+(\d+) FLOP/pair", line)
        if m:
            mean[m.group(1)] = int(m.group(2))
    sys.path.insert(0, ROOT)
    import bench
    assert bench.FLOP_PER_PAIR == {"pair_kernel": mean["k_electrostatics mut"],
                                   "dipole_field_pairs": mean["k_dipole_field"],
                                   "fixed_field_pairs": mean["k_fixed_field"]}


@pytest.mark.parametrize("alpha,cutoff", [(3.4, 0.9), (3.5, 0.8), (4.0, 0.7)])
def test_cg_radial_polynomials_against_long_double(tmp_path, alpha, cutoff):
    """The CG pair kernel's radial functions (cg_radial.h: erfc(x) exp(x^2) and the Boys
    functions as fitted polynomials, Thole factors from the inverse damping product)
    against long double over the whole list range: b_1, b_2 within 6e-7 of the pair's
    bare 1/r^3, 3/r^5, and no worse than the general FP32 radial functions of the other
    pair kernels (tests/native/cg_radial_check.cpp)."""
    import shutil
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "cg_radial_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "mpidopenmmplugin_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "cg_radial_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, str(alpha), str(cutoff)], check=True, capture_output=True, text=True).stdout
    vals = {}
    for line in out.splitlines():
        p = line.split()
        vals[p[0]] = (float(p[3]), float(p[8]))  # b1, b2 errors on the bare scale
    poly, general = vals["polynomial"], vals["general"]
    assert poly[0] < 6e-7 and poly[1] < 6e-7, out
    assert poly[0] <= 1.1 * general[0] and poly[1] <= 1.1 * general[1], out
