"""Extract the reference's known-answer tests into a JSON fixture.

Reads platforms/reference/tests/TestReferenceMPIDForce.cpp of the reference tree AS
TEXT (nothing there is compiled or run) and writes tests/golden/reference_tests.json:

* the three fixture systems the tests build -- the 4-atom charge square
  (TestReferenceMPIDForce.cpp:64-107), the 6-atom water dimer (:109-660) and the
  12-atom methanol dimer (:662-880) -- as flat per-atom parameter lists;
* the 14 tests run by main() (:1702-1730): their nonbonded method, PME parameters,
  polarisation type, Thole width, 1-4 scale, and the golden energy / forces with the
  tolerance the test asserts.

Usage:  python tests/golden/extract_reference_tests.py [REFERENCE_ROOT]
The JSON is committed; the tests read only the JSON.
"""
import json
import re
import sys
from pathlib import Path

NM_PER_ANGSTROM = 0.1
AXIS = {"ZThenX": 0, "Bisector": 1, "ZBisect": 2, "ThreeFold": 3, "ZOnly": 4, "NoAxisType": 5}
COVALENT = {"Covalent12": 0, "Covalent13": 1, "Covalent14": 2, "Covalent15": 3,
            "PolarizationCovalent11": 4, "PolarizationCovalent12": 5,
            "PolarizationCovalent13": 6, "PolarizationCovalent14": 7}
POLTYPE = {"Mutual": 0, "Direct": 1, "Extrapolated": 2}
# MPIDForce constructor defaults (openmmapi/src/MPIDForce.cpp:43-50).
DEFAULTS = dict(polarization_type=2, max_iter=60, mutual_eps=1e-5, default_thole=5.0,
                scale14=1.0, extrap_coeffs=[-0.154, 0.017, 0.658, 0.474])


def num_list(text):
    return [float(x) for x in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", text)]


def function_body(src, name):
    m = re.search(r"void\s+%s\s*\([^)]*\)\s*\{" % re.escape(name), src)
    if not m:
        raise KeyError(name)
    depth, i = 1, m.end()
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    return src[m.end():i - 1]


def strip_disabled_blocks(body):
    # `if(!do_x){ ... }` blocks zero parameters when a flag is off; every test keeps
    # all flags on, so those blocks are dropped.
    return re.sub(r"if\s*\(\s*!do_\w+\s*\)\s*\{[^{}]*\}", "", body)


def parse_box_fixture(body, natoms):
    body = strip_disabled_blocks(body)
    arrays = {}
    for m in re.finditer(r"(?:const\s+)?(?:double|int)\s+(\w+)\s*\[\s*\d+\s*\]\s*=\s*\{(.*?)\};", body, re.S):
        arrays[m.group(1)] = num_list(m.group(2))
    for m in re.finditer(r"std::vector<\w+>\s+(\w+)\s*\(\s*&(\w+)\[0\]\s*,\s*&\w+\[\d+\]\s*\)\s*;", body):
        arrays[m.group(1)] = arrays[m.group(2)]
    for m in re.finditer(r"std::vector<double>\s+(\w+)\s*\{(.*?)\}\s*;", body, re.S):
        arrays[m.group(1)] = num_list(m.group(2))
    maps = {}
    for m in re.finditer(r"(\w+)map\[\"(\w+)\"\]\s*=\s*(.*?);", body, re.S):
        kind, key, rhs = m.group(1), m.group(2), m.group(3).strip()
        if kind in maps and key in maps[kind]:
            continue
        if rhs.startswith("MPIDForce::"):
            val = AXIS[rhs.split("::")[1]]
        elif rhs.startswith("std::vector<double>{"):
            val = num_list(rhs[len("std::vector<double>"):])
        elif rhs.startswith("std::vector<int>()"):
            val = []
        elif rhs in arrays:
            val = arrays[rhs]
        else:
            val = float(rhs)
        maps.setdefault(kind, {})[key] = val
    types_m = re.search(r"const char\*\s*atom_types\[\d+\]\s*=\s*\{(.*?)\};", body, re.S)
    types = re.findall(r"\"(\w+)\"", types_m.group(1))
    coords_m = re.search(r"if\s*\(\s*natoms\s*==\s*%d\s*\)\s*\{\s*const double coords\[\d+\]\[3\]\s*=\s*\{(.*?)\};" % natoms,
                         body, re.S)
    xyz = num_list(coords_m.group(1))
    assert len(xyz) == 3 * natoms
    # How the axis atoms are derived from anchors differs between the two fixtures:
    # the water fixture always offsets X (TestReferenceMPIDForce.cpp:631-632), the
    # methanol fixture maps a zero X anchor to -1 (:863-864).
    x_zero_means_none = "anchormap[element][1]==0" in body.replace(" ", "")
    atoms = []
    for a in range(natoms):
        t = types[a % len(types)]
        anc = [int(v) for v in maps["anchor"][t]]
        atoms.append(dict(
            type=t,
            pos=[c * NM_PER_ANGSTROM for c in xyz[3 * a:3 * a + 3]],
            charge=maps["charge"][t],
            dipole=list(maps["dipole"][t]),
            quadrupole=list(maps["quadrupole"][t]),
            octopole=list(maps["octopole"][t]),
            axis_type=int(maps["axes"][t]),
            atom_z=a + anc[0],
            atom_x=(-1 if (x_zero_means_none and anc[1] == 0) else a + anc[1]),
            atom_y=(-1 if anc[2] == 0 else a + anc[2]),
            thole=maps["thole"][t],
            polarity=list(maps["polar"][t]),
            covalent={
                "0": [a + int(d) for d in maps.get("cov12", {}).get(t, [])],
                "1": [a + int(d) for d in maps.get("cov13", {}).get(t, [])],
                "4": [a + int(d) for d in maps.get("polgrp", {}).get(t, [])],
            },
        ))
    return atoms


def parse_charge_square(body):
    pos = [num_list(m.group(1)) for m in re.finditer(r"positions\.push_back\(Vec3\((.*?)\)\)", body)]
    atoms = []
    for m in re.finditer(r"addMultipole\((.*?)\);", body):
        charge = float(m.group(1).split(",")[0])
        atoms.append(dict(type="Q", charge=charge, dipole=[0.0] * 3, quadrupole=[0.0] * 6, octopole=[0.0] * 10,
                          axis_type=AXIS["NoAxisType"], atom_z=0, atom_x=0, atom_y=0, thole=0.0,
                          polarity=[0.0, 0.0, 0.0], covalent={}))
    for a, p in zip(atoms, pos):
        a["pos"] = p
    for m in re.finditer(r"setCovalentMap\((\d+),\s*MPIDForce::(\w+),\s*\{(.*?)\}\)", body):
        atoms[int(m.group(1))]["covalent"][str(COVALENT[m.group(2)])] = [int(v) for v in num_list(m.group(3))]
    return atoms


def parse_dimer_test(name, body):
    t = dict(name=name, **DEFAULTS)
    t["system"] = "waterbox" if "make_waterbox" in body else "methanolbox"
    t["natoms"] = int(re.search(r"numAtoms\s*=\s*(\d+)", body).group(1))
    t["box"] = float(re.search(r"boxEdgeLength\s*=\s*([\d.eE+-]+)\s*\*\s*OpenMM::NmPerAngstrom", body).group(1)) * NM_PER_ANGSTROM
    m = re.search(r"cutoff\s*=\s*([\d.eE+-]+)\s*\*\s*OpenMM::NmPerAngstrom", body)
    t["cutoff"] = float(m.group(1)) * NM_PER_ANGSTROM if m else 1.0
    t["nonbonded_method"] = 1 if "MPIDForce::PME)" in body else 0
    if t["nonbonded_method"] == 1:
        t["ewald_alpha"] = float(re.search(r"const double alpha\s*=\s*([\d.eE+-]+)", body).group(1))
        g = int(re.search(r"const int grid\s*=\s*(\d+)", body).group(1))
        t["grid"] = [g, g, g]
    t["default_thole"] = float(re.search(r"setDefaultTholeWidth\(([\d.eE+-]+)\)", body).group(1))
    t["polarization_type"] = POLTYPE[re.search(r"setPolarizationType\(MPIDForce::(\w+)\)", body).group(1)]
    m = re.search(r"setMutualInducedTargetEpsilon\(([\d.eE+-]+)\)", body)
    if m:
        t["mutual_eps"] = float(m.group(1))
    t["ref_energy"] = float(re.search(r"double refenergy\s*=\s*([\d.eE+-]+);", body).group(1))
    forces = {}
    for m in re.finditer(r"refforces\[\s*(\d+)\]\s*=\s*Vec3\((.*?)\);", body):
        forces[int(m.group(1))] = num_list(m.group(2))
    t["ref_forces"] = [forces[i] for i in range(t["natoms"])]
    t["energy_tol"] = 1e-4
    t["force_tol"] = 1e-4
    return t


def parse_scaling_test(name, body):
    """The 1-4 scaling tests build three systems each (TestReferenceMPIDForce.cpp:1603-1700)."""
    pme = "PME" in name
    out = []
    box = float(re.search(r"boxEdgeLength\s*=\s*([\d.eE+-]+)\s*\*\s*OpenMM::NmPerAngstrom", body).group(1)) * NM_PER_ANGSTROM
    blocks = re.split(r"make_charge_square\(", body)[1:]
    for k, blk in enumerate(blocks):
        t = dict(name="%s[%d]" % (name, k), **DEFAULTS)
        t.update(system="charge_square", natoms=4, box=box, nonbonded_method=1 if pme else 0, cutoff=1.0)
        m = re.search(r"set14ScaleFactor\(([\d.eE+-]+)\)", blk)
        t["scale14"] = float(m.group(1)) if m else 1.0
        if pme:
            t["cutoff"] = float(re.search(r"const double cutoff\s*=\s*([\d.eE+-]+)\s*\*\s*OpenMM::NmPerAngstrom", body).group(1)) * NM_PER_ANGSTROM
            pp = num_list(re.search(r"setPMEParameters\((.*?)\)", blk).group(1).replace("grid", str(
                int(re.search(r"const int grid\s*=\s*(\d+)", body).group(1)))))
            t["ewald_alpha"] = pp[0]
            t["grid"] = [int(v) for v in pp[1:4]]
        m = re.search(r"ASSERT_EQUAL_TOL\(energy,\s*([-\d./ ]+),\s*([\d.eE+-]+)\)", blk)
        expr = m.group(1).strip()
        assert re.fullmatch(r"[-\d./ ]+", expr)
        t["ref_energy"] = float(eval(expr))  # a literal such as -1389.35/2
        t["energy_tol"] = float(m.group(2))
        t["ref_forces"] = None
        out.append(t)
    return out


def main():
    root = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    src = (root / "platforms/reference/tests/TestReferenceMPIDForce.cpp").read_text()
    systems = {
        "charge_square": parse_charge_square(function_body(src, "make_charge_square")),
        "waterbox": parse_box_fixture(function_body(src, "make_waterbox"), 6),
        "methanolbox": parse_box_fixture(function_body(src, "make_methanolbox"), 12),
    }
    main_body = function_body(src, "main") if re.search(r"void\s+main", src) else src[src.index("int main("):]
    order = re.findall(r"\b(test\w+)\(\);", main_body)
    tests = []
    for name in order:
        body = function_body(src, name)
        if name.startswith("test14Scaling"):
            tests.extend(parse_scaling_test(name, body))
        else:
            tests.append(parse_dimer_test(name, body))
    out = dict(source="platforms/reference/tests/TestReferenceMPIDForce.cpp", systems=systems, tests=tests)
    dst = Path(__file__).with_name("reference_tests.json")
    dst.write_text(json.dumps(out, indent=1))
    print("wrote %s: %d tests" % (dst, len(tests)))


if __name__ == "__main__":
    main()
