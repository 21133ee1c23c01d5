"""Make tests/golden/hubbard_example.json from the reference's only shipped input set,
example/Hubb_model/primitive_Cell_ipt/ (Hk.HWR, input.parm, input.solver).

The reference ships no outputs for this example, so the fixture holds its INPUTS: the hopping rows of Hk.HWR
(read_HR's format, src/read_TB_parm.cpp:6-76) and the run settings the hot path reads (k grid, beta,
N_MATSUBARA, N_TAU, U, U', J, N_ELECTRONS, MIXING, DC_TYPE, N_d, MAGNETISM, SOLVER_TYPE).  The GPU test runs
the DMFT loop body on these inputs through the library and through the oracle and compares them.

    python tests/golden/make_hubbard_example.py [path to the example directory]

Run in the build container (the reference tree is not on the GPU machine); the JSON it writes is committed.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT = "/root/reference/example/Hubb_model/primitive_Cell_ipt"


def parse_settings(text):
    """`KEY = value` lines with `//` comments (the reference's input.parm / input.solver syntax)."""
    out = {}
    for ln in text.splitlines():
        ln = ln.split("//", 1)[0].strip()
        m = re.match(r"^([A-Za-z_']+)\s*=\s*(.*)$", ln)
        if m and m.group(2):
            out[m.group(1)] = m.group(2).split()
    return out


def parse_hwr(text):
    """Norbital headers and the `Rx Ry Rz a1 a2 i j Re Im` rows, indices kept 1-based as in the file."""
    norb, rows = [], []
    for ln in text.splitlines():
        m = re.match(r"^\s*Norbital of Atom\s*=\s*(\d+)", ln)
        if m:
            norb.append(int(m.group(1)))
            continue
        p = ln.split()
        if len(p) == 9:
            rows.append([int(x) for x in p[:7]] + [float(p[7]), float(p[8])])
    return norb, rows


def main(src):
    with open(os.path.join(src, "Hk.HWR")) as f:
        norb, rows = parse_hwr(f.read())
    with open(os.path.join(src, "input.parm")) as f:
        parm = parse_settings(f.read())
    with open(os.path.join(src, "input.solver")) as f:
        solver = parse_settings(f.read())
    kx, ky, kz = (int(x) for x in parm["K_POINTS"][:3])
    fixture = {
        "source": "example/Hubb_model/primitive_Cell_ipt (Hk.HWR, input.parm, input.solver)",
        "norbital_of_atom": norb,
        "hwr_rows": rows,
        "k_points": [kx, ky, kz],
        "solver_type": parm["SOLVER_TYPE"][0],
        "mixing": float(parm["MIXING"][0]),
        "n_electrons": float(parm["N_ELECTRONS"][0]),
        "magnetism": int(parm["MAGNETISM"][0]),
        "dc_type": parm["DC_TYPE"][0],
        "n_d": float(parm["N_d"][0]),
        "hartree_orbitals_range": [int(x) for x in parm["HARTREE_ORBITALS_RANGE"][:2]],
        "n_orbitals": int(solver["N_ORBITALS"][0]),
        "U": float(solver["U"][0]),
        "Uprime": float(solver["U'"][0]),
        "J": float(solver["J"][0]),
        "beta": float(solver["BETA"][0]),
        "n_matsubara": int(solver["N_MATSUBARA"][0]),
        "n_tau": int(solver["N_TAU"][0]),
    }
    out = os.path.join(HERE, "hubbard_example.json")
    lines = []
    for key, val in fixture.items():
        if key == "hwr_rows":
            rows_txt = ",\n  ".join(json.dumps(r) for r in val)
            lines.append(' "%s": [\n  %s\n ]' % (key, rows_txt))
        else:
            lines.append(" %s: %s" % (json.dumps(key), json.dumps(val)))
    with open(out, "w") as f:
        f.write("{\n" + ",\n".join(lines) + "\n}\n")
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT)
