"""Generate tests/golden/polpair.json from the Tinker9 sources.

Known answers of the Na+/Cl- pair with a POLPAIR Thole coefficient
(test/polpair.cpp: PolPair-Ewald, PolPair-NonEwald):
  test/file/polpair/nacl.xyz, nacl.key      20 A box, cutoff 7, polpair 7 15 0.05
  test/file/commit_6fe8e913/amoeba09.prm     multipole / polarize records, scales
  test/ref/polpair.1.txt (Ewald), .2.txt     total energy (multipole +
                                             polarization), virial, gradient
Reads the files as text; run in a checkout that has the reference at
REFERENCE_ROOT (default /root/reference).  Machines without the checkout never run this.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_localframe_golden import REF, read_prm  # noqa: E402


def read_xyz(path):
    """Tinker .xyz, with or without a box line after the title."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    first = 2 if not lines[1].split()[0].isdigit() else 1
    atoms = []
    for ln in lines[first : first + n]:
        t = ln.split()
        atoms.append({"index": int(t[0]), "name": t[1], "xyz": [float(v) for v in t[2:5]], "type": int(t[5]),
                      "bonds": [int(v) for v in t[6:]]})
    return atoms


def read_ref(path):
    """Total energy, 3x3 virial and per-atom gradient of a Tinker analyze listing."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = {"gradient": []}
    for i, ln in enumerate(lines):
        t = ln.split()
        if ln.strip().startswith("Total Potential Energy"):
            out["energy"] = float(t[-2])
        elif ln.strip().startswith("Internal Virial Tensor"):
            rows = [t[-3:], lines[i + 1].split(), lines[i + 2].split()]
            out["virial"] = [[float(v) for v in r] for r in rows]
        elif t and t[0] == "Anlyt":
            out["gradient"].append([float(v) for v in t[2:5]])
    return out


def main():
    atoms = read_xyz(os.path.join(REF, "test/file/polpair/nacl.xyz"))
    types = sorted({a["type"] for a in atoms})
    scales, mpole, polar = read_prm(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), types)
    kw, pairs = {}, []
    with open(os.path.join(REF, "test/file/polpair/nacl.key")) as f:
        for ln in f:
            t = ln.split()
            if not t:
                continue
            if t[0].lower() == "polpair":
                pairs.append([int(t[1]), int(t[2]), float(t[3])])
            else:
                kw[t[0].lower()] = t[1:]
    fixture = {
        "source": "Tinker9 test/polpair.cpp, test/file/polpair/{nacl.xyz,nacl.key}, "
        "test/ref/polpair.{1,2}.txt, test/file/commit_6fe8e913/amoeba09.prm",
        "atoms": atoms,
        "scales": scales,
        "multipole": mpole,
        "polarize": polar,
        "box": float(kw["a-axis"][0]),
        "cutoff": float(kw["cutoff"][0]),
        "polpair": pairs,
        "eps": {"energy": 1e-4, "gradient": 1e-4, "virial": 1e-3},  # test/polpair.cpp:20-22
        "expected": {
            "ewald": read_ref(os.path.join(REF, "test/ref/polpair.1.txt")),
            "nonewald": read_ref(os.path.join(REF, "test/ref/polpair.2.txt")),
        },
    }
    out = os.path.join(HERE, "polpair.json")
    with open(out, "w") as f:
        json.dump(fixture, f, indent=1)
    print("wrote", out, file=sys.stderr)


if __name__ == "__main__":
    main()
