"""Generate tests/golden/extfield.json from the Tinker9 sources.

Known answers of four AMOEBA waters and a Na+ (placed two boxes away along x
and one along -z, so the unwrapped coordinates matter) in a uniform external
field of (150, -300, 450) MV/cm (test/extfield.cpp:15-173):
  test/file/extfield/water4_Na_shifted.{xyz,key}   18.643 A box, PME, 7 A,
                                                   mutual polarization
  test/file/commit_92528f7d/amoebabio18.prm         multipole / polarize, scales
  test/ref/extfield.1.txt  multipole term only      energy, virial, gradient
  test/ref/extfield.2.txt  polarization term only
  test/ref/extfield.3.txt  both
Reads the files as text; run in a checkout that has the reference at
REFERENCE_ROOT (default /root/reference).  Machines without the checkout never run this.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_localframe_golden import REF, read_prm  # noqa: E402
from make_polpair_golden import read_xyz  # noqa: E402

FIELD_MV_CM = [150.0, -300.0, 450.0]  # test/extfield.cpp:11
ELEFIELD = 1439.96455  # MV/cm per e/A^2 (ext/interface/cpp/tinker/detail/units.hh:21)


def read_ref(path):
    """Energy (total or the single component listed), 3x3 virial, gradient."""
    with open(path) as f:
        lines = f.read().splitlines()
    out = {"gradient": []}
    for i, ln in enumerate(lines):
        t = ln.split()
        s = ln.strip()
        if s.startswith("Total Potential Energy"):
            out["energy"] = float(t[-2])
        elif s.startswith(("Atomic Multipoles", "Polarization", "Bond Stretching", "Urey-Bradley")):
            out["energy"] = float(t[-2])
        elif s.startswith("Internal Virial Tensor"):
            rows = [t[-3:], lines[i + 1].split(), lines[i + 2].split()]
            out["virial"] = [[float(v) for v in r] for r in rows]
        elif t and t[0] == "Anlyt":
            out["gradient"].append([float(v) for v in t[2:5]])
    return out


def main():
    base = os.path.join(REF, "test/file/extfield/water4_Na_shifted")
    atoms = read_xyz(base + ".xyz")
    types = sorted({a["type"] for a in atoms})
    scales, mpole, polar = read_prm(os.path.join(REF, "test/file/commit_92528f7d/amoebabio18.prm"), types)
    mass = {}
    with open(os.path.join(REF, "test/file/commit_92528f7d/amoebabio18.prm")) as f:
        for ln in f:
            t = ln.split()
            if len(t) > 2 and t[0] == "atom" and int(t[1]) in types:
                mass[str(int(t[1]))] = float(t[-2])
    kw = {}
    with open(base + ".key") as f:
        for ln in f:
            t = ln.split()
            if t:
                kw[t[0].lower()] = t[1:]
    fixture = {
        "source": "Tinker9 test/extfield.cpp, test/file/extfield/water4_Na_shifted.{xyz,key}, "
        "test/file/commit_92528f7d/amoebabio18.prm, test/ref/extfield.{1,2,3}.txt",
        "atoms": atoms,
        "scales": scales,
        "multipole": mpole,
        "polarize": polar,
        "mass": mass,
        "box": float(kw["a-axis"][0]),
        "ewald_cutoff": float(kw["ewald-cutoff"][0]),
        "polar_eps": float(kw["polar-eps"][0]),
        "field_e_per_a2": [v / ELEFIELD for v in FIELD_MV_CM],
        "eps": {"energy": 1e-4, "gradient": 1e-4, "virial": 1e-3},  # test/extfield.cpp:24-26
        "expected": {
            "mpole": read_ref(os.path.join(REF, "test/ref/extfield.1.txt")),
            "polar": read_ref(os.path.join(REF, "test/ref/extfield.2.txt")),
            "mplar": read_ref(os.path.join(REF, "test/ref/extfield.3.txt")),
        },
    }
    out = os.path.join(HERE, "extfield.json")
    with open(out, "w") as f:
        json.dump(fixture, f, indent=1)
    print("wrote", out, file=sys.stderr)


if __name__ == "__main__":
    main()
