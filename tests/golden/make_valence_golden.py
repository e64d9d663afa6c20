"""Generate tests/golden/valence.json from the Tinker9 sources.

Known answers of the valence terms the AMOEBA water MD step uses:
  bond   test/bond.cpp (Bond-Trpcage): test/file/trpcage/trpcage.xyz,
         test/file/commit_6fe8e913/amoebapro13.prm, test/ref/bond.txt
         (304 atoms, 310 bonds, anharmonic bond-cubic / bond-quartic)
  urey   test/urey.cpp (Urey-Ten-Water): test/file/water10/h2o10.xyz,
         test/file/commit_6fe8e913/water03.prm, test/ref/urey.txt
Bond and Urey-Bradley parameters are resolved here from the atom classes
(the parameter files' atom records).  Reads the files as text; run in a
checkout that has the reference at REFERENCE_ROOT (default /root/reference).
Machines without the checkout never run this.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_extfield_golden import read_ref  # noqa: E402
from make_localframe_golden import REF  # noqa: E402
from make_polpair_golden import read_xyz  # noqa: E402


def read_params(path):
    """atom type -> class, bond / ureybrad records by class, global terms."""
    cls, bond, urey, glob = {}, {}, {}, {}
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if not t:
                continue
            key = t[0].lower()
            if key == "atom":
                cls[int(t[1])] = int(t[2])
            elif key == "bond":
                a, b = int(t[1]), int(t[2])
                bond[(min(a, b), max(a, b))] = (float(t[3]), float(t[4]))
            elif key == "ureybrad":
                a, m, b = int(t[1]), int(t[2]), int(t[3])
                urey[(min(a, b), m, max(a, b))] = (float(t[4]), float(t[5]))
            elif key in ("bond-cubic", "bond-quartic", "urey-cubic", "urey-quartic"):
                glob[key] = float(t[1])
    return cls, bond, urey, glob


def bonds_of(atoms):
    return sorted({(min(a["index"], b) - 1, max(a["index"], b) - 1) for a in atoms for b in a["bonds"]})


def main():
    out = {"source": "Tinker9 test/bond.cpp, test/urey.cpp, test/file/trpcage/trpcage.xyz, "
           "test/file/water10/h2o10.xyz, test/file/commit_6fe8e913/{amoebapro13,water03}.prm, "
           "test/ref/{bond,urey}.txt"}
    atoms = read_xyz(os.path.join(REF, "test/file/trpcage/trpcage.xyz"))
    cls, bond, _, glob = read_params(os.path.join(REF, "test/file/commit_6fe8e913/amoebapro13.prm"))
    bl = []
    for i, k in bonds_of(atoms):
        ci, ck = cls[atoms[i]["type"]], cls[atoms[k]["type"]]
        kb, r0 = bond[(min(ci, ck), max(ci, ck))]
        bl.append([i, k, kb, r0])
    out["bond"] = {"xyz": [a["xyz"] for a in atoms], "bonds": bl, "cubic": glob.get("bond-cubic", 0.0),
                   "quartic": glob.get("bond-quartic", 0.0), "eps": {"energy": 1e-4, "gradient": 1e-4, "virial": 1e-3},
                   "expected": read_ref(os.path.join(REF, "test/ref/bond.txt"))}
    atoms = read_xyz(os.path.join(REF, "test/file/water10/h2o10.xyz"))
    cls, _, urey, glob = read_params(os.path.join(REF, "test/file/commit_6fe8e913/water03.prm"))
    adj = {a["index"] - 1: [b - 1 for b in a["bonds"]] for a in atoms}
    ul = []
    for m, nb in sorted(adj.items()):
        for x in range(len(nb)):
            for y in range(x + 1, len(nb)):
                a, b = nb[x], nb[y]
                ca, cm, cb = cls[atoms[a]["type"]], cls[atoms[m]["type"]], cls[atoms[b]["type"]]
                key = (min(ca, cb), cm, max(ca, cb))
                if key in urey:
                    ul.append([a, m, b, urey[key][0], urey[key][1]])
    out["urey"] = {"xyz": [a["xyz"] for a in atoms], "ureys": ul, "cubic": glob.get("urey-cubic", 0.0),
                   "quartic": glob.get("urey-quartic", 0.0), "eps": {"energy": 1e-4, "gradient": 1e-4, "virial": 1e-3},
                   "expected": read_ref(os.path.join(REF, "test/ref/urey.txt"))}
    path = os.path.join(HERE, "valence.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, file=sys.stderr)


if __name__ == "__main__":
    main()
