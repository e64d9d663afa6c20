"""Generate tests/golden/local_frame.json from the Tinker9 sources.

Reads, as text, the 22-atom local-frame test case of the reference:
  test/file/local_frame/local_frame.xyz       coordinates, types, bonds
  test/file/commit_6fe8e913/amoeba09.prm       multipole / polarize records
                                               and the scale-factor keywords
  test/localframe.cpp                          known answers (Fortran Tinker)
and writes one JSON fixture.  Run in a checkout that has the reference at
REFERENCE_ROOT (default /root/reference); machines without the checkout never run this.
"""
import json
import os
import re
import sys

REF = os.environ.get("REFERENCE_ROOT", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))


def read_xyz(path):
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[0].split()[0])
    atoms = []
    for ln in lines[1 : 1 + n]:
        t = ln.split()
        atoms.append(
            {
                "index": int(t[0]),
                "name": t[1],
                "xyz": [float(t[2]), float(t[3]), float(t[4])],
                "type": int(t[5]),
                "bonds": [int(v) for v in t[6:]],
            }
        )
    return atoms


SCALE_KEYS = [
    "mpole-12-scale", "mpole-13-scale", "mpole-14-scale", "mpole-15-scale",
    "polar-12-scale", "polar-13-scale", "polar-14-scale", "polar-15-scale",
    "polar-12-intra", "polar-13-intra", "polar-14-intra", "polar-15-intra",
    "direct-11-scale", "direct-12-scale", "direct-13-scale", "direct-14-scale",
    "mutual-11-scale", "mutual-12-scale", "mutual-13-scale", "mutual-14-scale",
]


def read_prm(path, types):
    with open(path) as f:
        lines = f.read().splitlines()
    scales, mpole, polar = {}, {}, {}
    i = 0
    while i < len(lines):
        t = lines[i].split()
        if not t:
            i += 1
            continue
        key = t[0].lower()
        if key in SCALE_KEYS:
            scales[key] = float(t[1])
        elif key == "multipole":
            ids = [int(v) for v in t[1:-1]]
            vals = [float(t[-1])]
            for j in range(1, 5):
                vals += [float(v) for v in lines[i + j].split()]
            if ids[0] in types:
                while len(ids) < 4:
                    ids.append(0)
                mpole.setdefault(str(ids[0]), []).append({"axes": ids[1:4], "values": vals})
            i += 5
            continue
        elif key == "polarize":
            ty = int(t[1])
            if ty in types:
                polar[str(ty)] = {
                    "alpha": float(t[2]),
                    "thole": float(t[3]),
                    "group": [int(v) for v in t[4:]],
                }
        i += 1
    return scales, mpole, polar


def parse_sections(src):
    """Split test/localframe.cpp into {test_case: {section: {name: value}}}."""
    out = {}
    cases = re.split(r'TEST_CASE\("', src)[1:]
    for c in cases:
        cname = c.split('"', 1)[0]
        parts = re.split(r'SECTION\("', c)
        secs = {"_case": parts[0]}
        for p in parts[1:]:
            secs[p.split('"', 1)[0]] = p
        out[cname] = {}
        for sname, body in secs.items():
            vals = {}
            for m in re.finditer(r"const double (\w+)\[\]\[3\] = \{(.*?)\};", body, re.S):
                nums = [float(v) for v in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", m.group(2))]
                vals[m.group(1)] = [nums[j : j + 3] for j in range(0, len(nums), 3)]
            for m in re.finditer(r"const double (\w+) = (-?[\d.]+(?:e-?\d+)?);", body):
                vals[m.group(1)] = float(m.group(2))
            for m in re.finditer(r"const int (\w+) = (\d+);", body):
                vals[m.group(1)] = int(m.group(2))
            out[cname][sname] = vals
    return out


def main():
    atoms = read_xyz(os.path.join(REF, "test/file/local_frame/local_frame.xyz"))
    types = sorted({a["type"] for a in atoms})
    scales, mpole, polar = read_prm(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), types)
    with open(os.path.join(REF, "test/localframe.cpp")) as f:
        sections = parse_sections(f.read())
    fixture = {
        "source": "Tinker9 test/localframe.cpp, test/file/local_frame/local_frame.xyz, "
        "test/file/commit_6fe8e913/amoeba09.prm",
        "atoms": atoms,
        "scales": scales,
        "multipole": mpole,
        "polarize": polar,
        "ewald": {"cutoff": 7.0, "box": 20.0, "list_buffer": 0.1},
        "usolve_cutoff": 0.01,
        "expected": sections,
    }
    out = os.path.join(HERE, "local_frame.json")
    with open(out, "w") as f:
        json.dump(fixture, f, indent=1)
    print("wrote", out, file=sys.stderr)


if __name__ == "__main__":
    main()
