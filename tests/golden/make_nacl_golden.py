"""Generate tests/golden/nacl.json from the Tinker9 sources.

Two-ion known answers of the multipole energy, gradient and virial:
  NaCl-2  test/nacl.cpp:211-239   non-Ewald, periodic 18.643 A box, 5 A cutoff,
          test/file/nacl/nacl1.xyz + nacl.key (amoeba09 charges)
  NaCl-3  test/nacl.cpp:242-301   PME (40^3 grid, 7 A cutoff, 20 A box),
          test/file/nacl/nacl4.xyz + nacl4.key, whose own multipole records
          (z-only frames with dipoles and quadrupoles) come before the
          parameter file's and the two ions are bonded (1-2 scale 0)
Reads the files as text; run in a checkout that has the reference at
REFERENCE_ROOT (default /root/reference).  Machines without the checkout never run this.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_localframe_golden import REF, read_prm, read_xyz  # noqa: E402


def read_key(path):
    """Keywords (lower-case first word -> rest) and the key file's own
    multipole records in parameter-file form."""
    with open(path) as f:
        lines = f.read().splitlines()
    kw, mpole = {}, {}
    i = 0
    while i < len(lines):
        t = lines[i].split()
        if not t or t[0].startswith("#"):
            i += 1
            continue
        key = t[0].lower()
        if key == "multipole":
            ids = [int(v) for v in t[1:-1]]
            vals = [float(t[-1])]
            for j in range(1, 5):
                vals += [float(v) for v in lines[i + j].split()]
            while len(ids) < 4:
                ids.append(0)
            mpole.setdefault(str(ids[0]), []).append({"axes": ids[1:4], "values": vals})
            i += 5
            continue
        kw[key] = t[1:]
        i += 1
    return kw, mpole


def parse_case(src, case):
    """ref_eng / ref_grad / ref_v of one TEST_CASE, comments stripped."""
    body = src.split('TEST_CASE("%s"' % case, 1)[1].split("TEST_CASE(", 1)[0]
    body = "\n".join(ln.split("//", 1)[0] for ln in body.splitlines())
    out = {}
    for m in re.finditer(r"const double (\w+)\[\]\[3\] = \{(.*?)\};", body, re.S):
        nums = [float(v) for v in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", m.group(2))]
        out[m.group(1)] = [nums[j : j + 3] for j in range(0, len(nums), 3)]
    for m in re.finditer(r"const double (\w+) = (-?[\d.]+(?:e-?\d+)?);", body):
        out[m.group(1)] = float(m.group(2))
    return out


def parse_sections(src, case_name):
    """{section title: {ref_eng, ref_grad, ref_v, eps}} of one TEST_CASE."""
    body = src.split('TEST_CASE("%s"' % case_name, 1)[1].split("TEST_CASE(", 1)[0]
    body = "\n".join(ln.split("//", 1)[0] for ln in body.splitlines())
    eps = re.search(r"const double eps = (-?[\d.]+(?:e-?\d+)?);", body)
    out = {}
    for part in body.split('SECTION("')[1:]:
        title = part.split('"', 1)[0].strip()
        vals = {"eps": float(eps.group(1))}
        for m in re.finditer(r"const double (\w+)\[\]\[3\] = \{(.*?)\};", part, re.S):
            nums = [float(v) for v in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", m.group(2))]
            vals[m.group(1)] = [nums[j : j + 3] for j in range(0, len(nums), 3)]
        for m in re.finditer(r"const double (\w+) = (-?[\d.]+(?:e-?\d+)?);", part):
            vals[m.group(1)] = float(m.group(2))
        x = re.search(r'test/file/nacl/(nacl\d\.xyz)', part)
        vals["xyz_file"] = x.group(1) if x else None
        vals["extra_keys"] = re.findall(r'key\d \+= "([^"]*)\\n"', part)
        out[title] = vals
    return out


def read_vdw(path, types):
    """vdw records (radius, epsilon[, reduction]) of the given types/classes."""
    out = {}
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if len(t) >= 4 and t[0] == "vdw" and int(t[1]) in types:
                out[t[1]] = [float(v) for v in t[2:]]
    return out


def case(xyz_file, key_file, src, name, ewald):
    atoms = read_xyz(os.path.join(REF, "test/file/nacl", xyz_file))
    types = sorted({a["type"] for a in atoms})
    scales, prm_mpole, polar = read_prm(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), types)
    kw, key_mpole = read_key(os.path.join(REF, "test/file/nacl", key_file))
    mpole = {t: key_mpole.get(t, []) + prm_mpole.get(t, []) for t in map(str, types)}
    box = float(kw["a-axis"][0])
    out = {
        "atoms": atoms,
        "scales": scales,
        "multipole": mpole,
        "polarize": polar,
        "box": box,
        "ewald": ewald,
        "cutoff": float(kw["ewald-cutoff"][0]) if ewald else float(kw["mpole-cutoff"][0]),
        "expected": parse_case(src, name),
    }
    if ewald:
        out["nfft"] = [int(v) for v in kw["pme-grid"][:3]]
    return out


def main():
    with open(os.path.join(REF, "test/nacl.cpp")) as f:
        src = f.read()
    kw, _ = read_key(os.path.join(REF, "test/file/nacl/nacl.key"))
    secs = parse_sections(src, "NaCl-1")
    ehal = {}
    for title, v in secs.items():
        if v["xyz_file"] is None or v["extra_keys"]:
            continue  # the long-range correction sections (vdw-correction) are not restated
        ehal[title] = {"atoms": read_xyz(os.path.join(REF, "test/file/nacl", v["xyz_file"])),
                       "ref_eng": v["ref_eng"], "ref_grad": v["ref_grad"], "ref_v": v["ref_v"], "eps": v["eps"]}
    fixture = {
        "source": "Tinker9 test/nacl.cpp, test/file/nacl/{nacl1.xyz,nacl2.xyz,nacl3.xyz,nacl4.xyz,nacl.key,"
        "nacl4.key}, test/file/commit_6fe8e913/amoeba09.prm",
        "NaCl-1": {
            "box": float(kw["a-axis"][0]),
            "vdw_cutoff": float(kw["vdw-cutoff"][0]),
            "vdw": read_vdw(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), {7, 15}),
            "cases": ehal,
        },
        "NaCl-2": case("nacl1.xyz", "nacl.key", src, "NaCl-2", False),
        "NaCl-3": case("nacl4.xyz", "nacl4.key", src, "NaCl-3", True),
    }
    out = os.path.join(HERE, "nacl.json")
    with open(out, "w") as f:
        json.dump(fixture, f, indent=1)
    print("wrote", out, file=sys.stderr)


if __name__ == "__main__":
    main()
