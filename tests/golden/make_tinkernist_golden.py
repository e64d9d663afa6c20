"""Generate tests/golden/tinkernist.npz from the Tinker9 sources.

Reads, as text, the 2,684-atom AMOEBA water box with four Na+/Cl- pairs
(30 A cube) of the reference's TinkerNIST test:
  test/ref/tinkernist.arc                     coordinates after MD steps 1 and 2
  test/ref/tinkernist.uind, .udir             induced and direct dipoles (Debye)
                                              at those coordinates
  test/file/tinkernist/water30.key            ewald, ewald-cutoff 7, polar-eps 1e-5
  test/file/commit_6fe8e913/amoeba09.prm       multipole / polarize records, scales
The reference test (test/tinkernist.cpp:195-365, TinkerNIST-SAVE1) compares
the first and last two atoms of each frame at 0.001; the fixture keeps every
atom.  Coordinates and dipoles are stored as the files' six-decimal integers.
Run in a checkout that has the reference at REFERENCE_ROOT (default
/root/reference); the GPU machine never runs this.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_localframe_golden import REF, read_prm  # noqa: E402


def read_frames(path):
    """Every frame of a Tinker .arc-style file: (box, names, xyz[f][n][3], types, bonds)."""
    with open(path) as f:
        lines = f.read().splitlines()
    frames, names, types, bonds, boxes = [], None, None, None, []
    i = 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i].split()[0])
        boxes.append([float(v) for v in lines[i + 1].split()[:3]])
        rows = [ln.split() for ln in lines[i + 2 : i + 2 + n]]
        frames.append([[float(t[2]), float(t[3]), float(t[4])] for t in rows])
        if names is None:
            names = [t[1] for t in rows]
            types = [int(t[5]) for t in rows]
            bonds = sorted({(min(int(t[0]), int(b)) - 1, max(int(t[0]), int(b)) - 1) for t in rows for b in t[6:]})
        i += 2 + n
    return boxes, names, np.array(frames), types, bonds


def read_dyn(path):
    """Positions and velocities of a Tinker .dyn restart (Fortran D exponents)."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[1].split()[0])
    def block(title):
        i = next(j for j, ln in enumerate(lines) if ln.strip().startswith(title)) + 1
        return np.array([[float(v.replace("D", "E")) for v in ln.split()] for ln in lines[i : i + n]])
    return block("Current Atomic Positions"), block("Current Atomic Velocities")


def read_md_params(path, types):
    """Masses by type, van der Waals records by class and the water valence
    records (bond 34-35, angle 35-34-35, Urey-Bradley 35-34-35)."""
    mass, cls, vdw, bond, angle, urey, glob = {}, {}, {}, {}, {}, {}, {}
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if not t:
                continue
            k = t[0].lower()
            if k == "atom" and int(t[1]) in types:
                cls[int(t[1])] = int(t[2])
                mass[int(t[1])] = float(t[-2])
            elif k == "vdw":
                vdw[int(t[1])] = [float(v) for v in t[2:]]
            elif k == "bond":
                bond[(int(t[1]), int(t[2]))] = [float(t[3]), float(t[4])]
            elif k == "angle":
                angle[(int(t[1]), int(t[2]), int(t[3]))] = [float(t[4]), float(t[5])]
            elif k == "ureybrad":
                urey[(int(t[1]), int(t[2]), int(t[3]))] = [float(t[4]), float(t[5])]
            elif k in ("bond-cubic", "bond-quartic", "angle-cubic", "angle-quartic", "angle-pentic", "angle-sextic",
                       "urey-cubic", "urey-quartic"):
                glob[k] = float(t[1])
    o, hyd = cls[36], cls[37]
    return {
        "mass": {str(t): mass[t] for t in types},
        "vdw": {str(t): vdw[cls[t]] for t in types},
        "bond": bond[(min(o, hyd), max(o, hyd))],
        "angle": angle[(hyd, o, hyd)],
        "urey": urey[(hyd, o, hyd)],
        "globals": glob,
    }


def fixed6(a):
    return np.rint(np.asarray(a) * 1e6).astype(np.int64)


def main():
    boxes, names, xyz, types, bonds = read_frames(os.path.join(REF, "test/ref/tinkernist.arc"))
    _, _, uind, _, _ = read_frames(os.path.join(REF, "test/ref/tinkernist.uind"))
    _, _, udir, _, _ = read_frames(os.path.join(REF, "test/ref/tinkernist.udir"))
    _, _, vel, _, _ = read_frames(os.path.join(REF, "test/ref/tinkernist.vel"))
    x0, v0 = read_dyn(os.path.join(REF, "test/file/tinkernist/water30.dyn"))
    md = read_md_params(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), sorted(set(types)))
    assert xyz.shape == uind.shape == udir.shape and xyz.shape[0] == 2
    scales, mpole, polar = read_prm(os.path.join(REF, "test/file/commit_6fe8e913/amoeba09.prm"), sorted(set(types)))
    meta = {
        "source": "Tinker9 test/tinkernist.cpp (TinkerNIST-SAVE1), test/ref/tinkernist.{arc,uind,udir}, "
        "test/file/tinkernist/water30.key, test/file/commit_6fe8e913/amoeba09.prm",
        "box": boxes[0],
        "ewald_cutoff": 7.0,
        "polar_eps": 1e-5,
        "reference_eps": 0.001,
        "scales": scales,
        "multipole": mpole,
        "polarize": polar,
        "md": md,
        "vdw_cutoff": 12.0,  # water30.key
        "dt_ps": 0.001,  # test/tinkernist.cpp:37 (NVE velocity Verlet)
        "md_eps": {"xyz": 0.001, "vel": 0.002},  # test/tinkernist.cpp:232-233
    }
    out = os.path.join(HERE, "tinkernist.npz")
    np.savez_compressed(
        out,
        meta=np.array(json.dumps(meta)),
        types=np.array(types, dtype=np.int32),
        bonds=np.array(bonds, dtype=np.int32),
        xyz_e6=fixed6(xyz),
        uind_e6=fixed6(uind),
        udir_e6=fixed6(udir),
        vel_e6=fixed6(vel),
        dyn_x=x0,
        dyn_v=v0,
    )
    print("wrote", out, os.path.getsize(out), "bytes", file=sys.stderr)


if __name__ == "__main__":
    main()
