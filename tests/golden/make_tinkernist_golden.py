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


def fixed6(a):
    return np.rint(np.asarray(a) * 1e6).astype(np.int64)


def main():
    boxes, names, xyz, types, bonds = read_frames(os.path.join(REF, "test/ref/tinkernist.arc"))
    _, _, uind, _, _ = read_frames(os.path.join(REF, "test/ref/tinkernist.uind"))
    _, _, udir, _, _ = read_frames(os.path.join(REF, "test/ref/tinkernist.udir"))
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
    )
    print("wrote", out, os.path.getsize(out), "bytes", file=sys.stderr)


if __name__ == "__main__":
    main()
