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
/root/reference); machines without the checkout never run this.
"""
import importlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from make_localframe_golden import REF, read_prm  # noqa: E402

tio = importlib.import_module("tinker-gpu_gb300.tinkerio")


def read_frames(path):
    """Every frame of a Tinker .arc-style file: (box, names, xyz[f][n][3], types, bonds)."""
    frames = tio.read_xyz(path)
    f0 = frames[0]
    return ([list(f.box[:3]) for f in frames], f0.names, np.array([f.xyz for f in frames]), f0.types.tolist(),
            f0.bonds)


def read_dyn(path):
    """Positions and velocities of a Tinker .dyn restart."""
    x, v, _, _, _ = tio.read_dyn(path)
    return x, v


def read_md_params(path, types):
    """Masses by type, van der Waals records by class and the water valence
    records (bond 34-35, angle 35-34-35, Urey-Bradley 35-34-35)."""
    P = tio.read_prm(path)
    cls = {t: P.atoms[t][0] for t in types}
    o, hyd = cls[36], cls[37]
    glob = {k: float(v[0]) for k, v in P.keywords.items()
            if k in ("bond-cubic", "bond-quartic", "angle-cubic", "angle-quartic", "angle-pentic", "angle-sextic",
                     "urey-cubic", "urey-quartic")}
    return {
        "mass": {str(t): P.atoms[t][3] for t in types},
        "vdw": {str(t): P.vdw[cls[t]] for t in types},
        "bond": list(P.bond[(min(o, hyd), max(o, hyd))]),
        "angle": list(P.angle[(hyd, o, hyd)]),
        "urey": list(P.urey[(hyd, o, hyd)]),
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
