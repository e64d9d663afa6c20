"""Tinker file formats (tinker-gpu_gb300/tinkerio.py): coordinate, dipole and
restart round trips, the layouts of the reference's files, and a System
assembled from .xyz / .key / .prm files equal to the one the TinkerNIST
fixture builds directly."""
import importlib
import os

import numpy as np
import pytest

import tn_fixture as T

tg = importlib.import_module("tinker-gpu_gb300")
tio = importlib.import_module("tinker-gpu_gb300.tinkerio")


def _frame(s, title="water box"):
    names = ["O" if t == tg.systems.WATER_O else "H" for t in s.types]
    box = None if s.box is None else tuple(s.box) + (90.0, 90.0, 90.0)
    return tio.Frame(title, names, s.xyz.copy(), s.types.copy(), tg.systems.lattice_bonds(s), box)


def test_xyz_round_trip_and_layout(tmp_path):
    s = tg.systems.make_config("water648")
    fr = _frame(s)
    p = tmp_path / "w.xyz"
    tio.write_xyz(p, fr)
    lines = p.read_text().splitlines()
    # "%6d  %s" title, " " + six "%12.6f" box values, "%6d  %-3s" + 3 x "%12.6f" + "%6d" + bonds
    assert lines[0] == f"{s.n:6d}  water box"
    assert len(lines[1]) == 1 + 6 * 12 and lines[1].startswith(f" {s.box[0]:12.6f}")
    assert lines[2].startswith("     1  O  ") and len(lines[2]) == 6 + 2 + 3 + 36 + 6 + 12
    back = tio.read_xyz(p)
    assert len(back) == 1
    b = back[0]
    assert b.names == fr.names and np.array_equal(b.types, fr.types) and b.bonds == sorted(fr.bonds)
    assert np.abs(b.xyz - fr.xyz).max() <= 5e-7 and b.box == pytest.approx(fr.box)


def test_arc_frames_and_dipole_files(tmp_path):
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    fr = _frame(s)
    arc = tmp_path / "w.arc"
    for t in range(3):
        fr.xyz = tr.frame(t)
        tio.write_xyz(arc, fr, append=t > 0)
    frames = tio.read_xyz(arc)
    assert len(frames) == 3
    for t in range(3):
        assert np.abs(frames[t].xyz - tr.frame(t)).max() <= 5e-7
    # .uind: the same layout, the dipole (Debye) in place of the position
    u = np.random.default_rng(1).normal(scale=0.5, size=(s.n, 3))
    tio.write_dipoles(tmp_path / "w.uind", fr, u)
    d = tio.read_xyz(tmp_path / "w.uind")[0]
    assert np.abs(d.xyz - u).max() <= 5e-7 and d.names == fr.names


def test_dyn_round_trip_and_number_format(tmp_path):
    # the layout of the reference's restart files (test/file/tinkernist/water30.dyn)
    assert tio._fortran_d(13.74607312280601) == "0.1374607312280601D+02"
    assert tio._fortran_d(-6.669383547023202) == "-0.6669383547023202D+01"
    assert tio._fortran_d(30.0) == "0.3000000000000000D+02"
    assert tio._fortran_d(0.0) == "0.0000000000000000D+00"
    assert tio._fortran_d(0.00123) == "0.1230000000000000D-02"
    rng = np.random.default_rng(2)
    x, v, a = (rng.normal(scale=sc, size=(20, 3)) for sc in (10.0, 3.0, 100.0))
    p = tmp_path / "w.dyn"
    tio.write_dyn(p, "test box", x, v, a, box=(30.0, 30.0, 30.0))
    text = p.read_text().splitlines()
    assert text[0] == " Number of Atoms and Title :" and text[2] == " Periodic Box Dimensions :"
    assert text[5] == " Current Atomic Positions :" and len(text[6]) == 78
    x2, v2, a2, alt, box = tio.read_dyn(p)
    for u, w in ((x, x2), (v, v2), (a, a2)):
        assert np.allclose(u, w, rtol=1e-15, atol=0)
    assert np.array_equal(alt, np.zeros_like(x)) and box == (30.0, 30.0, 30.0, 90.0, 90.0, 90.0)


@pytest.mark.parametrize("edge, n", [(30.0, 36), (18.643, 24), (49.31, 60), (98.62, 120), (61.7, 75)])
def test_default_pme_grid(edge, n):
    assert tio.pme_grid_size(edge) == n


def _tinkernist_files(d):
    """The TinkerNIST run written as Tinker files from the committed fixture
    (the parameter subset in prm syntax; atom class = atom type)."""
    s, mass, v0, fx = T.md_system()
    m = fx["meta"]
    md = m["md"]
    label = {36: ("O", 8, 2), 37: ("H", 1, 1), 7: ("Na+", 11, 0), 15: ("Cl-", 17, 0)}
    names = [label[t][0] for t in fx["types"]]
    box = tuple(m["box"]) + (90.0, 90.0, 90.0)
    fr = tio.Frame("AMOEBA Water Box", names, np.array(fx["dyn_x"]), np.array(fx["types"]), fx["bonds"], box)
    tio.write_xyz(os.path.join(d, "nist.xyz"), fr)
    with open(os.path.join(d, "nist.key"), "w") as f:
        f.write("parameters  nist\n# comment line\nverbose\n")
        f.write(f"a-axis {m['box'][0]}\nneighbor-list\nvdw-cutoff {m['vdw_cutoff']}\newald\n")
        f.write(f"ewald-cutoff {m['ewald_cutoff']}\npme-grid {T.NFFT} {T.NFFT} {T.NFFT}\npolar-eps {m['polar_eps']}\n")
        f.write("polar-predict\n")  # as test/file/water30/water30.key
    lines = []
    for k, v in m["scales"].items():
        lines.append(f"{k:<24s}{v}")
    for k, v in {"vdw-12-scale": 0.0, "vdw-13-scale": 0.0, "vdw-14-scale": 1.0}.items():
        lines.append(f"{k:<24s}{v}")
    for k, v in md["globals"].items():
        lines.append(f"{k:<24s}{v}")
    for t in sorted(int(k) for k in md["mass"]):
        nm, z, val = label[t]
        lines.append(f'atom {t} {t} {nm} "{nm} of the test" {z} {md["mass"][str(t)]} {val}')
        vr = md["vdw"][str(t)]
        lines.append("vdw " + " ".join(str(x) for x in [t] + list(vr)))
    lines.append(f"bond 36 37 {md['bond'][0]} {md['bond'][1]}")
    lines.append(f"angle 37 36 37 {md['angle'][0]} {md['angle'][1]}")
    lines.append(f"ureybrad 37 36 37 {md['urey'][0]} {md['urey'][1]}")
    for t, recs in m["multipole"].items():
        for r in recs:
            ax = [a for a in r["axes"] if a != 0] if r["axes"][2] == 0 else r["axes"]
            v = r["values"]
            lines.append(f"multipole {t} " + " ".join(str(a) for a in ax) + f" {v[0]}")
            lines.append(" ".join(str(x) for x in v[1:4]))
            lines.append(str(v[4]))
            lines.append(" ".join(str(x) for x in v[5:7]))
            lines.append(" ".join(str(x) for x in v[7:10]))
    for t, p in m["polarize"].items():
        lines.append(f"polarize {t} {p['alpha']} {p['thole']} " + " ".join(str(g) for g in p["group"]))
    with open(os.path.join(d, "nist.prm"), "w") as f:
        f.write("\n".join(lines) + "\n")
    return s, mass


def test_system_from_tinker_files(tmp_path):
    ref, mass = _tinkernist_files(str(tmp_path))
    s = tio.system_from_tinker(os.path.join(tmp_path, "nist.xyz"))
    assert np.allclose(s.xyz, ref.xyz, atol=5e-7) and np.array_equal(s.types, ref.types)
    assert np.array_equal(s.frames, ref.frames) and np.allclose(s.pole, ref.pole)
    assert np.allclose(s.polarity, ref.polarity) and np.allclose(s.thole, ref.thole)
    assert np.array_equal(s.excl_ik, ref.excl_ik) and np.allclose(s.excl_scale, ref.excl_scale)
    assert np.allclose(s.box, ref.box)
    for k in ("use_ewald", "nfft", "ewald_cutoff", "bsorder"):
        assert s.settings[k] == ref.settings[k], k
    assert s.settings["poleps"] == 1e-5  # the key's polar-eps
    assert s.settings["predictor"] == 1  # polar-predict without a modifier: ASPC
    assert s.settings["aewald"] == pytest.approx(ref.settings["aewald"], rel=1e-12)
    for k in ("vtype", "radmin", "epsilon", "red", "parent", "scaled_ik", "scaled_v"):
        assert np.allclose(np.asarray(getattr(s.vdw, k)), np.asarray(getattr(ref.vdw, k))), k
    assert s.vdw.off == ref.vdw.off and s.vdw.taper == pytest.approx(ref.vdw.taper)
    for k in ("bonds", "angles", "ureys"):
        a = np.asarray(getattr(s.valence, k))
        b = np.asarray(getattr(ref.valence, k))
        assert a.shape == b.shape and np.allclose(a[np.lexsort(a.T[::-1])], b[np.lexsort(b.T[::-1])]), k
    assert s.valence.bond_cubic == ref.valence.bond_cubic and s.valence.angle_terms == ref.valence.angle_terms
    P = tio.read_prm(os.path.join(tmp_path, "nist.prm"))
    assert np.allclose(tio.masses(s.types, P), mass)


def test_predictor_keyword():
    """POLAR-PREDICT as the reference maps its modifier (src/amoeba/epolar.cpp:426-444):
    ASPC 1, GEAR 2, absent 0; no modifier ASPC; LSQR has no GPU path."""
    assert tio.predictor_from_keys({}) == 0
    assert tio.predictor_from_keys({"polar-predict": []}) == 1
    assert tio.predictor_from_keys({"polar-predict": ["aspc"]}) == 1
    assert tio.predictor_from_keys({"polar-predict": ["GEAR"]}) == 2
    with pytest.raises(ValueError):
        tio.predictor_from_keys({"polar-predict": ["LSQR"]})
