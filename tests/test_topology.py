"""Host-side set-up: frames, multipole units, scale table."""
import numpy as np

import lf_fixture as L


def test_water_scales_and_frames(tg):
    s = tg.systems.make_config("water648")
    assert s.n == 648
    nmol = 216
    # O-H1, O-H2, H1-H2 per molecule, m = d = p = 0, u = 1
    assert len(s.excl_ik) == 3 * nmol
    assert np.allclose(s.excl_scale[:, :3], 0) and np.allclose(s.excl_scale[:, 3], 1)
    assert (s.frames[0::3, 3] == tg.topology.LF_BISECTOR).all()
    assert (s.frames[1::3, 3] == tg.topology.LF_Z_THEN_X).all()
    # dipoles in e*A: 0.14279 bohr -> 0.0755619 A
    assert abs(s.pole[0, 3] - 0.14279 * tg.units.BOHR) < 1e-12
    assert abs(s.pole[0, 4] - 0.37928 * tg.units.BOHR ** 2 / 3) < 1e-12
    assert np.allclose(s.pdamp, s.polarity ** (1 / 6))


def test_water_geometry(tg):
    s = tg.systems.make_config("water648")
    o, h1, h2 = s.xyz[0], s.xyz[1], s.xyz[2]
    assert abs(np.linalg.norm(h1 - o) - 0.9572) < 1e-12
    c = np.dot(h1 - o, h2 - o) / 0.9572 ** 2
    assert abs(np.degrees(np.arccos(c)) - 104.52) < 1e-9


def test_localframe_topology():
    s, fx = L.system(0)
    # acetonitrile N (9) to methyl H (12..14) are 1-4 inside one group: p-intra 0.5, m 0.4, d 0
    ik = [tuple(r) for r in s.excl_ik]
    row = s.excl_scale[ik.index((8, 11))]
    assert np.allclose(row, [0.4, 0.0, 0.5, 1.0])
    # NH3 frames: N 3-Fold, H Z-Bisect
    assert s.frames[14, 3] == 5 and s.frames[15, 3] == 4


def test_nacl_config(tg):
    s = tg.systems.make_config("nacl23142")
    assert s.n == 23142
    assert (s.types == tg.systems.NA_ION).sum() == 21 and (s.types == tg.systems.CL_ION).sum() == 21


def test_trajectory_is_smooth(tg):
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a, b = tr.frame(0), tr.frame(1)
    d = np.linalg.norm(a - b, axis=1)
    assert d.max() < 0.05
    # rigid geometry preserved
    assert abs(np.linalg.norm(b[1] - b[0]) - 0.9572) < 1e-9
