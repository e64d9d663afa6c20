"""FP64 numpy oracle of the terms around induce() on the MD path: the
buffered 14-7 van der Waals energy and the bond / angle / Urey-Bradley
valence energies.  Test infrastructure only (tests, smoke, bench baselines);
gradients and virials come from central differences of these energies
(oracle.py's _fd / _strain_fd).

  hal_energy      include/seq/pair_hal.h:52-96 (pair_hal_v2, vlambda = 1),
                  include/math/switch.h:22-33 (switchTaper5), reduced sites as
                  src/cu/ehal.cu (xred = red (x - x_parent) + x_parent)
  bond_energy     include/seq/bond.h:44-59 (HARMONIC with cubic / quartic,
                  bondunit 1)
  angle_energy    include/seq/angle.h:88-115 (HARMONIC, angle in degrees,
                  angunit (pi/180)^2, cubic ... sextic)
  urey_energy     include/seq/urey.h:44-53 (ureyunit 1, cubic / quartic)
"""
import numpy as np

HAL_DELTA, HAL_GAMMA = 0.07, 0.12


def _image(d, box):
    if box is None:
        return d
    box = np.asarray(box, dtype=np.float64)
    return d - box * np.round(d / box)


def hal_sites(xyz, vdw, box):
    """Reduced van der Waals sites [n][3]."""
    xyz = np.asarray(xyz, dtype=np.float64)
    p = np.asarray(vdw.parent)
    return xyz[p] + np.asarray(vdw.red)[:, None] * _image(xyz - xyz[p], box)


def hal_pair(r, rv, eps, taper, off):
    """Energy of pairs at distance r (arrays)."""
    rho = r / rv
    t1 = ((1 + HAL_DELTA) / (rho + HAL_DELTA)) ** 7
    t2 = (1 + HAL_GAMMA) / (rho ** 7 + HAL_GAMMA)
    e = eps * t1 * (t2 - 2)
    x = (r - off) / (taper - off) if off > taper else np.zeros_like(r)
    s = x ** 3 * (6 * x * x - 15 * x + 10)
    return np.where(r > taper, e * s, e)


def hal_energy(system, xyz=None, box="system"):
    """Total buffered 14-7 energy, kcal/mol (all pairs, minimum image)."""
    v = system.vdw
    xyz = system.xyz if xyz is None else xyz
    box = system.box if isinstance(box, str) else box
    x = hal_sites(xyz, v, box)
    n = len(x)
    scale = np.ones((n, n))
    for (i, k), s in zip(np.asarray(v.scaled_ik).reshape(-1, 2), np.asarray(v.scaled_v)):
        scale[i, k] = scale[k, i] = s
    iu, ku = np.triu_indices(n, 1)
    d = _image(x[ku] - x[iu], box)
    r = np.sqrt((d * d).sum(1))
    t = np.asarray(v.vtype)
    rv = np.asarray(v.radmin)[t[iu], t[ku]]
    eps = np.asarray(v.epsilon)[t[iu], t[ku]] * scale[iu, ku]
    m = (r <= v.off) & (eps != 0)
    return float(hal_pair(r[m], rv[m], eps[m], v.taper, v.off).sum())


def _image_opt(d, box):
    return d if box is None else _image(d, box)


def bond_energy(xyz, bonds, cubic, quartic, box=None):
    """bonds: rows (i, k, force constant, ideal length)."""
    b = np.asarray(bonds, dtype=np.float64).reshape(-1, 4)
    i, k = b[:, 0].astype(int), b[:, 1].astype(int)
    x = np.asarray(xyz, dtype=np.float64)
    r = np.sqrt((_image_opt(x[i] - x[k], box) ** 2).sum(1))
    dt = r - b[:, 3]
    return float((b[:, 2] * dt * dt * (1 + cubic * dt + quartic * dt * dt)).sum())


def angle_energy(xyz, angles, cubic, quartic, pentic, sextic, box=None):
    """angles: rows (a, vertex, c, force constant, ideal angle in degrees)."""
    g = np.asarray(angles, dtype=np.float64).reshape(-1, 5)
    a, m, c = (g[:, j].astype(int) for j in range(3))
    x = np.asarray(xyz, dtype=np.float64)
    u = _image_opt(x[a] - x[m], box)
    v = _image_opt(x[c] - x[m], box)
    cos = (u * v).sum(1) / np.sqrt((u * u).sum(1) * (v * v).sum(1))
    ang = np.degrees(np.arccos(np.clip(cos, -1, 1)))
    dt = ang - g[:, 4]
    unit = (np.pi / 180) ** 2
    return float((unit * g[:, 3] * dt ** 2 * (1 + cubic * dt + quartic * dt ** 2 + pentic * dt ** 3 + sextic * dt ** 4)).sum())


def urey_energy(xyz, ureys, cubic, quartic, box=None):
    """ureys: rows (a, vertex, c, force constant, ideal a-c distance)."""
    u = np.asarray(ureys, dtype=np.float64).reshape(-1, 5)
    a, c = u[:, 0].astype(int), u[:, 2].astype(int)
    x = np.asarray(xyz, dtype=np.float64)
    r = np.sqrt((_image_opt(x[a] - x[c], box) ** 2).sum(1))
    dt = r - u[:, 4]
    return float((u[:, 3] * dt * dt * (1 + cubic * dt + quartic * dt * dt)).sum())
