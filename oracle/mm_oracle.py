"""FP64 numpy oracle of the terms around induce() on the MD path: the
buffered 14-7 van der Waals energy and the bond / angle / Urey-Bradley
valence energies.  Test infrastructure only (tests, smoke, bench baselines);
gradients and virials come from central differences of these energies
(oracle.py's _fd / _strain_fd).

  hal_energy      include/seq/pair_hal.h:52-96 (pair_hal_v2, vlambda = 1),
                  include/math/switch.h:22-33 (switchTaper5), reduced sites as
                  src/cu/ehal.cu (xred = red (x - x_parent) + x_parent)
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
