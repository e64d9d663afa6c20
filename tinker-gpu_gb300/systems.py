"""Seeded synthetic AMOEBA systems and the host-side description the library
consumes.

Water model: AMOEBA-WATER-2003 (Tinker test/file/commit_6fe8e913/water03.prm,
multipoles :139-150, polarize :159-160, scale factors :31-54), identical to
types 36/37 of amoeba09.prm.  Ions: amoeba09.prm Na+ (type 7, multipole :1221,
polarize :3051) and Cl- (type 15, :1261, :3059).  Geometry: rigid water,
O-H 0.9572 A, H-O-H 104.52 degrees.
"""
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import topology as topo

# type ids follow water03.prm for water and amoeba09.prm for the ions
WATER_O, WATER_H, NA_ION, CL_ION = 1, 2, 7, 15

# multipole records (kz, kx, ky, values in parameter-file units)
AMOEBA_RECORDS = {
    WATER_O: [(-2, -2, 0, [-0.51966, 0.0, 0.0, 0.14279, 0.37928, 0.0, -0.41809, 0.0, 0.0, 0.03881])],
    WATER_H: [(1, 2, 0, [0.25983, -0.03859, 0.0, -0.05818, -0.03673, 0.0, -0.10739, -0.00203, 0.0, 0.14412])],
    NA_ION: [(0, 0, 0, [1.0] + [0.0] * 9)],
    CL_ION: [(0, 0, 0, [-1.0] + [0.0] * 9)],
}
# polarizability (A^3), Thole, polarization-group partner types
AMOEBA_POLAR = {
    WATER_O: (0.837, 0.39, (WATER_H,)),
    WATER_H: (0.496, 0.39, (WATER_O,)),
    NA_ION: (0.12, 0.39, ()),
    CL_ION: (4.0, 0.39, ()),
}

# buffered 14-7 records (R0 diameter A, eps kcal/mol, reduction): water03.prm
# vdw 1 / 2 (= amoeba09.prm classes 34 / 35, :481-482), ions amoeba09.prm
# :454 and :462; vdw-12/13/14 scales 0 / 0 / 1 (amoeba09.prm:31-33)
AMOEBA_VDW = {
    WATER_O: (3.405, 0.110, 0.0),
    WATER_H: (2.655, 0.0135, 0.91),
    NA_ION: (2.955, 0.280, 0.0),
    CL_ION: (4.120, 0.340, 0.0),
}
AMOEBA_VDW_SCALES = {"vdw-12-scale": 0.0, "vdw-13-scale": 0.0, "vdw-14-scale": 1.0, "vdw-15-scale": 1.0}
VDW_CUTOFF = 9.0  # A, the benchmark configurations' van der Waals cutoff

# water valence (water03.prm :107, :118, :129 and its global terms :11-17):
# O-H bond, H-O-H angle, H-H Urey-Bradley
WATER_BOND = (556.85, 0.9572)
WATER_ANGLE = (48.70, 108.50)
WATER_UREY = (-7.60, 1.5537)
BOND_CUBIC, BOND_QUARTIC = -2.55, 3.793125
ANGLE_TERMS = (-0.014, 0.000056, -0.0000007, 0.000000022)

OH_BOND = 0.9572
HOH_ANGLE = 104.52


@dataclass
class VdwParams:
    """Buffered 14-7 van der Waals data for t9gb_set_vdw."""

    vtype: np.ndarray  # [n] index into the pair tables
    radmin: np.ndarray  # [t][t] combined R0, A
    epsilon: np.ndarray  # [t][t] combined well depth, kcal/mol
    red: np.ndarray  # [n] reduction factor toward parent (0: none)
    parent: np.ndarray  # [n] 0-based; the atom itself without reduction
    scaled_ik: np.ndarray  # [m][2]
    scaled_v: np.ndarray  # [m]
    taper: float
    off: float


def hal_params(types, bonds, records, scales, off, taper=None):
    """Tinker's buffered 14-7 set-up (kvdw): per-atom (R, eps, red) records
    keyed by atom type, CUBIC-MEAN radii and HHG well depths, the reduction
    parent = the first bonded neighbour, vdw-1x-scale pairs by bond
    separation, taper = 0.9 x cutoff unless given.
    records: type -> (radius, epsilon, reduction); scales: {'vdw-12-scale': ...}."""
    n = len(types)
    kinds = sorted(set(int(t) for t in types))
    idx = {t: j for j, t in enumerate(kinds)}
    R = np.array([records[t][0] for t in kinds], dtype=np.float64)
    E = np.array([records[t][1] for t in kinds], dtype=np.float64)
    r3, r2 = R[:, None] ** 3 + R[None, :] ** 3, R[:, None] ** 2 + R[None, :] ** 2
    radmin = np.where(r2 > 0, r3 / np.where(r2 > 0, r2, 1.0), 0.0)
    se = np.sqrt(E)
    den = (se[:, None] + se[None, :]) ** 2
    epsilon = np.where(den > 0, 4.0 * E[:, None] * E[None, :] / np.where(den > 0, den, 1.0), 0.0)
    adj, sep = topo.bond_distance_lists(n, bonds, 4)
    red = np.zeros(n)
    parent = np.arange(n, dtype=np.int32)
    for i, t in enumerate(types):
        r = records[int(t)][2] if len(records[int(t)]) > 2 else 0.0
        if r and adj[i]:
            red[i] = r
            parent[i] = adj[i][0]
    ik, sv = [], []
    for i in range(n):
        for k, d in sep[i].items():
            if k > i and 1 <= d <= 4:
                v = scales.get(f"vdw-1{d + 1}-scale", 1.0)
                if v != 1.0:
                    ik.append((i, k))
                    sv.append(v)
    return VdwParams(
        vtype=np.array([idx[int(t)] for t in types], dtype=np.int32),
        radmin=radmin,
        epsilon=epsilon,
        red=red,
        parent=parent,
        scaled_ik=np.array(ik, dtype=np.int32).reshape(-1, 2),
        scaled_v=np.array(sv, dtype=np.float64),
        taper=0.9 * off if taper is None else taper,
        off=off,
    )


@dataclass
class ValenceParams:
    """Bond / angle / Urey-Bradley terms for t9gb_set_valence."""

    bonds: np.ndarray  # [nb][4]: i, k, force constant, ideal length
    angles: np.ndarray  # [na][5]: a, vertex, c, force constant, ideal degrees
    ureys: np.ndarray  # [nu][5]: a, vertex, c, force constant, ideal 1-3 length
    bond_cubic: float = 0.0
    bond_quartic: float = 0.0
    angle_terms: tuple = (0.0, 0.0, 0.0, 0.0)  # cubic, quartic, pentic, sextic
    urey_cubic: float = 0.0
    urey_quartic: float = 0.0


@dataclass
class System:
    """Everything the polarization path needs about one system."""

    xyz: np.ndarray  # [n][3] float64, molecules kept whole (not wrapped)
    types: np.ndarray  # [n] int
    frames: np.ndarray  # [n][4] int32: zaxis, xaxis, yaxis (1-based signed), kind
    pole: np.ndarray  # [n][10] local-frame multipoles, MPL order
    polarity: np.ndarray  # [n]
    thole: np.ndarray  # [n]
    pdamp: np.ndarray  # [n]
    excl_ik: np.ndarray  # [m][2] int32, i < k
    excl_scale: np.ndarray  # [m][4]: m, d, p, u
    box: Optional[np.ndarray] = None  # orthorhombic edge lengths, None = no PBC
    mol_start: Optional[np.ndarray] = None  # first atom of each molecule
    mol_size: Optional[np.ndarray] = None
    name: str = ""
    settings: dict = field(default_factory=dict)
    ptype: Optional[np.ndarray] = None  # [n] polarization type, with thole_table
    thole_table: Optional[np.ndarray] = None  # [t][t] per-type-pair Thole coefficient
    exfld: Optional[np.ndarray] = None  # uniform external field [3], e/A^2
    vdw: Optional[VdwParams] = None  # buffered 14-7 van der Waals
    valence: Optional[ValenceParams] = None  # bond / angle / Urey-Bradley

    @property
    def n(self):
        return int(self.xyz.shape[0])


def build_system(xyz, types, bonds, records, polar, scales=None, box=None, name="", mol_start=None, mol_size=None):
    """Assemble frames, multipoles, polarizabilities and scaled pairs."""
    n = len(types)
    types = list(int(t) for t in types)
    adj, _ = topo.bond_distance_lists(n, bonds, 1)
    frames, pole = topo.assign_frames(types, adj, records)
    alpha = np.array([polar[t][0] for t in types], dtype=np.float64)
    thole = np.array([polar[t][1] for t in types], dtype=np.float64)
    pdamp = alpha ** (1.0 / 6.0)
    grp = topo.polar_groups(types, bonds, {t: set(v[2]) for t, v in polar.items()})
    sc = dict(topo.DEFAULT_SCALES)
    if scales:
        sc.update(scales)
    ik, scl = topo.scale_table(n, bonds, grp, sc)
    return System(
        xyz=np.asarray(xyz, dtype=np.float64).reshape(n, 3),
        types=np.array(types, dtype=np.int32),
        frames=frames,
        pole=pole,
        polarity=alpha,
        thole=thole,
        pdamp=pdamp,
        excl_ik=ik,
        excl_scale=scl,
        box=None if box is None else np.asarray(box, dtype=np.float64),
        name=name,
        mol_start=mol_start,
        mol_size=mol_size,
    )


def _random_rotations(rng, m):
    """Uniform rotations on SO(3) from uniform unit quaternions (Shoemake)."""
    u1, u2, u3 = rng.random(m), rng.random(m), rng.random(m)
    q = np.stack(
        [
            np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
            np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
            np.sqrt(u1) * np.sin(2 * np.pi * u3),
            np.sqrt(u1) * np.cos(2 * np.pi * u3),
        ],
        axis=1,
    )
    return quat_to_mat(q)


def quat_to_mat(q):
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    r = np.empty((q.shape[0], 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z)
    r[:, 0, 1] = 2 * (x * y - z * w)
    r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w)
    r[:, 1, 1] = 1 - 2 * (x * x + z * z)
    r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w)
    r[:, 2, 1] = 2 * (y * z + x * w)
    r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def water_geometry():
    """Body-frame O, H1, H2 positions (O at the origin, molecule in xz)."""
    half = math.radians(HOH_ANGLE) / 2
    return np.array(
        [
            [0.0, 0.0, 0.0],
            [OH_BOND * math.sin(half), 0.0, OH_BOND * math.cos(half)],
            [-OH_BOND * math.sin(half), 0.0, OH_BOND * math.cos(half)],
        ]
    )


@dataclass
class Lattice:
    """Seeded lattice of rigid molecules: centres, orientations, species."""

    centers: np.ndarray  # [m][3]
    rot: np.ndarray  # [m][3][3]
    species: np.ndarray  # [m]: 0 water, 1 Na+, 2 Cl-
    box: float


def make_lattice(nside, box, seed, jitter=0.1, n_sites=None, n_ion_pairs=0):
    rng = np.random.default_rng(seed)
    spacing = box / nside
    g = (np.arange(nside) + 0.5) * spacing - box / 2
    cx, cy, cz = np.meshgrid(g, g, g, indexing="ij")
    centers = np.stack([cx.ravel(), cy.ravel(), cz.ravel()], axis=1)
    if n_sites is not None and n_sites < len(centers):
        pick = np.sort(rng.permutation(len(centers))[:n_sites])
        centers = centers[pick]
    m = len(centers)
    centers = centers + rng.uniform(-jitter, jitter, size=(m, 3))
    rot = _random_rotations(rng, m)
    species = np.zeros(m, dtype=np.int32)
    if n_ion_pairs:
        ions = rng.permutation(m)[: 2 * n_ion_pairs]
        species[ions[:n_ion_pairs]] = 1
        species[ions[n_ion_pairs:]] = 2
    return Lattice(centers=centers, rot=rot, species=species, box=box)


def lattice_system(lat: Lattice, name=""):
    """Expand a lattice into atoms (O, H, H per water; one atom per ion)."""
    geom = water_geometry()
    xyz, types, bonds, mstart, msize = [], [], [], [], []
    for j in range(len(lat.centers)):
        base = len(types)
        mstart.append(base)
        if lat.species[j] == 0:
            pos = lat.centers[j] + geom @ lat.rot[j].T
            xyz.extend(pos.tolist())
            types.extend([WATER_O, WATER_H, WATER_H])
            bonds.extend([(base, base + 1), (base, base + 2)])
            msize.append(3)
        else:
            xyz.append(lat.centers[j].tolist())
            types.append(NA_ION if lat.species[j] == 1 else CL_ION)
            msize.append(1)
    return build_system(
        xyz,
        types,
        bonds,
        AMOEBA_RECORDS,
        AMOEBA_POLAR,
        box=[lat.box] * 3,
        name=name,
        mol_start=np.array(mstart, dtype=np.int64),
        mol_size=np.array(msize, dtype=np.int64),
    )


# The benchmark configurations: (molecules per side, box A, seed, PME grid,
# sites kept, ion pairs)
CONFIGS = {
    "water648": dict(nside=6, box=18.643, seed=0, nfft=24),
    "water12288": dict(nside=16, box=49.31, seed=1, nfft=64),
    "nacl23142": dict(nside=20, box=61.7, seed=2, nfft=72, n_sites=7742, n_ion_pairs=21),
    "water98304": dict(nside=32, box=98.62, seed=4, nfft=128),
}

# Polarization settings shared by every configuration.  Tinker keeps these
# keyword defaults in Fortran (kpolar, kewald, kneigh), absent from the
# reference checkout, so they are set here explicitly.
DEFAULT_SETTINGS = dict(
    aewald=0.5446,  # 1/A, Ewald coefficient for a 7 A cutoff at 1e-8
    ewald_cutoff=7.0,
    bsorder=5,
    poleps=1.0e-6,  # Debye, RMS residual
    politer=100,
    pcgprec=1,
    pcgguess=1,
    pcgpeek=1.0,
    udiag=2.0,  # uaccel
    usolve_cutoff=4.5,
    pbuffer=2.0,  # preconditioner list buffer
    list_buffer=2.0,
)


def make_config(name, vdw=False, valence=False, **over):
    """A benchmark configuration; vdw=True also attaches the buffered 14-7
    term (9 A cutoff, taper from 8.1 A), valence=True the water bond, angle
    and Urey-Bradley terms (the MD force field)."""
    cfg = dict(CONFIGS[name])
    cfg.update(over)
    lat = make_lattice(
        cfg["nside"],
        cfg["box"],
        cfg["seed"],
        n_sites=cfg.get("n_sites"),
        n_ion_pairs=cfg.get("n_ion_pairs", 0),
    )
    s = lattice_system(lat, name=name)
    s.settings = dict(DEFAULT_SETTINGS)
    s.settings["nfft"] = (cfg["nfft"],) * 3
    s.settings["use_ewald"] = 1
    s.lattice = lat
    if vdw:
        bonds = lattice_bonds(s)
        s.vdw = hal_params(s.types.tolist(), bonds, AMOEBA_VDW, AMOEBA_VDW_SCALES, VDW_CUTOFF)
    if valence:
        s.valence = water_valence(s)
    return s


def water_valence(s, bond=WATER_BOND, angle=WATER_ANGLE, urey=WATER_UREY):
    """Valence terms of the waters of a system (molecules of three atoms,
    oxygen first)."""
    b, a, u = [], [], []
    for st, sz in zip(s.mol_start, s.mol_size):
        if sz == 3:
            o, h1, h2 = int(st), int(st) + 1, int(st) + 2
            b += [(o, h1) + bond, (o, h2) + bond]
            a.append((h1, o, h2) + angle)
            u.append((h1, o, h2) + urey)
    return ValenceParams(bonds=np.array(b, dtype=np.float64).reshape(-1, 4),
                         angles=np.array(a, dtype=np.float64).reshape(-1, 5),
                         ureys=np.array(u, dtype=np.float64).reshape(-1, 5), bond_cubic=BOND_CUBIC,
                         bond_quartic=BOND_QUARTIC, angle_terms=ANGLE_TERMS)


def lattice_bonds(s):
    """O-H bonds of the lattice waters (molecule starts and sizes)."""
    bonds = []
    for st, sz in zip(s.mol_start, s.mol_size):
        if sz == 3:
            bonds.extend([(int(st), int(st) + 1), (int(st), int(st) + 2)])
    return bonds


class Trajectory:
    """Smooth seeded motion of rigid molecules about their lattice sites.

    Each molecule rattles (translation amplitude ~0.15 A, periods 80-200 fs)
    and librates (rotation amplitude ~20 degrees about a seeded axis, periods
    40-120 fs).  Frames 1 fs apart are correlated the way MD frames are, which
    is what the dipole predictors and the learned guess rely on.
    """

    def __init__(self, system, seed=11, dt_fs=1.0):
        lat = system.lattice
        rng = np.random.default_rng(seed)
        m = len(lat.centers)
        self.sys = system
        self.lat = lat
        self.dt = dt_fs
        d = rng.normal(size=(m, 3))
        self.tdir = d / np.linalg.norm(d, axis=1, keepdims=True) * 0.15
        self.tw = 2 * np.pi / rng.uniform(80, 200, size=m)
        self.tph = rng.uniform(0, 2 * np.pi, size=m)
        a = rng.normal(size=(m, 3))
        self.raxis = a / np.linalg.norm(a, axis=1, keepdims=True)
        self.ramp = np.radians(20.0)
        self.rw = 2 * np.pi / rng.uniform(40, 120, size=m)
        self.rph = rng.uniform(0, 2 * np.pi, size=m)
        self.geom = water_geometry()

    def frame(self, step):
        t = step * self.dt
        lat = self.lat
        c = lat.centers + self.tdir * np.sin(self.tw * t + self.tph)[:, None]
        ang = self.ramp * np.sin(self.rw * t + self.rph)
        k = self.raxis
        kx = np.zeros((len(k), 3, 3))
        kx[:, 0, 1], kx[:, 0, 2] = -k[:, 2], k[:, 1]
        kx[:, 1, 0], kx[:, 1, 2] = k[:, 2], -k[:, 0]
        kx[:, 2, 0], kx[:, 2, 1] = -k[:, 1], k[:, 0]
        s, cth = np.sin(ang)[:, None, None], np.cos(ang)[:, None, None]
        rlib = np.eye(3)[None] + s * kx + (1 - cth) * (kx @ kx)
        rot = rlib @ lat.rot
        xyz = np.empty((self.sys.n, 3))
        water = lat.species == 0
        starts = self.sys.mol_start
        wpos = c[water][:, None, :] + np.einsum("mij,aj->mai", rot[water], self.geom)
        ws = starts[water]
        for a in range(3):
            xyz[ws + a] = wpos[:, a, :]
        ions = ~water
        xyz[starts[ions]] = c[ions]
        return xyz


def ewald_coefficient(cutoff, eps=1.0e-8):
    """Ewald coefficient a with erfc(a r_c) / r_c = eps: doubling then 60+
    bisection steps, the rule Tinker applies when no coefficient is given
    (published with Tinker's ewaldcof routine)."""
    from math import erfc

    x, i = 0.5, 0
    ratio = eps + 1.0
    while ratio >= eps:
        i += 1
        x *= 2.0
        ratio = erfc(x * cutoff) / cutoff
    lo, hi = 0.0, x
    for _ in range(i + 60):
        x = 0.5 * (lo + hi)
        if erfc(x * cutoff) / cutoff >= eps:
            lo = x
        else:
            hi = x
    return x
