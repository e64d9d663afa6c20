"""Tinker file formats around the polarization path.

Readers: coordinates (.xyz, and .arc with every frame), keyword files (.key),
the parameter records the path uses (.prm: atom, vdw, bond, angle, ureybrad,
multipole, polarize and the scale / global keywords), MD restarts (.dyn).
Writers: coordinate frames (.xyz / appended .arc), induced and direct dipoles
(.uind / .udir: the coordinate layout with the dipole in Debye in place of the
position), MD restarts (.dyn).  `system_from_tinker` assembles a System (and
its van der Waals and valence terms) from an .xyz, its .key and the .prm the
key names, with Tinker's defaults for what the key leaves out.

The text layouts are Tinker's: the coordinate reader and writer of the
reference (src/rwcrd.cpp:200-290 read: title line, optional box line of six
numbers, one line per atom "index name x y z type bonds..."; :393-480 write:
"%6d  %s" title, " " + six "%12.6f" box values, "%6d  %-3s" + three "%12.6f"
+ "%6d" type + "%6d" per bond, wider fields for large coordinates) and the
restart files of its tests (test/file/tinkernist/water30.dyn: labelled blocks,
three Fortran D-exponent numbers per line).
"""
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import systems as S

# ---------------------------------------------------------------------------
# coordinates


@dataclass
class Frame:
    """One coordinate frame of an .xyz / .arc file (0-based atom indices)."""

    title: str
    names: list
    xyz: np.ndarray  # [n][3]
    types: np.ndarray  # [n]
    bonds: list  # sorted (i, k), i < k
    box: tuple = None  # (a, b, c, alpha, beta, gamma) or None

    @property
    def n(self):
        return len(self.names)


def _is_box_line(line):
    t = line.split()
    if len(t) < 6:
        return False
    try:
        [float(v) for v in t[:6]]
    except ValueError:
        return False
    return True


def read_xyz(path):
    """Every frame of a Tinker .xyz / .arc file."""
    with open(path) as f:
        lines = f.read().splitlines()
    frames, i = [], 0
    while i < len(lines) and lines[i].strip():
        head = lines[i].split(None, 1)
        n = int(head[0])
        title = head[1].strip() if len(head) > 1 else ""
        i += 1
        box = None
        if i < len(lines) and _is_box_line(lines[i]):
            box = tuple(float(v) for v in lines[i].split()[:6])
            i += 1
        names, xyz, types, bset = [], np.zeros((n, 3)), np.zeros(n, dtype=np.int32), set()
        for a in range(n):
            t = lines[i + a].split()
            idx = int(t[0]) - 1
            names.append(t[1])
            xyz[idx] = [float(t[2]), float(t[3]), float(t[4])]
            types[idx] = int(t[5]) if len(t) > 5 else 0
            for b in t[6:]:
                k = int(b) - 1
                bset.add((min(idx, k), max(idx, k)))
        i += n
        frames.append(Frame(title, names, xyz, types, sorted(bset), box))
    return frames


def _xyz_widths(values):
    lo, hi = min(0.0, float(np.min(values))), max(0.0, float(np.max(values)))
    w = 12
    if lo <= -1000.0 or hi >= 10000.0:
        w = 13
    if lo <= -10000.0 or hi >= 100000.0:
        w = 14
    return w


def format_frame(frame, values=None):
    """Text of one frame; values replaces the coordinates (dipole files)."""
    vals = frame.xyz if values is None else np.asarray(values, dtype=np.float64)
    n = frame.n
    iw = 6 if n < 1000000 else 7 if n < 10000000 else 8
    w = _xyz_widths(vals)
    out = [f"{n:{iw}d}  {frame.title}" if frame.title else f"{n:{iw}d}"]
    if frame.box is not None:
        out.append(" " + "".join(f"{v:{w}.6f}" for v in frame.box))
    nbr = [[] for _ in range(n)]
    for i, k in frame.bonds:
        nbr[i].append(k)
        nbr[k].append(i)
    for a in range(n):
        line = f"{a + 1:{iw}d}  {frame.names[a]:<3s}" + "".join(f"{v:{w}.6f}" for v in vals[a])
        line += f"{int(frame.types[a]):6d}" + "".join(f"{k + 1:6d}" for k in sorted(nbr[a]))
        out.append(line)
    return "\n".join(out) + "\n"


def write_xyz(path, frame, append=False):
    """One frame (append=True adds it to an .arc trajectory)."""
    with open(path, "a" if append else "w") as f:
        f.write(format_frame(frame))


def write_dipoles(path, frame, dipoles_debye, append=False):
    """An .uind / .udir file: the frame's layout with the dipoles (Debye)."""
    with open(path, "a" if append else "w") as f:
        f.write(format_frame(frame, dipoles_debye))


# ---------------------------------------------------------------------------
# MD restart (.dyn)

_DYN_BLOCKS = ("Current Atomic Positions", "Current Atomic Velocities", "Current Atomic Accelerations",
               "Alternate Atomic Accelerations")


def _fortran_d(v):
    """A number as Fortran's 0.ddddD+ee (16 digits after the point)."""
    if v == 0.0 or not math.isfinite(v):
        return "0.0000000000000000D+00" if v == 0.0 else repr(v)
    e = math.floor(math.log10(abs(v))) + 1
    m = v / 10.0 ** e
    s = f"{m:.16f}"
    if s.lstrip("-").startswith("1."):  # rounding carried into the next decade
        e += 1
        s = f"{v / 10.0 ** e:.16f}"
    sign = "-" if s.startswith("-") else ""
    return f"{sign}{s.lstrip('-')}D{'+' if e >= 0 else '-'}{abs(e):02d}"


def _dyn_line(vals):
    return "".join(f"{_fortran_d(float(v)):>26s}" for v in vals)


def write_dyn(path, title, xyz, vel, acc=None, acc_alt=None, box=None):
    """A Tinker MD restart: positions (A), velocities (A/ps), accelerations
    (A/ps^2; zero when not given), box lengths and angles."""
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    n = len(xyz)
    blocks = [xyz, np.asarray(vel, dtype=np.float64).reshape(n, 3),
              np.zeros((n, 3)) if acc is None else np.asarray(acc, dtype=np.float64).reshape(n, 3),
              np.zeros((n, 3)) if acc_alt is None else np.asarray(acc_alt, dtype=np.float64).reshape(n, 3)]
    out = [" Number of Atoms and Title :", f"{n:6d}  {title}"]
    if box is not None:
        b = list(box) + [90.0, 90.0, 90.0][: 6 - len(box)] if len(box) < 6 else list(box)
        out += [" Periodic Box Dimensions :", _dyn_line(b[:3]), _dyn_line(b[3:6])]
    for name, arr in zip(_DYN_BLOCKS, blocks):
        out.append(f" {name} :")
        out += [_dyn_line(r) for r in arr]
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def read_dyn(path):
    """(positions, velocities, accelerations, alternate accelerations, box)
    of a Tinker .dyn restart; box = (a, b, c, alpha, beta, gamma) or None."""
    with open(path) as f:
        lines = f.read().splitlines()
    n = int(lines[1].split()[0])

    def nums(ln):
        return [float(v.replace("D", "E").replace("d", "e")) for v in ln.split()]

    def block(title, rows):
        for j, ln in enumerate(lines):
            if ln.strip().startswith(title):
                return np.array([nums(r) for r in lines[j + 1 : j + 1 + rows]])
        return None

    box = block("Periodic Box Dimensions", 2)
    return (block(_DYN_BLOCKS[0], n), block(_DYN_BLOCKS[1], n), block(_DYN_BLOCKS[2], n), block(_DYN_BLOCKS[3], n),
            None if box is None else tuple(box.reshape(-1)))


# ---------------------------------------------------------------------------
# keyword and parameter files


def read_key(path):
    """Keywords of a .key file: lower-case keyword -> list of value strings
    (the last occurrence wins; a keyword without values maps to [])."""
    keys = {}
    with open(path) as f:
        for ln in f:
            s = ln.split("#", 1)[0].split("!", 1)[0].strip()
            if not s:
                continue
            t = s.split()
            keys[t[0].lower()] = t[1:]
    return keys


@dataclass
class Params:
    """The parameter records the polarization path and its MD terms use."""

    atoms: dict = field(default_factory=dict)  # type -> (class, name, atomic number, mass, valence)
    vdw: dict = field(default_factory=dict)  # class -> [radius, epsilon, reduction]
    bond: dict = field(default_factory=dict)  # (c1, c2), c1 <= c2 -> (k, r0)
    angle: dict = field(default_factory=dict)  # (c1, c2, c3), c1 <= c3 -> (k, theta0 degrees)
    urey: dict = field(default_factory=dict)  # (c1, c2, c3), c1 <= c3 -> (k, r13)
    multipole: dict = field(default_factory=dict)  # type -> [(kz, kx, ky, 10 values)]
    polarize: dict = field(default_factory=dict)  # type -> (alpha, thole, group partner types)
    keywords: dict = field(default_factory=dict)  # lower-case keyword -> value strings


def read_prm(path):
    """The records of a Tinker parameter file that this library consumes."""
    P = Params()
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines):
        t = lines[i].split()
        if not t or t[0].startswith("#") or t[0].startswith("!"):
            i += 1
            continue
        k = t[0].lower()
        if k == "atom":
            # atom type class name "description" atomic-number mass valence
            ty, cl = int(t[1]), int(t[2])
            P.atoms[ty] = (cl, t[3], int(t[-3]), float(t[-2]), int(t[-1]))
        elif k == "vdw":
            P.vdw[int(t[1])] = [float(v) for v in t[2:5]]
        elif k == "bond":
            c1, c2 = sorted((int(t[1]), int(t[2])))
            P.bond[(c1, c2)] = (float(t[3]), float(t[4]))
        elif k in ("angle", "ureybrad"):
            c1, c2, c3 = int(t[1]), int(t[2]), int(t[3])
            key = (c1, c2, c3) if c1 <= c3 else (c3, c2, c1)
            (P.angle if k == "angle" else P.urey)[key] = (float(t[4]), float(t[5]))
        elif k == "multipole":
            ids = [int(v) for v in t[1:-1]]
            vals = [float(t[-1])]
            for j in range(1, 5):
                vals += [float(v) for v in lines[i + j].split()]
            while len(ids) < 4:
                ids.append(0)
            P.multipole.setdefault(ids[0], []).append((ids[1], ids[2], ids[3], vals))
            i += 5
            continue
        elif k == "polarize":
            P.polarize[int(t[1])] = (float(t[2]), float(t[3]), tuple(int(v) for v in t[4:]))
        else:
            P.keywords[k] = t[1:]
        i += 1
    return P


# ---------------------------------------------------------------------------
# a System from the files

# Tinker keyword defaults the path depends on (kewald, kpolar, kvdw)
DEFAULT_EWALD_CUTOFF = 9.0
DEFAULT_VDW_CUTOFF = 9.0
PME_POINTS_PER_A = 1.2


def pme_grid_size(length):
    """The smallest FFT size with prime factors 2, 3, 5 at or above
    1.2 points per A of the box edge (Tinker's default PME grid)."""
    need = max(1, int(math.ceil(PME_POINTS_PER_A * length - 1e-9)))
    m = need
    while True:
        r = m
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def _fkey(keys, name, default):
    v = keys.get(name)
    return float(v[0]) if v else default


def _scales(params, keys):
    sc = {}
    for src in (params.keywords, keys):
        for k, v in src.items():
            if k.endswith("-scale") or k.endswith("-intra"):
                if v:
                    sc[k] = float(v[0])
    return sc


def resolve_files(xyz_path, key_path=None, prm_path=None):
    """(key path or None, parameter-file path) for a coordinate file: the
    .key beside the .xyz unless given, and the parameter file that the key
    names (relative to the key, .prm added when missing) unless given."""
    if key_path is None:
        cand = os.path.splitext(xyz_path)[0] + ".key"
        key_path = cand if os.path.exists(cand) else None
    if prm_path is None:
        pv = read_key(key_path).get("parameters") if key_path else None
        if not pv:
            raise ValueError("no parameter file: give prm_path or a 'parameters' keyword")
        prm_path = pv[0]
        if not os.path.isabs(prm_path):
            prm_path = os.path.join(os.path.dirname(key_path), prm_path)
        if not os.path.exists(prm_path) and os.path.exists(prm_path + ".prm"):
            prm_path += ".prm"
    return key_path, prm_path


def predictor_from_keys(keys):
    """The induced-dipole predictor a keyword file selects, as the reference
    maps it (src/amoeba/epolar.cpp:426-444): POLAR-PREDICT ASPC -> 1, GEAR ->
    2; no POLAR-PREDICT -> 0 (none).  POLAR-PREDICT without a modifier (as in
    the reference's test/file/water30/water30.key) -> 1: the Fortran keyword
    reader that fills the reference's default modifier is not part of the
    reference, and ASPC is the predictor its CUDA path and its tests use.
    LSQR, which the reference's CUDA path lacks, raises ValueError."""
    if "polar-predict" not in keys:
        return 0
    v = keys["polar-predict"]
    mod = v[0].upper() if v else "ASPC"
    if mod == "ASPC":
        return 1
    if mod == "GEAR":
        return 2
    raise ValueError(f"polar-predict {mod}: only ASPC and GEAR have a GPU path")


def system_from_tinker(xyz_path, key_path=None, prm_path=None, frame=0, vdw=True, valence=True):
    """A System from a Tinker coordinate file, its keyword file (default: the
    .key beside the .xyz) and the parameter file the key names (or prm_path).
    Settings follow the keywords: ewald, ewald-cutoff, ewald-alpha,
    pme-grid, pme-order, polar-eps, polar-iter, usolve-cutoff, usolve-diag,
    pcg-peek, pcg-guess, pcg-precond, neighbor-list buffer (list-buffer),
    a-axis / b-axis / c-axis (else the file's box line), vdw-cutoff,
    vdw-taper, polar-predict (settings["predictor"], predictor_from_keys);
    Tinker's defaults otherwise."""
    fr = read_xyz(xyz_path)[frame]
    key_path, prm_path = resolve_files(xyz_path, key_path, prm_path)
    keys = read_key(key_path) if key_path else {}
    P = read_prm(prm_path)
    types = [int(t) for t in fr.types]
    kinds = sorted(set(types))
    missing = [t for t in kinds if t not in P.multipole or t not in P.polarize]
    if missing:
        raise ValueError(f"no multipole / polarize record for atom types {missing}")
    records = {t: P.multipole[t] for t in kinds}
    polar = {t: P.polarize[t] for t in kinds}
    # box: keywords first, then the coordinate file's box line
    box = None
    if "a-axis" in keys:
        a = _fkey(keys, "a-axis", 0.0)
        box = (a, _fkey(keys, "b-axis", a), _fkey(keys, "c-axis", a))
    elif fr.box is not None:
        box = tuple(fr.box[:3])
    s = S.build_system(fr.xyz, types, fr.bonds, records, polar, scales=_scales(P, keys), box=box,
                       name=fr.title)
    st = dict(S.DEFAULT_SETTINGS)
    ewald = "ewald" in keys and box is not None
    st["use_ewald"] = 1 if ewald else 0
    cut = _fkey(keys, "ewald-cutoff", DEFAULT_EWALD_CUTOFF) if ewald else _fkey(keys, "mpole-cutoff", 1.0e9)
    st["ewald_cutoff"] = cut
    if ewald:
        st["aewald"] = _fkey(keys, "ewald-alpha", S.ewald_coefficient(cut))
        g = keys.get("pme-grid")
        if g:
            nf = [int(v) for v in g[:3]]
            nf += [nf[-1]] * (3 - len(nf))
        else:
            nf = [pme_grid_size(L) for L in box]
        st["nfft"] = tuple(nf)
        st["bsorder"] = int(_fkey(keys, "pme-order", 5))
    st["poleps"] = _fkey(keys, "polar-eps", st["poleps"])
    st["politer"] = int(_fkey(keys, "polar-iter", st["politer"]))
    st["usolve_cutoff"] = _fkey(keys, "usolve-cutoff", st["usolve_cutoff"])
    st["udiag"] = _fkey(keys, "usolve-diag", st["udiag"])
    st["pcgpeek"] = _fkey(keys, "pcg-peek", st["pcgpeek"])
    if "pcg-noguess" in keys:
        st["pcgguess"] = 0
    if "pcg-noprecond" in keys:
        st["pcgprec"] = 0
    st["list_buffer"] = _fkey(keys, "list-buffer", st["list_buffer"])
    st["predictor"] = predictor_from_keys(keys)
    s.settings = st
    if vdw and P.vdw:
        vrec = {}
        for t in kinds:
            cl = P.atoms[t][0]
            v = P.vdw[cl]
            vrec[t] = (v[0], v[1], v[2] if len(v) > 2 else 0.0)
        vsc = {k: v for k, v in _scales(P, keys).items() if k.startswith("vdw-")}
        sc = dict(S.AMOEBA_VDW_SCALES)
        sc.update(vsc)
        off = _fkey(keys, "vdw-cutoff", DEFAULT_VDW_CUTOFF)
        taper = _fkey(keys, "vdw-taper", 0.9) if "vdw-taper" in keys else None
        if taper is not None and taper <= 1.0:
            taper *= off  # a fraction of the cutoff
        s.vdw = S.hal_params(types, fr.bonds, vrec, sc, off, taper)
    if valence:
        s.valence = valence_terms(types, fr.bonds, P)
    return s


def valence_terms(types, bonds, P):
    """Bond, angle and Urey-Bradley terms of a molecule graph from the
    parameter records (by atom class; harmonic angles, first ideal value)."""
    cls = [P.atoms[int(t)][0] for t in types]
    n = len(types)
    adj = [[] for _ in range(n)]
    b = []
    for i, k in bonds:
        adj[i].append(k)
        adj[k].append(i)
        rec = P.bond.get(tuple(sorted((cls[i], cls[k]))))
        if rec:
            b.append((i, k) + rec)
    a, u = [], []
    for m in range(n):
        nb = sorted(adj[m])
        for x in range(len(nb)):
            for y in range(x + 1, len(nb)):
                i, k = nb[x], nb[y]
                key = (cls[i], cls[m], cls[k]) if cls[i] <= cls[k] else (cls[k], cls[m], cls[i])
                if key in P.angle:
                    a.append((i, m, k) + P.angle[key])
                if key in P.urey:
                    u.append((i, m, k) + P.urey[key])
    g = P.keywords
    f = lambda name: float(g[name][0]) if g.get(name) else 0.0
    return S.ValenceParams(
        bonds=np.array(b, dtype=np.float64).reshape(-1, 4),
        angles=np.array(a, dtype=np.float64).reshape(-1, 5),
        ureys=np.array(u, dtype=np.float64).reshape(-1, 5),
        bond_cubic=f("bond-cubic"), bond_quartic=f("bond-quartic"),
        angle_terms=(f("angle-cubic"), f("angle-quartic"), f("angle-pentic"), f("angle-sextic")),
        urey_cubic=f("urey-cubic"), urey_quartic=f("urey-quartic"))


def masses(types, P):
    """Atomic masses by atom type from the parameter records."""
    return np.array([P.atoms[int(t)][3] for t in types], dtype=np.float64)
