"""ctypes front end of the FP64 oracle (oracle/t9_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker.  The product library
never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libt9oracle.so")
SRC = os.path.join(HERE, "t9_oracle.c")


def build(force=False):
    """Compile the oracle with gcc (OpenMP, -O2, portable flags)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class OrSystem(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("x", C.POINTER(C.c_double)),
        ("y", C.POINTER(C.c_double)),
        ("z", C.POINTER(C.c_double)),
        ("rpole", C.POINTER(C.c_double)),
        ("polarity", C.POINTER(C.c_double)),
        ("thole", C.POINTER(C.c_double)),
        ("pdamp", C.POINTER(C.c_double)),
        ("nexcl", C.c_int),
        ("excl_ik", C.POINTER(C.c_int)),
        ("excl_scale", C.POINTER(C.c_double)),
        ("periodic", C.c_int),
        ("box", C.c_double * 3),
        ("use_ewald", C.c_int),
        ("aewald", C.c_double),
        ("nfft", C.c_int * 3),
        ("bsorder", C.c_int),
        ("cutoff", C.c_double),
        ("electric", C.c_double),
        ("nthl", C.c_int),
        ("ptype", C.POINTER(C.c_int)),
        ("thl", C.POINTER(C.c_double)),
        ("exfld", C.c_double * 3),
        ("real_only", C.c_int),
    ]


class OrInduceOpts(C.Structure):
    _fields_ = [
        ("poleps", C.c_double),
        ("politer", C.c_int),
        ("pcgpeek", C.c_double),
        ("udiag", C.c_double),
        ("pcgprec", C.c_int),
        ("precond_cutoff", C.c_double),
        ("guess", C.c_int),
        ("debye", C.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        dp = C.POINTER(C.c_double)
        _lib.or_rotpole.argtypes = [C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp, dp]
        _lib.or_frames.argtypes = [C.c_int, C.POINTER(C.c_int), dp, dp, dp, dp]
        _lib.or_dfield.argtypes = [C.POINTER(OrSystem), dp, dp]
        _lib.or_ufield.argtypes = [C.POINTER(OrSystem), dp, dp, dp, dp]
        _lib.or_induce.argtypes = [C.POINTER(OrSystem), C.POINTER(OrInduceOpts), dp, dp, dp, dp, dp]
        _lib.or_induce.restype = C.c_int
        _lib.or_sparse_precond_apply.argtypes = [C.POINTER(OrSystem), C.c_double, C.c_double, dp, dp, dp, dp]
        _lib.or_bsmod.argtypes = [C.c_int, C.c_int, dp]
        _lib.or_bsplgen_export.argtypes = [C.c_double, C.c_int, C.c_int, dp]
        _lib.or_aspc_sum.argtypes = [C.c_int, C.c_int, dp, dp]
        _lib.or_gear_sum.argtypes = [C.c_int, C.c_int, dp, dp]
        _lib.or_empole_energy.argtypes = [C.POINTER(OrSystem), dp]
        _lib.or_empole_energy.restype = C.c_double
        _lib.or_epolar_energy_dot.argtypes = [C.POINTER(OrSystem), dp, dp]
        _lib.or_epolar_energy_dot.restype = C.c_double
        _lib.or_set_threads.argtypes = [C.c_int]
        _lib.or_nthreads.restype = C.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def set_threads(t):
    lib().or_set_threads(int(t))


def nthreads():
    return lib().or_nthreads()


def rotpole(system, xyz=None):
    """Global-frame multipoles [n][10] for the current coordinates."""
    xyz = np.ascontiguousarray(system.xyz if xyz is None else xyz, dtype=np.float64)
    x, y, z = [np.ascontiguousarray(xyz[:, d]) for d in range(3)]
    frames = np.ascontiguousarray(system.frames, dtype=np.int32)
    pole = np.ascontiguousarray(system.pole, dtype=np.float64).copy()
    out = np.zeros_like(pole)
    lib().or_rotpole(system.n, _ip(frames), _dp(pole), _dp(x), _dp(y), _dp(z), _dp(out))
    return out


def frames(system, xyz=None):
    """Local multipole frames [n][3][3], rows = x, y, z axes in the global frame."""
    xyz = np.ascontiguousarray(system.xyz if xyz is None else xyz, dtype=np.float64)
    x, y, z = [np.ascontiguousarray(xyz[:, d]) for d in range(3)]
    fr = np.ascontiguousarray(system.frames, dtype=np.int32)
    out = np.zeros((system.n, 9))
    lib().or_frames(system.n, _ip(fr), _dp(x), _dp(y), _dp(z), _dp(out))
    return out.reshape(system.n, 3, 3)


class OracleSystem:
    """Holds the numpy buffers an or_system points at."""

    def __init__(self, system, xyz=None, rpole=None, use_ewald=None, cutoff=None, nfft=None, real_only=False):
        st = system.settings
        xyz = np.ascontiguousarray(system.xyz if xyz is None else xyz, dtype=np.float64)
        self.x, self.y, self.z = [np.ascontiguousarray(xyz[:, d]) for d in range(3)]
        self.rpole = np.ascontiguousarray(rotpole(system, xyz) if rpole is None else rpole, dtype=np.float64)
        self.polarity = np.ascontiguousarray(system.polarity, dtype=np.float64)
        self.thole = np.ascontiguousarray(system.thole, dtype=np.float64)
        self.pdamp = np.ascontiguousarray(system.pdamp, dtype=np.float64)
        self.excl_ik = np.ascontiguousarray(system.excl_ik, dtype=np.int32).reshape(-1)
        self.excl_scale = np.ascontiguousarray(system.excl_scale, dtype=np.float64).reshape(-1)
        s = OrSystem()
        s.n = system.n
        s.x, s.y, s.z = _dp(self.x), _dp(self.y), _dp(self.z)
        s.rpole = _dp(self.rpole)
        s.polarity, s.thole, s.pdamp = _dp(self.polarity), _dp(self.thole), _dp(self.pdamp)
        s.nexcl = len(self.excl_ik) // 2
        s.excl_ik = _ip(self.excl_ik)
        s.excl_scale = _dp(self.excl_scale)
        ew = st.get("use_ewald", 1) if use_ewald is None else use_ewald
        s.periodic = 1 if system.box is not None else 0
        if system.box is not None:
            for d in range(3):
                s.box[d] = float(system.box[d])
        s.use_ewald = int(ew)
        s.aewald = float(st.get("aewald", 0.0))
        nf = st.get("nfft", (0, 0, 0)) if nfft is None else nfft
        for d in range(3):
            s.nfft[d] = int(nf[d])
        s.bsorder = int(st.get("bsorder", 5))
        s.cutoff = float(st.get("ewald_cutoff", 1.0e9) if cutoff is None else cutoff)
        from_units = __import__("importlib").import_module("tinker-gpu_gb300.units")
        s.electric = from_units.ELECTRIC
        ef = getattr(system, "exfld", None)
        if ef is not None:
            for d in range(3):
                s.exfld[d] = float(ef[d])
        if getattr(system, "ptype", None) is not None:
            self.ptype = np.ascontiguousarray(system.ptype, dtype=np.int32)
            self.thl = np.ascontiguousarray(system.thole_table, dtype=np.float64)
            s.nthl = int(self.thl.shape[0])
            s.ptype, s.thl = _ip(self.ptype), _dp(self.thl)
        s.real_only = 1 if real_only else 0
        self.s = s
        self.n = system.n
        self.settings = st

    def dfield(self):
        f = np.zeros((self.n, 3))
        fp = np.zeros((self.n, 3))
        lib().or_dfield(C.byref(self.s), _dp(f), _dp(fp))
        return f, fp

    def ufield(self, uind, uinp):
        uind = np.ascontiguousarray(uind, dtype=np.float64)
        uinp = np.ascontiguousarray(uinp, dtype=np.float64)
        f = np.zeros((self.n, 3))
        fp = np.zeros((self.n, 3))
        lib().or_ufield(C.byref(self.s), _dp(uind), _dp(uinp), _dp(f), _dp(fp))
        return f, fp

    def opts(self, guess=None, politer=None, poleps=None, pcgprec=None):
        from_units = __import__("importlib").import_module("tinker-gpu_gb300.units")
        st = self.settings
        o = OrInduceOpts()
        o.poleps = float(st.get("poleps", 1e-6) if poleps is None else poleps)
        o.politer = int(st.get("politer", 100) if politer is None else politer)
        o.pcgpeek = float(st.get("pcgpeek", 1.0))
        o.udiag = float(st.get("udiag", 2.0))
        o.pcgprec = int(st.get("pcgprec", 1) if pcgprec is None else pcgprec)
        o.precond_cutoff = float(st.get("usolve_cutoff", 4.5) + st.get("pbuffer", 2.0))
        o.guess = int(1 if guess is None else guess)
        o.debye = from_units.DEBYE
        return o

    def induce(self, guess=None, uind0=None, uinp0=None, **kw):
        """Returns (uind, uinp, udir, udirp, iterations, final eps in Debye)."""
        uind = np.zeros((self.n, 3)) if uind0 is None else np.array(uind0, dtype=np.float64)
        uinp = np.zeros((self.n, 3)) if uinp0 is None else np.array(uinp0, dtype=np.float64)
        if guess is None:
            guess = 2 if uind0 is not None else 1
        udir = np.zeros((self.n, 3))
        udirp = np.zeros((self.n, 3))
        eps = C.c_double(0)
        o = self.opts(guess=guess, **kw)
        it = lib().or_induce(C.byref(self.s), C.byref(o), _dp(uind), _dp(uinp), _dp(udir), _dp(udirp), C.byref(eps))
        return uind, uinp, udir, udirp, it, eps.value

    def empole_energy(self):
        """(total, [real, recip, self]) permanent-multipole energy, kcal/mol."""
        parts = np.zeros(3)
        e = lib().or_empole_energy(C.byref(self.s), _dp(parts))
        return e, parts

    def epolar_energy(self, uind=None, udirp=None):
        """Polarization energy by the dot product; solves induce() when no dipoles are given."""
        if uind is None:
            uind, _, _, udirp, *_ = self.induce()
        uind = np.ascontiguousarray(uind, dtype=np.float64)
        udirp = np.ascontiguousarray(udirp, dtype=np.float64)
        return lib().or_epolar_energy_dot(C.byref(self.s), _dp(uind), _dp(udirp))

    def sparse_precond(self, rsd, rsdp):
        rsd = np.ascontiguousarray(rsd, dtype=np.float64)
        rsdp = np.ascontiguousarray(rsdp, dtype=np.float64)
        z = np.zeros((self.n, 3))
        zp = np.zeros((self.n, 3))
        st = self.settings
        cut = float(st.get("usolve_cutoff", 4.5) + st.get("pbuffer", 2.0))
        lib().or_sparse_precond_apply(C.byref(self.s), cut, float(st.get("udiag", 2.0)), _dp(rsd), _dp(rsdp), _dp(z), _dp(zp))
        return z, zp


# ---------------------------------------------------------------------------
# gradients by central differences of the FP64 energies
#
# empole: E(x) with the multipoles re-rotated into each displaced geometry,
# so the frame (torque) terms are included.  epolar: the reference's
# polarization gradient (src/amoeba/epolar.cpp, include/seq/pair_polar.h,
# src/cu/epolarrecip.cu) is the gradient at fixed induced dipoles of
#   G(x) = -1/2 f [ u_p . E_d(x) + u_d . E_p(x) + u_d . E_u(u_p)(x) ]
# with E_d / E_p the d- / p-scaled permanent fields (dfield) and E_u the
# mutual field (ufield); the permanent multipoles again follow the frames.
# Both reproduce the reference's golden gradients (test/localframe.cpp).


def _fd(fun, xyz, atoms, h):
    g = np.zeros((len(atoms), 3))
    for j, a in enumerate(atoms):
        for d in range(3):
            xp = xyz.copy()
            xp[a, d] += h
            xm = xyz.copy()
            xm[a, d] -= h
            g[j, d] = (fun(xp) - fun(xm)) / (2 * h)
    return g


def empole_gradient_fd(system, xyz=None, atoms=None, h=1e-5, **kw):
    """dE_mpole/dx [len(atoms)][3], kcal/mol/A."""
    xyz = np.array(system.xyz if xyz is None else xyz, dtype=np.float64)
    atoms = range(system.n) if atoms is None else atoms
    return _fd(lambda x: OracleSystem(system, x, **kw).empole_energy()[0], xyz, list(atoms), h)


def epolar_g(system, xyz, uind, uinp, **kw):
    o = OracleSystem(system, xyz, **kw)
    fd, fp = o.dfield()
    _, fu = o.ufield(np.zeros_like(uinp), uinp)
    return -0.5 * o.s.electric * ((uinp * fd).sum() + (uind * fp).sum() + (uind * fu).sum())


def epolar_gradient_fd(system, uind, uinp, xyz=None, atoms=None, h=1e-5, **kw):
    """Polarization gradient at fixed dipoles [len(atoms)][3], kcal/mol/A."""
    xyz = np.array(system.xyz if xyz is None else xyz, dtype=np.float64)
    atoms = range(system.n) if atoms is None else atoms
    ud = np.asarray(uind, dtype=np.float64)
    up = np.asarray(uinp, dtype=np.float64)
    return _fd(lambda x: epolar_g(system, x, ud, up, **kw), xyz, list(atoms), h)


def _strain_fd(system, fun, diag_only, h):
    """dF/d(eps)_ab for x -> (I + eps) x (box edges scaled with the diagonal)."""
    import dataclasses

    S = np.zeros((3, 3))
    for a in range(3):
        for b in range(3):
            if diag_only and a != b:
                S[a, b] = np.nan
                continue
            vals = []
            for sg in (1, -1):
                eps = np.zeros((3, 3))
                eps[a, b] = sg * h
                x = np.asarray(system.xyz, dtype=np.float64) @ (np.eye(3) + eps).T
                box = None if system.box is None else np.asarray(system.box, dtype=np.float64) * (1 + np.diag(eps))
                vals.append(fun(dataclasses.replace(system, xyz=x, box=box)))
            S[a, b] = (vals[0] - vals[1]) / (2 * h)
    return S


def empole_virial_fd(system, diag_only=False, h=1e-6, **kw):
    """Virial dE_mpole/d(eps) [3][3] (orthorhombic PBC: diagonal only, the
    off-diagonal entries are NaN)."""
    return _strain_fd(system, lambda s2: OracleSystem(s2, **kw).empole_energy()[0], diag_only, h)


def epolar_virial_fd(system, uind, uinp, diag_only=False, h=1e-6, **kw):
    """Polarization virial at fixed dipoles, dG/d(eps) [3][3]."""
    ud = np.asarray(uind, dtype=np.float64)
    up = np.asarray(uinp, dtype=np.float64)
    return _strain_fd(system, lambda s2: epolar_g(s2, s2.xyz, ud, up, **kw), diag_only, h)


def bsmod(nfft, order=5):
    out = np.zeros(nfft)
    lib().or_bsmod(nfft, order, _dp(out))
    return out


def bsplgen(w, order=5, level=4):
    th = np.zeros(4 * order)
    lib().or_bsplgen_export(float(w), order, level, _dp(th))
    return th.reshape(order, 4)


def aspc_sum(hist, nualt):
    hist = np.ascontiguousarray(hist, dtype=np.float64)
    n3 = hist[0].size
    out = np.zeros(n3)
    lib().or_aspc_sum(n3, int(nualt), _dp(hist), _dp(out))
    return out


def gear_sum(hist, nualt):
    hist = np.ascontiguousarray(hist, dtype=np.float64)
    n3 = hist[0].size
    out = np.zeros(n3)
    lib().or_gear_sum(n3, int(nualt), _dp(hist), _dp(out))
    return out
