"""ctypes front end of the reference-code harness oracle/_ref/libt9ref.so
(oracle/ref_harness.cpp: the reference's own pair, frame and B-spline
routines compiled from its source in double precision).

TEST INFRASTRUCTURE ONLY: used by tests/ to check the FP64 oracle against
the reference's own arithmetic.  available() is False where the reference
checkout is absent and the library was not built.
"""
import ctypes as C

import numpy as np

from . import build_ref


class RefSystem(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("x", C.POINTER(C.c_double)),
        ("y", C.POINTER(C.c_double)),
        ("z", C.POINTER(C.c_double)),
        ("rpole", C.POINTER(C.c_double)),
        ("pdamp", C.POINTER(C.c_double)),
        ("thole", C.POINTER(C.c_double)),
        ("nexcl", C.c_int),
        ("excl_ik", C.POINTER(C.c_int)),
        ("excl_scale", C.POINTER(C.c_double)),
        ("periodic", C.c_int),
        ("box", C.c_double * 3),
        ("use_ewald", C.c_int),
        ("aewald", C.c_double),
        ("cutoff", C.c_double),
        ("electric", C.c_double),
    ]


_lib = None


def available():
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            return None
        L = C.CDLL(path)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.ref_rotpole.argtypes = [C.c_int, ip, dp, dp, dp, dp, dp]
        L.ref_dfield_real.argtypes = [C.POINTER(RefSystem), dp, dp]
        L.ref_ufield_real.argtypes = [C.POINTER(RefSystem), dp, dp, dp, dp]
        L.ref_empole_real.argtypes = [C.POINTER(RefSystem)]
        L.ref_empole_real.restype = C.c_double
        L.ref_bsplgen.argtypes = [C.c_double, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def rotpole(system, xyz=None):
    xyz = np.asarray(system.xyz if xyz is None else xyz, dtype=np.float64)
    x, y, z = [np.ascontiguousarray(xyz[:, d]) for d in range(3)]
    fr = np.ascontiguousarray(system.frames, dtype=np.int32)
    pole = np.ascontiguousarray(system.pole, dtype=np.float64)
    out = np.zeros((system.n, 10))
    lib().ref_rotpole(system.n, fr.ctypes.data_as(C.POINTER(C.c_int)), _dp(pole), _dp(x), _dp(y), _dp(z), _dp(out))
    return out


class RefHarness:
    """The reference's real-space pair sums on one system (global-frame
    multipoles from the reference's own rotpole)."""

    def __init__(self, system, use_ewald=None, cutoff=None, electric=None):
        st = system.settings
        xyz = np.asarray(system.xyz, dtype=np.float64)
        self.x, self.y, self.z = [np.ascontiguousarray(xyz[:, d]) for d in range(3)]
        self.rpole = rotpole(system)
        self.pdamp = np.ascontiguousarray(system.pdamp, dtype=np.float64)
        self.thole = np.ascontiguousarray(system.thole, dtype=np.float64)
        self.eik = np.ascontiguousarray(system.excl_ik, dtype=np.int32).reshape(-1)
        self.esc = np.ascontiguousarray(system.excl_scale, dtype=np.float64).reshape(-1)
        s = RefSystem()
        s.n = system.n
        s.x, s.y, s.z = _dp(self.x), _dp(self.y), _dp(self.z)
        s.rpole, s.pdamp, s.thole = _dp(self.rpole), _dp(self.pdamp), _dp(self.thole)
        s.nexcl = len(self.eik) // 2
        s.excl_ik = self.eik.ctypes.data_as(C.POINTER(C.c_int))
        s.excl_scale = _dp(self.esc)
        s.periodic = 1 if system.box is not None else 0
        if system.box is not None:
            for d in range(3):
                s.box[d] = float(system.box[d])
        s.use_ewald = int(st.get("use_ewald", 1) if use_ewald is None else use_ewald)
        s.aewald = float(st.get("aewald", 0.0)) if s.use_ewald else 0.0
        s.cutoff = float(st.get("ewald_cutoff", 1.0e9) if cutoff is None else cutoff)
        if electric is None:
            electric = __import__("importlib").import_module("tinker-gpu_gb300.units").ELECTRIC
        s.electric = float(electric)
        self.s = s
        self.n = system.n

    def dfield(self):
        f, fp = np.zeros((self.n, 3)), np.zeros((self.n, 3))
        lib().ref_dfield_real(C.byref(self.s), _dp(f), _dp(fp))
        return f, fp

    def ufield(self, uind, uinp):
        ud = np.ascontiguousarray(uind, dtype=np.float64)
        up = np.ascontiguousarray(uinp, dtype=np.float64)
        f, fp = np.zeros((self.n, 3)), np.zeros((self.n, 3))
        lib().ref_ufield_real(C.byref(self.s), _dp(ud), _dp(up), _dp(f), _dp(fp))
        return f, fp

    def empole(self):
        return lib().ref_empole_real(C.byref(self.s))


def bsplgen(w):
    th = np.zeros(20)
    lib().ref_bsplgen(float(w), _dp(th))
    return th.reshape(5, 4)
