"""ctypes binding of the C ABI in include/t9gb.h and a thin Python host API.

The CUDA library (csrc/_build/libt9gb.so) is the only compute path: if it is
missing or cannot load, every entry point here raises; there is no CPU
fallback.  Device buffers are torch CUDA tensors (torch is used for device
memory and streams only).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from .units import DEBYE, ELECTRIC

LIB_PATH = _build.LIB

T9GB_OK, T9GB_NOT_CONVERGED, T9GB_NAN_DETECTED, T9GB_BAD_ARG, T9GB_CUDA_ERR, T9GB_NO_DEVICE, T9GB_NOT_READY = range(7)
T9GB_TOO_LARGE = 7
T9GB_NOALLOC_MAX_ATOMS = 8192

# every symbol include/t9gb.h declares
EXPORTS = [
    "t9gb_create", "t9gb_destroy", "t9gb_status_string", "t9gb_last_error", "t9gb_set_stream", "t9gb_set_topology",
    "t9gb_set_xyz_host", "t9gb_set_xyz_device", "t9gb_nblist_build", "t9gb_mpole_init", "t9gb_dfield", "t9gb_ufield",
    "t9gb_sparse_precond_apply", "t9gb_induce", "t9gb_induce_host", "t9gb_induce_stats", "t9gb_get_udir",
    "t9gb_get_uind", "t9gb_empole_energy", "t9gb_epolar_energy", "t9gb_use_graph", "t9gb_nblist_stats",
    "t9gb_profile_enable", "t9gb_profile_read", "t9gb_profile_name", "t9gb_ufield_noalloc", "t9gb_learn_config",
    "t9gb_learn_policy", "t9gb_learn_reset", "t9gb_learn_stats", "t9gb_learn_get_weights", "t9gb_learn_set_weights",
    "t9gb_learn_eval", "t9gb_learn_adamw", "t9gb_learn_features", "t9gb_empole", "t9gb_epolar", "t9gb_emplar",
    "t9gb_energy_components", "t9gb_pme_own_fft", "t9gb_pair_lanes", "t9gb_force_lanes", "t9gb_set_pcg_fusion",
    "t9gb_set_thole_pairs", "t9gb_set_external_field", "t9gb_set_vdw", "t9gb_ehal", "t9gb_set_valence",
    "t9gb_evalence", "t9gb_md_init", "t9gb_md_run", "t9gb_md_state", "t9gb_md_positions_device", "t9gb_md_stats",
    "t9gb_set_xyz_soa_device", "t9gb_diag_precond_apply", "t9gb_gradient_fixed", "t9gb_pme_fft_cluster",
    "t9gb_copy_error", "t9gb_pair_staging", "t9gb_learn_tensor_path", "t9gb_learn_extrapolation",
    "t9gb_learn_extrapolation_state",
]
CALC_ENERGY, CALC_GRAD, CALC_VIRIAL = 0x010, 0x020, 0x040

LEARN_NFEAT = 32
LEARN_NPARAM = 6792
LEARN_TRAIN, LEARN_USE = 1, 2


class T9Config(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("box", C.c_double * 3),
        ("use_ewald", C.c_int),
        ("aewald", C.c_double),
        ("nfft", C.c_int * 3),
        ("bsorder", C.c_int),
        ("cutoff", C.c_double),
        ("list_buffer", C.c_double),
        ("usolve_cutoff", C.c_double),
        ("pbuffer", C.c_double),
        ("poleps", C.c_double),
        ("politer", C.c_int),
        ("pcgpeek", C.c_double),
        ("udiag", C.c_double),
        ("pcgprec", C.c_int),
        ("pcgguess", C.c_int),
        ("predictor", C.c_int),
        ("electric", C.c_double),
        ("debye", C.c_double),
    ]


class T9Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None


def load(path=None):
    """Load libt9gb.so; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise T9Error(-1, f"CUDA library not built: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    vp, ip, dp, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p
    lib.t9gb_create.argtypes = [C.POINTER(T9Config), C.POINTER(vp)]
    lib.t9gb_destroy.argtypes = [vp]
    lib.t9gb_destroy.restype = None
    lib.t9gb_status_string.argtypes = [C.c_int]
    lib.t9gb_status_string.restype = C.c_char_p
    lib.t9gb_last_error.argtypes = [vp]
    lib.t9gb_last_error.restype = C.c_char_p
    lib.t9gb_set_stream.argtypes = [vp, vp]
    lib.t9gb_set_topology.argtypes = [vp, ip, dp, dp, dp, dp, C.c_int, ip, dp]
    lib.t9gb_set_xyz_host.argtypes = [vp, dp]
    lib.t9gb_set_xyz_device.argtypes = [vp, fp]
    lib.t9gb_nblist_build.argtypes = [vp]
    lib.t9gb_mpole_init.argtypes = [vp]
    lib.t9gb_dfield.argtypes = [vp, fp, fp]
    lib.t9gb_ufield.argtypes = [vp, fp, fp, fp, fp]
    lib.t9gb_sparse_precond_apply.argtypes = [vp, fp, fp, fp, fp]
    lib.t9gb_induce.argtypes = [vp, fp, fp]
    lib.t9gb_induce_host.argtypes = [vp, dp, dp, dp]
    lib.t9gb_induce_stats.argtypes = [vp, ip, dp, ip]
    lib.t9gb_get_udir.argtypes = [vp, fp, fp]
    lib.t9gb_get_uind.argtypes = [vp, fp, fp]
    lib.t9gb_empole_energy.argtypes = [vp, dp, dp]
    lib.t9gb_epolar_energy.argtypes = [vp, dp]
    lib.t9gb_use_graph.argtypes = [vp, C.c_int]
    lib.t9gb_nblist_stats.argtypes = [vp, ip, C.POINTER(C.c_longlong), ip]
    lib.t9gb_profile_enable.argtypes = [vp, C.c_int]
    lib.t9gb_profile_read.argtypes = [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.c_int]
    lib.t9gb_profile_name.argtypes = [C.c_int]
    lib.t9gb_profile_name.restype = C.c_char_p
    lib.t9gb_ufield_noalloc.argtypes = [C.c_int, dp, C.c_double, fp, fp, fp, fp, fp, fp, fp, vp]
    flp = C.POINTER(C.c_float)
    lib.t9gb_learn_config.argtypes = [vp, C.c_int, C.c_double, C.c_double]
    lib.t9gb_learn_reset.argtypes = [vp, C.c_uint]
    lib.t9gb_learn_policy.argtypes = [vp, C.c_int]
    lib.t9gb_learn_stats.argtypes = [vp, ip, dp, dp, dp, ip]
    lib.t9gb_learn_get_weights.argtypes = [vp, flp, C.c_int]
    lib.t9gb_learn_set_weights.argtypes = [vp, flp, C.c_int]
    lib.t9gb_learn_eval.argtypes = [vp, C.c_int, flp, flp, flp, flp, dp]
    lib.t9gb_learn_adamw.argtypes = [vp]
    lib.t9gb_learn_features.argtypes = [vp, fp]
    lib.t9gb_energy_components.argtypes = [vp, dp]
    lib.t9gb_pme_own_fft.argtypes = [vp, C.c_int]
    lib.t9gb_pme_fft_cluster.argtypes = [vp, C.c_int]
    lib.t9gb_copy_error.argtypes = [vp, ip]
    lib.t9gb_pair_staging.argtypes = [vp, C.c_int]
    lib.t9gb_learn_tensor_path.argtypes = [vp, C.c_int]
    lib.t9gb_learn_extrapolation.argtypes = [vp, C.c_int]
    lib.t9gb_learn_extrapolation_state.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                   C.POINTER(C.c_float)]
    lib.t9gb_pair_lanes.argtypes = [vp, C.c_int]
    lib.t9gb_set_pcg_fusion.argtypes = [vp, C.c_int]
    lib.t9gb_force_lanes.argtypes = [vp, C.c_int]
    lib.t9gb_set_thole_pairs.argtypes = [vp, C.c_int, ip, dp]
    lib.t9gb_set_external_field.argtypes = [vp, dp]
    lib.t9gb_set_vdw.argtypes = [vp, C.c_int, ip, dp, dp, dp, ip, C.c_int, ip, dp, C.c_double, C.c_double]
    lib.t9gb_ehal.argtypes = [vp, C.c_int, dp, fp, dp]
    lib.t9gb_set_valence.argtypes = [vp, C.c_int, ip, dp, dp, C.c_double, C.c_double, C.c_int, ip, dp, dp, dp,
                                     C.c_int, ip, dp, dp, C.c_double, C.c_double]
    lib.t9gb_evalence.argtypes = [vp, C.c_int, dp, fp, dp]
    lib.t9gb_md_init.argtypes = [vp, dp, dp, dp]
    lib.t9gb_md_run.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, C.c_ulonglong, dp,
                                dp]
    lib.t9gb_md_state.argtypes = [vp, dp, dp, fp]
    lib.t9gb_md_positions_device.argtypes = [vp, fp]
    lib.t9gb_md_stats.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    lib.t9gb_set_xyz_soa_device.argtypes = [vp, fp, fp, fp]
    lib.t9gb_diag_precond_apply.argtypes = [vp, fp, fp, fp, fp]
    lib.t9gb_gradient_fixed.argtypes = [vp, fp, C.c_int, vp, vp, vp]
    for name in ("t9gb_empole", "t9gb_epolar", "t9gb_emplar"):
        getattr(lib, name).argtypes = [vp, C.c_int, dp, fp, dp]
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_config(system, predictor=0, **over):
    st = dict(system.settings)
    st.update(over)
    cfg = T9Config()
    cfg.n = system.n
    if system.box is not None:
        for d in range(3):
            cfg.box[d] = float(system.box[d])
    cfg.use_ewald = int(st.get("use_ewald", 1))
    cfg.aewald = float(st.get("aewald", 0.0))
    nf = st.get("nfft", (0, 0, 0))
    for d in range(3):
        cfg.nfft[d] = int(nf[d])
    cfg.bsorder = int(st.get("bsorder", 5))
    cfg.cutoff = float(st.get("ewald_cutoff", 1.0e9))
    cfg.list_buffer = float(st.get("list_buffer", 2.0))
    cfg.usolve_cutoff = float(st.get("usolve_cutoff", 4.5))
    cfg.pbuffer = float(st.get("pbuffer", 2.0))
    cfg.poleps = float(st.get("poleps", 1e-6))
    cfg.politer = int(st.get("politer", 100))
    cfg.pcgpeek = float(st.get("pcgpeek", 1.0))
    cfg.udiag = float(st.get("udiag", 2.0))
    cfg.pcgprec = int(st.get("pcgprec", 1))
    cfg.pcgguess = int(st.get("pcgguess", 1))
    cfg.predictor = int(predictor)
    cfg.electric = ELECTRIC
    cfg.debye = DEBYE
    return cfg


class Engine:
    """One library context for one system (mirrors the reference's global
    state for the polarization path)."""

    def __init__(self, system, predictor=0, stream=None, **over):
        import torch

        self.torch = torch
        self.lib = load()
        self.sys = system
        self.n = system.n
        self.cfg = make_config(system, predictor=predictor, **over)
        h = C.c_void_p()
        self._check(self.lib.t9gb_create(C.byref(self.cfg), C.byref(h)), None)
        self.h = h
        s = stream if stream is not None else torch.cuda.current_stream()
        self._check(self.lib.t9gb_set_stream(self.h, C.c_void_p(s.cuda_stream)))
        frames = np.ascontiguousarray(system.frames, dtype=np.int32)
        pole = np.ascontiguousarray(system.pole, dtype=np.float64)
        pol = np.ascontiguousarray(system.polarity, dtype=np.float64)
        thl = np.ascontiguousarray(system.thole, dtype=np.float64)
        pdm = np.ascontiguousarray(system.pdamp, dtype=np.float64)
        eik = np.ascontiguousarray(system.excl_ik, dtype=np.int32).reshape(-1)
        esc = np.ascontiguousarray(system.excl_scale, dtype=np.float64).reshape(-1)
        self._check(
            self.lib.t9gb_set_topology(
                self.h, _ip(frames), _dp(pole), _dp(pol), _dp(thl), _dp(pdm), len(eik) // 2, _ip(eik), _dp(esc)
            )
        )
        if getattr(system, "ptype", None) is not None:
            self.set_thole_pairs(system.ptype, system.thole_table)
        if getattr(system, "exfld", None) is not None:
            self.set_external_field(system.exfld)
        if getattr(system, "vdw", None) is not None:
            self.set_vdw(system.vdw)
        if getattr(system, "valence", None) is not None:
            self.set_valence(system.valence)

    def set_valence(self, v):
        """v: systems.ValenceParams (bonds, angles, Urey-Bradley pairs)."""
        b = np.asarray(v.bonds, dtype=np.float64).reshape(-1, 4)
        a = np.asarray(v.angles, dtype=np.float64).reshape(-1, 5)
        u = np.asarray(v.ureys, dtype=np.float64).reshape(-1, 5)
        keep = (np.ascontiguousarray(b[:, :2], dtype=np.int32), np.ascontiguousarray(b[:, 2]),
                np.ascontiguousarray(b[:, 3]), np.ascontiguousarray(a[:, :3], dtype=np.int32),
                np.ascontiguousarray(a[:, 3]), np.ascontiguousarray(a[:, 4]),
                np.ascontiguousarray(v.angle_terms, dtype=np.float64), np.ascontiguousarray(u[:, :3], dtype=np.int32),
                np.ascontiguousarray(u[:, 3]), np.ascontiguousarray(u[:, 4]))
        self._val_keep = keep
        self._check(self.lib.t9gb_set_valence(
            self.h, len(b), _ip(keep[0]), _dp(keep[1]), _dp(keep[2]), float(v.bond_cubic), float(v.bond_quartic),
            len(a), _ip(keep[3]), _dp(keep[4]), _dp(keep[5]), _dp(keep[6]),
            len(u), _ip(keep[7]), _dp(keep[8]), _dp(keep[9]), float(v.urey_cubic), float(v.urey_quartic)))

    def set_vdw(self, v):
        """v: systems.VdwParams (per-atom types, pair tables, reduction,
        scaled pairs, taper and cutoff), or None to remove the term."""
        if v is None:
            self._check(self.lib.t9gb_set_vdw(self.h, 0, None, None, None, None, None, 0, None, None, 0.0, 0.0))
            return
        vt = np.ascontiguousarray(v.vtype, dtype=np.int32)
        rm = np.ascontiguousarray(v.radmin, dtype=np.float64)
        ep = np.ascontiguousarray(v.epsilon, dtype=np.float64)
        rd = np.ascontiguousarray(v.red, dtype=np.float64)
        pa = np.ascontiguousarray(v.parent, dtype=np.int32)
        ik = np.ascontiguousarray(v.scaled_ik, dtype=np.int32).reshape(-1)
        sv = np.ascontiguousarray(v.scaled_v, dtype=np.float64)
        self._vdw_keep = (vt, rm, ep, rd, pa, ik, sv)
        self._check(self.lib.t9gb_set_vdw(self.h, int(rm.shape[0]), _ip(vt), _dp(rm), _dp(ep), _dp(rd), _ip(pa),
                                          len(sv), _ip(ik), _dp(sv), float(v.taper), float(v.off)))

    def set_external_field(self, field):
        """Uniform external field [3] in e/A^2, or None."""
        if field is None:
            self._check(self.lib.t9gb_set_external_field(self.h, None))
            return
        ef = np.ascontiguousarray(field, dtype=np.float64)
        self._check(self.lib.t9gb_set_external_field(self.h, _dp(ef)))

    def set_thole_pairs(self, ptype, table):
        """Per-type-pair Thole coefficients (ptype [n] 0-based, table [t][t]);
        ptype None restores min(thole_i, thole_k)."""
        if ptype is None:
            self._check(self.lib.t9gb_set_thole_pairs(self.h, 0, None, None))
            return
        pt = np.ascontiguousarray(ptype, dtype=np.int32)
        tb = np.ascontiguousarray(table, dtype=np.float64)
        self._check(self.lib.t9gb_set_thole_pairs(self.h, int(tb.shape[0]), _ip(pt), _dp(tb)))

    def _check(self, rc, h=-1, allow=()):
        if rc == T9GB_OK or rc in allow:
            return rc
        msg = self.lib.t9gb_status_string(rc).decode()
        hh = self.h if h == -1 else h
        if hh:
            msg += ": " + self.lib.t9gb_last_error(hh).decode()
        raise T9Error(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.t9gb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state ----
    def set_xyz(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self._check(self.lib.t9gb_set_xyz_host(self.h, _dp(xyz)))

    def set_xyz_device(self, xyz_t):
        self._check(self.lib.t9gb_set_xyz_device(self.h, C.c_void_p(xyz_t.data_ptr())))

    def nblist_build(self):
        self._check(self.lib.t9gb_nblist_build(self.h))

    def mpole_init(self):
        self._check(self.lib.t9gb_mpole_init(self.h))

    def prepare(self, xyz=None):
        self.set_xyz(self.sys.xyz if xyz is None else xyz)
        self.nblist_build()
        self.mpole_init()

    # ---- fields ----
    def _empty3(self):
        return self.torch.zeros((self.n, 3), dtype=self.torch.float32, device="cuda")

    def dfield(self):
        f, fp = self._empty3(), self._empty3()
        self._check(self.lib.t9gb_dfield(self.h, C.c_void_p(f.data_ptr()), C.c_void_p(fp.data_ptr())))
        return f, fp

    def ufield(self, uind, uinp):
        t = self.torch
        ud = t.as_tensor(np.asarray(uind, dtype=np.float32), device="cuda").contiguous()
        up = t.as_tensor(np.asarray(uinp, dtype=np.float32), device="cuda").contiguous()
        f, fp = self._empty3(), self._empty3()
        self._check(
            self.lib.t9gb_ufield(
                self.h, C.c_void_p(ud.data_ptr()), C.c_void_p(up.data_ptr()), C.c_void_p(f.data_ptr()),
                C.c_void_p(fp.data_ptr()),
            )
        )
        return f, fp

    def diag_precond(self, rsd, rsdp):
        t = self.torch
        r = t.as_tensor(np.asarray(rsd, dtype=np.float32), device="cuda").contiguous()
        rp = t.as_tensor(np.asarray(rsdp, dtype=np.float32), device="cuda").contiguous()
        z, zp = self._empty3(), self._empty3()
        self._check(
            self.lib.t9gb_diag_precond_apply(
                self.h, C.c_void_p(r.data_ptr()), C.c_void_p(rp.data_ptr()), C.c_void_p(z.data_ptr()),
                C.c_void_p(zp.data_ptr()),
            )
        )
        return z, zp

    def gradient_fixed(self, grad, accumulate=None):
        """Float gradient [n][3] (device) -> the reference's fixed-point
        gx, gy, gz (int64 device tensors, two's-complement u64 words)."""
        t = self.torch
        out = accumulate if accumulate is not None else [t.zeros(self.n, dtype=t.int64, device="cuda")
                                                          for _ in range(3)]
        self._check(self.lib.t9gb_gradient_fixed(self.h, C.c_void_p(grad.data_ptr()), 1 if accumulate is not None else 0,
                                                 *[C.c_void_p(o.data_ptr()) for o in out]))
        return out

    def sparse_precond(self, rsd, rsdp):
        t = self.torch
        r = t.as_tensor(np.asarray(rsd, dtype=np.float32), device="cuda").contiguous()
        rp = t.as_tensor(np.asarray(rsdp, dtype=np.float32), device="cuda").contiguous()
        z, zp = self._empty3(), self._empty3()
        self._check(
            self.lib.t9gb_sparse_precond_apply(
                self.h, C.c_void_p(r.data_ptr()), C.c_void_p(rp.data_ptr()), C.c_void_p(z.data_ptr()),
                C.c_void_p(zp.data_ptr()),
            )
        )
        return z, zp

    def induce(self, out=None):
        ud, up = (self._empty3(), self._empty3()) if out is None else out
        rc = self.lib.t9gb_induce(self.h, C.c_void_p(ud.data_ptr()), C.c_void_p(up.data_ptr()))
        self._check(rc, allow=(T9GB_NOT_CONVERGED, T9GB_NAN_DETECTED))
        return ud, up, rc

    def induce_host(self, xyz, uind=None, uinp=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        ud = np.zeros((self.n, 3)) if uind is None else uind
        up = np.zeros((self.n, 3)) if uinp is None else uinp
        rc = self.lib.t9gb_induce_host(self.h, _dp(xyz), _dp(ud), _dp(up))
        self._check(rc, allow=(T9GB_NOT_CONVERGED, T9GB_NAN_DETECTED))
        return ud, up, rc

    def stats(self):
        it, eps, st = C.c_int(), C.c_double(), C.c_int()
        self.lib.t9gb_induce_stats(self.h, C.byref(it), C.byref(eps), C.byref(st))
        return it.value, eps.value, st.value

    def empole_energy(self):
        """(total, [real, recip, self]) permanent-multipole energy, kcal/mol."""
        e = C.c_double()
        parts = np.zeros(3)
        self._check(self.lib.t9gb_empole_energy(self.h, C.byref(e), _dp(parts)))
        return e.value, parts

    def epolar_energy(self):
        """Polarization energy (dot-product form) of the last induce(), kcal/mol."""
        e = C.c_double()
        self._check(self.lib.t9gb_epolar_energy(self.h, C.byref(e)))
        return e.value

    def pme_own_fft(self, enable=True):
        """Fused power-of-two FFT (default where supported) or cuFFT."""
        self._check(self.lib.t9gb_pme_own_fft(self.h, 1 if enable else 0))

    def fft_cluster(self, ctas=4):
        """CTAs per z plane in the fused transform's plane passes (0: one)."""
        self._check(self.lib.t9gb_pme_fft_cluster(self.h, int(ctas)))

    def pair_staging(self, enable=True):
        """Staged (shared-memory) or global-memory rows in the field and
        preconditioner pair kernels."""
        self._check(self.lib.t9gb_pair_staging(self.h, 1 if enable else 0))

    def copy_error(self):
        """Bit 0: a pair-kernel staging copy, bit 1: a transform slab copy
        timed out (0 in normal operation)."""
        f = C.c_int()
        self._check(self.lib.t9gb_copy_error(self.h, C.byref(f)))
        return f.value

    def pair_lanes(self, lanes=16):
        self._check(self.lib.t9gb_pair_lanes(self.h, int(lanes)))

    def force_lanes(self, lanes=4):
        self._check(self.lib.t9gb_force_lanes(self.h, int(lanes)))

    def pcg_fusion(self, mask=121):
        """Fusion and overlap of the CG solve (bit 0 preconditioner + dots,
        bit 1 direction formed by its readers, bit 2 Ap fused into the gather,
        bit 3 the predicted guess's field beside the permanent field, bit 4
        programmatic dependent launch of the loop's kernels)."""
        self._check(self.lib.t9gb_set_pcg_fusion(self.h, int(mask)))

    def use_graph(self, enable=True):
        self._check(self.lib.t9gb_use_graph(self.h, 1 if enable else 0))

    def list_stats(self):
        a, b, c = C.c_int(), C.c_longlong(), C.c_int()
        self._check(self.lib.t9gb_nblist_stats(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"capacity": a.value, "entries": b.value, "scaled_pairs": c.value}

    def profile(self, enable=True):
        self._check(self.lib.t9gb_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self, reset=True):
        """{category: (total_ms, launches)} accumulated since the last reset."""
        out = {}
        for c in range(10):
            ms, cnt = C.c_double(), C.c_longlong()
            self._check(self.lib.t9gb_profile_read(self.h, c, C.byref(ms), C.byref(cnt), 1 if reset else 0))
            out[self.lib.t9gb_profile_name(c).decode()] = (ms.value, cnt.value)
        return out

    def udir(self):
        f, fp = self._empty3(), self._empty3()
        self._check(self.lib.t9gb_get_udir(self.h, C.c_void_p(f.data_ptr()), C.c_void_p(fp.data_ptr())))
        return f, fp

    def uind(self):
        """Induced dipoles (d, p) of the last solve, [n][3] CUDA tensors, e A."""
        f, fp = self._empty3(), self._empty3()
        self._check(self.lib.t9gb_get_uind(self.h, C.c_void_p(f.data_ptr()), C.c_void_p(fp.data_ptr())))
        return f, fp

    # ---- learned initial guess ----
    def learn_config(self, mode, lr=1e-3, weight_decay=1e-2):
        """mode: LEARN_TRAIN (1) train after each solve, LEARN_USE (2) start from
        the learned guess with the residual fallback, 3 both, 0 off."""
        self._check(self.lib.t9gb_learn_config(self.h, int(mode), float(lr), float(weight_decay)))

    def learn_reset(self, seed=1):
        self._check(self.lib.t9gb_learn_reset(self.h, int(seed)))

    def learn_policy(self, probe_every=1):
        self._check(self.lib.t9gb_learn_policy(self.h, int(probe_every)))

    def learn_stats(self):
        """(choice bits, eps0 plain, eps0 learned, loss, compared) of the last solve."""
        ch, a, b, l, cmp_ = C.c_int(), C.c_double(), C.c_double(), C.c_double(), C.c_int()
        self._check(self.lib.t9gb_learn_stats(self.h, C.byref(ch), C.byref(a), C.byref(b), C.byref(l),
                                              C.byref(cmp_)))
        return ch.value, a.value, b.value, l.value, cmp_.value

    def learn_weights(self, w=None):
        """Returns the FP32 master weights; sets them first when w is given."""
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float32)
            self._check(self.lib.t9gb_learn_set_weights(self.h, _fp(w), w.size))
        out = np.zeros(LEARN_NPARAM, dtype=np.float32)
        self._check(self.lib.t9gb_learn_get_weights(self.h, _fp(out), LEARN_NPARAM))
        return out

    def learn_eval(self, x, t):
        """Forward + backward on host rows: returns (y [rows][3], grad, loss)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        rows = x.shape[0]
        y = np.zeros((rows, 3), dtype=np.float32)
        g = np.zeros(LEARN_NPARAM, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.t9gb_learn_eval(self.h, rows, _fp(x), _fp(t), _fp(y), _fp(g), C.byref(loss)))
        return y, g, loss.value

    def learn_tensor_path(self, path=1):
        """0: mma.sync GEMMs; 1: the fused tcgen05 forward pass."""
        self._check(self.lib.t9gb_learn_tensor_path(self.h, int(path)))

    def learn_extrapolation(self, order=8):
        """Learned extrapolation of the predictor ring over `order` frames (2-8 with ASPC,
        2-5 with Gear); 0 restores the predictor's own coefficients."""
        self._check(self.lib.t9gb_learn_extrapolation(self.h, int(order)))

    def learn_extrapolation_state(self):
        """(fits, rejected fits, the 16 ring coefficients by frame age) after the last solve."""
        fits, rej, cf = C.c_int(), C.c_int(), (C.c_float * 16)()
        self._check(self.lib.t9gb_learn_extrapolation_state(self.h, C.byref(fits), C.byref(rej), cf))
        return fits.value, rej.value, np.array(cf[:], dtype=np.float32)

    def learn_adamw(self):
        self._check(self.lib.t9gb_learn_adamw(self.h))

    def learn_features(self):
        """Raw features of the last solve, [2n][32] (d rows then p rows)."""
        out = self.torch.zeros((2 * self.n, LEARN_NFEAT), dtype=self.torch.float32, device="cuda")
        self._check(self.lib.t9gb_learn_features(self.h, C.c_void_p(out.data_ptr())))
        self.torch.cuda.synchronize()
        return out.cpu().numpy()

    # ---- energies and gradients (calc flags of the reference) ----
    def _eg(self, fn, vers):
        e = C.c_double()
        g = self._empty3() if vers & CALC_GRAD else None
        v = np.zeros(9)
        rc = fn(self.h, int(vers), C.byref(e), C.c_void_p(g.data_ptr()) if g is not None else None,
                _dp(v) if vers & CALC_VIRIAL else None)
        self._check(rc, allow=(T9GB_NOT_CONVERGED,))
        if vers & CALC_VIRIAL:
            return e.value, g, v.reshape(3, 3)
        return e.value, g

    # ---- molecular dynamics ----
    def md_init(self, xyz, mass, vel=None):
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        m = np.ascontiguousarray(mass, dtype=np.float64)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        self._check(self.lib.t9gb_md_init(self.h, _dp(x), _dp(m), None if v is None else _dp(v)))

    def md_run(self, nsteps, dt_ps=0.001, thermostat=0, kelvin=298.0, tau_ps=0.1, nfree=0, seed=1):
        """Returns (kinetic energy kcal/mol, temperature K, status)."""
        ek, t = C.c_double(), C.c_double()
        rc = self.lib.t9gb_md_run(self.h, int(nsteps), float(dt_ps), int(thermostat), float(kelvin), float(tau_ps),
                                  int(nfree), int(seed), C.byref(ek), C.byref(t))
        self._check(rc, allow=(T9GB_NOT_CONVERGED,))
        return ek.value, t.value, rc

    def md_state(self):
        """(positions, velocities, gradient) of the trajectory."""
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        g = self._empty3()
        self._check(self.lib.t9gb_md_state(self.h, _dp(x), _dp(v), C.c_void_p(g.data_ptr())))
        return x, v, g

    def md_positions_device(self, out):
        """Current positions into a float32 CUDA tensor [n][3], in stream order."""
        if not (out.is_cuda and out.dtype == self.torch.float32 and out.is_contiguous()
                and tuple(out.shape) == (self.n, 3)):
            raise ValueError("md_positions_device: want a contiguous float32 CUDA tensor [n][3]")
        self._check(self.lib.t9gb_md_positions_device(self.h, C.c_void_p(out.data_ptr())))

    def md_stats(self):
        """(steps, PCG iterations) since md_init."""
        st, it = C.c_longlong(), C.c_longlong()
        self._check(self.lib.t9gb_md_stats(self.h, C.byref(st), C.byref(it)))
        return st.value, it.value

    def evalence(self, vers=CALC_ENERGY | CALC_GRAD):
        """Bond + angle + Urey-Bradley: (energy, gradient[, virial])."""
        return self._eg(self.lib.t9gb_evalence, vers)

    def ehal(self, vers=CALC_ENERGY | CALC_GRAD):
        """Buffered 14-7 van der Waals: (energy, gradient) or with CALC_VIRIAL
        (energy, gradient, virial)."""
        return self._eg(self.lib.t9gb_ehal, vers)

    def energy_components(self):
        """[multipole real, recip, self, polarization] of the last energy evaluation."""
        out = np.zeros(4)
        self._check(self.lib.t9gb_energy_components(self.h, _dp(out)))
        return out

    def empole(self, vers=CALC_ENERGY | CALC_GRAD):
        """(energy, gradient [n][3] device) of the permanent multipoles."""
        return self._eg(self.lib.t9gb_empole, vers)

    def epolar(self, vers=CALC_ENERGY | CALC_GRAD):
        """Solves induce(), then (energy, gradient) of the polarization."""
        return self._eg(self.lib.t9gb_epolar, vers)

    def emplar(self, vers=CALC_ENERGY | CALC_GRAD):
        """Both terms in one pass: (energy, gradient)."""
        return self._eg(self.lib.t9gb_emplar, vers)
