import importlib

import numpy as np


def engine_for(system, **kw):
    abi = importlib.import_module("tinker-gpu_gb300.abi")
    e = abi.Engine(system, **kw)
    e.prepare()
    return e


def rel_err(a, ref):
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = max(np.abs(ref).max(), 1e-30)
    return np.abs(a - ref).max() / scale


def rms_err(a, ref):
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.sqrt(((a - ref) ** 2).sum(axis=-1).mean()))


def cpu(t):
    return t.detach().double().cpu().numpy()


def water_cluster(tg, nmol=40):
    """A non-periodic cut of the 648-atom water box: the first nmol molecules,
    damped Coulomb without cutoff."""
    import dataclasses

    s = tg.systems.make_config("water648")
    na = 3 * nmol
    keep = (s.excl_ik[:, 0] < na) & (s.excl_ik[:, 1] < na)
    c = dataclasses.replace(s, xyz=s.xyz[:na].copy(), types=s.types[:na], frames=s.frames[:na].copy(),
                            pole=s.pole[:na], polarity=s.polarity[:na], thole=s.thole[:na], pdamp=s.pdamp[:na],
                            excl_ik=s.excl_ik[keep], excl_scale=s.excl_scale[keep], box=None, mol_start=None,
                            mol_size=None)
    st = dict(s.settings)
    st.update(use_ewald=0, ewald_cutoff=1.0e9, nfft=(0, 0, 0), aewald=0.0)
    c.settings = st
    return c
