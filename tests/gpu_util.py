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
