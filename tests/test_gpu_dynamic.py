"""MD from Tinker files (tinker-gpu_gb300/dynamic.py): the TinkerNIST run of
the reference (test/tinkernist.cpp:195-365) driven from an .xyz, .key, .prm
and the water30 restart written as files, checked on the .arc frames and
.uind dipoles it writes against the reference's saved trajectory and
induced dipoles (every atom)."""
import importlib
import os

import numpy as np
import pytest

import tn_fixture as T
from test_tinkerio import _tinkernist_files

pytestmark = pytest.mark.gpu


def test_dynamic_from_tinker_files(gpu_lib, tmp_path):
    tio = importlib.import_module("tinker-gpu_gb300.tinkerio")
    dyn = importlib.import_module("tinker-gpu_gb300.dynamic")
    d = str(tmp_path)
    _tinkernist_files(d)
    fx = T.load()
    m = fx["meta"]
    tio.write_dyn(os.path.join(d, "nist.dyn"), "AMOEBA Water Box", fx["dyn_x"], fx["dyn_v"], box=tuple(m["box"]))
    out = dyn.run(os.path.join(d, "nist.xyz"), nsteps=2, dt_fs=1000 * m["dt_ps"], save_every=1,
                  dyn_in=os.path.join(d, "nist.dyn"), arc=os.path.join(d, "nist.arc"),
                  uind_out=os.path.join(d, "nist.uind"), dyn_out=os.path.join(d, "out.dyn"))
    assert out["steps"] == 2
    frames = tio.read_xyz(os.path.join(d, "nist.arc"))
    dip = tio.read_xyz(os.path.join(d, "nist.uind"))
    assert len(frames) == 2 and len(dip) == 2
    box = np.asarray(m["box"])
    for k in range(2):
        dx = frames[k].xyz - fx["xyz"][k]
        dx -= box * np.round(dx / box)  # the reference wraps molecules before saving
        du = dip[k].xyz - fx["uind"][k]
        print(f"frame {k + 1}: positions max {np.abs(dx).max():.2e} A, dipoles max {np.abs(du).max():.2e} D")
        assert np.abs(dx).max() < m["md_eps"]["xyz"]
        assert np.abs(du).max() < m["reference_eps"]
    x, v, _, _, b = tio.read_dyn(os.path.join(d, "out.dyn"))
    assert np.allclose(x, out["xyz"], rtol=1e-15) and np.allclose(v, out["vel"], rtol=1e-15)


def test_dynamic_learned_extrapolation(gpu_lib, tmp_path):
    """The same run continued for 40 steps with the learned extrapolation of
    the ASPC ring (dynamic.run(extrapolation=8)): the trajectory stays on the
    plain ASPC one (the solves meet the same 1e-6 D tolerance)."""
    dyn = importlib.import_module("tinker-gpu_gb300.dynamic")
    tio = importlib.import_module("tinker-gpu_gb300.tinkerio")
    d = str(tmp_path)
    _tinkernist_files(d)
    fx = T.load()
    m = fx["meta"]
    tio.write_dyn(os.path.join(d, "nist.dyn"), "AMOEBA Water Box", fx["dyn_x"], fx["dyn_v"], box=tuple(m["box"]))
    kw = dict(nsteps=40, dt_fs=1000 * m["dt_ps"], dyn_in=os.path.join(d, "nist.dyn"))
    a = dyn.run(os.path.join(d, "nist.xyz"), **kw)
    b = dyn.run(os.path.join(d, "nist.xyz"), extrapolation=8, **kw)
    assert a["steps"] == b["steps"] == 40
    dx = np.abs(a["xyz"] - b["xyz"]).max()
    print(f"40 steps: positions differ by {dx:.2e} A")
    assert dx < 3e-5  # measured 3e-6 A: dipoles within the tolerance from different starts
