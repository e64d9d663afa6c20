"""Bond, angle and Urey-Bradley terms on the GPU (t9gb_evalence): the
known answers of Tinker9 test/bond.cpp (304-atom protein, anharmonic bonds)
and test/urey.cpp (ten waters), and the 648-atom water box against the FP64
oracle (energy, gradient by central differences, virial)."""
import importlib
import json
import os

import numpy as np
import pytest

from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu
tg = importlib.import_module("tinker-gpu_gb300")
CALC_ALL = 0x070


def placeholder_system(xyz, box=None):
    """Atoms without multipoles or polarizability: only the terms under test."""
    n = len(xyz)
    records = {0: [(0, 0, 0, [0.0] * 10)]}
    s = tg.systems.build_system(xyz, [0] * n, [], records, {0: (0.0, 0.39, ())}, box=box, name="valence")
    st = dict(tg.systems.DEFAULT_SETTINGS)
    st.update(use_ewald=0, ewald_cutoff=1.0e9 if box is None else 7.0, nfft=(0, 0, 0), aewald=0.0)
    s.settings = st
    return s


@pytest.mark.parametrize("term", ["bond", "urey"])
def test_valence_known_answers(gpu_lib, term):
    with open(os.path.join(os.path.dirname(__file__), "golden", "valence.json")) as f:
        d = json.load(f)[term]
    s = placeholder_system(d["xyz"])
    empty = np.zeros((0, 5))
    if term == "bond":
        s.valence = tg.systems.ValenceParams(bonds=np.array(d["bonds"]), angles=empty, ureys=empty,
                                             bond_cubic=d["cubic"], bond_quartic=d["quartic"])
    else:
        s.valence = tg.systems.ValenceParams(bonds=np.zeros((0, 4)), angles=empty, ureys=np.array(d["ureys"]),
                                             urey_cubic=d["cubic"], urey_quartic=d["quartic"])
    e = engine_for(s)
    en, g, w = e.evalence(CALC_ALL)
    ex = d["expected"]
    g = cpu(g)
    print(term, en, ex["energy"], np.abs(g - np.array(ex["gradient"])).max(), np.abs(w - np.array(ex["virial"])).max())
    # the reference test's margins widened to FP32 (its own mixed build uses 0.004 / 0.006 for bonds)
    assert abs(en - ex["energy"]) < 2e-4
    assert np.abs(g - np.array(ex["gradient"])).max() < 4e-3
    assert np.abs(w - np.array(ex["virial"])).max() < 6e-3


def test_water_valence_vs_oracle(gpu_lib, oracle):
    from oracle import mm_oracle

    s = tg.systems.make_config("water648", valence=True)
    v = s.valence
    e = engine_for(s)
    en, g, w = e.evalence(CALC_ALL)

    def f(x):
        return (mm_oracle.bond_energy(x, v.bonds, v.bond_cubic, v.bond_quartic, s.box)
                + mm_oracle.angle_energy(x, v.angles, *v.angle_terms, box=s.box)
                + mm_oracle.urey_energy(x, v.ureys, v.urey_cubic, v.urey_quartic, s.box))

    x = np.asarray(s.xyz, dtype=np.float64)
    eo = f(x)
    print("evalence", en, "oracle", eo)
    assert abs(en - eo) < 1e-5 * abs(eo) + 1e-4
    atoms = list(range(0, 648, 37))
    go = oracle._fd(f, x, atoms, 1e-6)
    d = cpu(g)[atoms] - go
    assert np.abs(d).max() < 1e-3
    wo = oracle._strain_fd(s, lambda s2: f(np.asarray(s2.xyz)), True, 1e-6)
    # FP32 coordinates: 5e-5 of the largest component
    assert np.abs(np.diag(w) - np.diag(wo)).max() < 1e-3 + 5e-5 * np.abs(np.diag(wo)).max()
