"""Buffered 14-7 van der Waals on the GPU (t9gb_ehal): the NaCl-1 known
answers of Tinker9 test/nacl.cpp, and the 648-atom water box with reduced
hydrogen sites against the FP64 oracle (energy, gradient by central
differences, virial diagonal by strain differences)."""
import numpy as np
import pytest

import nacl_fixture as N
from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu

CALC_ALL = 0x070
HAL_TITLES = ["- ehal -- no switch", "- ehal -- switch, near cut", "- ehal -- switch, near off"]


@pytest.mark.parametrize("title", HAL_TITLES)
def test_nacl_hal_known_answers(gpu_lib, title):
    s, ex = N.hal_system(title)
    e = engine_for(s)
    en, g, w = e.ehal(CALC_ALL)
    g = cpu(g)
    print(title, en, g.tolist(), w.tolist())
    # the reference's 1e-3 margin; FP32 pair arithmetic
    assert abs(en - ex["ref_eng"]) < 1e-3
    assert np.abs(g - np.array(ex["ref_grad"])).max() < 1e-3
    assert np.abs(w - np.array(ex["ref_v"])).max() < 2e-3


def test_water_hal_vs_oracle(gpu_lib, oracle, tg):
    from oracle import mm_oracle

    s = tg.systems.make_config("water648", vdw=True)
    e = engine_for(s)
    en, g, w = e.ehal(CALC_ALL)
    eo = mm_oracle.hal_energy(s)
    print("ehal", en, "oracle", eo)
    assert abs(en - eo) < 2e-5 * abs(eo) + 1e-4
    atoms = [0, 1, 2, 100, 101, 102, 300, 647]
    go = oracle._fd(lambda x: mm_oracle.hal_energy(s, x), np.asarray(s.xyz, dtype=np.float64), atoms, 1e-5)
    d = cpu(g)[atoms] - go
    print("gradient max err", np.abs(d).max(), "max |g|", np.abs(go).max())
    assert np.abs(d).max() < 2e-4
    wo = oracle._strain_fd(s, lambda s2: mm_oracle.hal_energy(s2), True, 1e-6)
    print("virial", np.diag(w), np.diag(wo))
    assert np.abs(np.diag(w) - np.diag(wo)).max() < 2e-3 + 2e-5 * np.abs(np.diag(wo)).max()


def test_vdw_leaves_the_dipoles(gpu_lib, tg):
    """The larger stored list (9 A van der Waals cutoff) filters to the same
    pairs for the fields: the same dipoles within FP32 summation order."""
    a = engine_for(tg.systems.make_config("water648"))
    b = engine_for(tg.systems.make_config("water648", vdw=True))
    ua, pa, _ = a.induce()
    ub, pb, _ = b.induce()
    assert np.abs(cpu(ua) - cpu(ub)).max() < 1e-6 and np.abs(cpu(pa) - cpu(pb)).max() < 1e-6
