"""Uniform external field (t9gb_set_external_field) on the GPU against the
known answers of Tinker9 test/extfield.cpp: multipole, polarization and
combined energy, gradient and full virial; and a field switched on, off and
on again between solves of one context."""
import numpy as np
import pytest

import ef_fixture as F
from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu

CALC_ALL = 0x070


@pytest.mark.parametrize("term", ["mpole", "polar", "mplar"])
def test_extfield_known_answers(gpu_lib, term):
    s, fx = F.system()
    ex, eps = fx["expected"][term], fx["eps"]
    e = engine_for(s)
    fn = {"mpole": e.empole, "polar": e.epolar, "mplar": e.emplar}[term]
    en, g, w = fn(CALC_ALL)
    g = cpu(g)
    print(term, en, np.abs(g - np.array(ex["gradient"])).max(), np.abs(w - np.array(ex["virial"])).max())
    assert abs(en - ex["energy"]) < eps["energy"]
    assert np.abs(g - np.array(ex["gradient"])).max() < eps["gradient"]
    assert np.abs(w - np.array(ex["virial"])).max() < eps["virial"]


def test_field_switches_between_solves(gpu_lib):
    s, _ = F.system()
    e = engine_for(s)
    on = e.induce_host(s.xyz)[0]
    e.set_external_field(None)
    off = e.induce_host(s.xyz)[0]
    e.set_external_field(s.exfld)
    again = e.induce_host(s.xyz)[0]
    s.exfld = None
    ref_off = engine_for(s).induce_host(s.xyz)[0]
    assert np.abs(on - off).max() > 1e-3
    assert np.array_equal(on, again) and np.array_equal(off, ref_off)
