"""Per-type-pair Thole coefficients (t9gb_set_thole_pairs) on the GPU: the
Na+/Cl- known answers of Tinker9 test/polpair.cpp (energy, gradient, full
virial; Ewald and non-Ewald), and a water box whose table equals
min(thole_i, thole_k) giving the same bits as no table."""
import numpy as np
import pytest

import pp_fixture as P
from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu

CALC_ALL = 0x070


@pytest.mark.parametrize("ewald", [1, 0], ids=["ewald", "nonewald"])
def test_polpair_known_answers(gpu_lib, ewald):
    s, ex, eps = P.system(ewald)
    e = engine_for(s)
    en, g, w = e.emplar(CALC_ALL)
    g = cpu(g)
    print(en, g.tolist(), w.tolist())
    assert abs(en - ex["energy"]) < eps["energy"]
    assert np.abs(g - np.array(ex["gradient"])).max() < eps["gradient"]
    assert np.abs(w - np.array(ex["virial"])).max() < eps["virial"]


def test_default_table_matches_min_rule(gpu_lib, tg):
    s = tg.systems.make_config("water648")
    a = engine_for(s)
    ua, pa, _ = a.induce()
    ea, ga = a.emplar()
    polar = {int(t): (0.0, float(s.thole[np.nonzero(s.types == t)[0][0]]), ()) for t in np.unique(s.types)}
    s.ptype, s.thole_table = P.thole_pairs([int(t) for t in s.types], polar, [])
    b = engine_for(s)
    ub, pb, _ = b.induce()
    eb, gb = b.emplar()
    assert np.array_equal(cpu(ua), cpu(ub)) and np.array_equal(cpu(pa), cpu(pb))
    assert ea == eb and np.array_equal(cpu(ga), cpu(gb))
