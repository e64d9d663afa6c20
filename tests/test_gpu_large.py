"""The 98,304-atom water box (PME grid 128^3), where an FP64 oracle solve is
too slow for a test.  Size-independent properties instead: convergence to the
RMS threshold, bit-identical graph and host-driven solves, the same mean
induced dipole as the 12,288-atom box of the same density, and fewer
iterations once the ASPC predictor has its 16 frames."""
import numpy as np
import pytest

from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(tg):
    return tg.systems.make_config("water98304")


def _mean_dipole(u):
    return float(np.linalg.norm(u, axis=1).mean())


def test_large_box_converges_and_graph_matches_stepwise(gpu_lib, tg, big):
    a = engine_for(big)
    b = engine_for(big)
    b.use_graph(False)
    ua, pa, rc = a.induce()
    ub, pb, _ = b.induce()
    it, eps, st = a.stats()
    assert rc == 0 and st == 0 and eps < 1e-6 and it < 40
    assert b.stats()[0] == it
    assert np.array_equal(cpu(ua), cpu(ub)) and np.array_equal(cpu(pa), cpu(pb))
    # eight times the molecules of water12288 in a box twice as wide
    small = engine_for(tg.systems.make_config("water12288"))
    us, _, _ = small.induce()
    m_big, m_small = _mean_dipole(cpu(ua)), _mean_dipole(cpu(us))
    print(f"mean |u_d| water98304 {m_big:.5f}, water12288 {m_small:.5f} e A; {it} iterations")
    assert abs(m_big - m_small) < 0.05 * m_small


def test_large_box_predictor_trajectory(gpu_lib, tg, big):
    traj = tg.systems.Trajectory(big)
    e = engine_for(big, predictor=1)
    its = []
    for k in range(20):
        _, _, rc = e.induce_host(traj.frame(k))
        it, eps, st = e.stats()
        assert rc == 0 and st == 0 and eps < 1e-6
        its.append(it)
    print("iterations", its)
    # alpha E starts for the first 16 frames, ASPC extrapolation afterwards
    assert np.mean(its[17:]) < np.mean(its[:16])
