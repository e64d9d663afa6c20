"""Staged real-space kernels (t9gb_pair_staging): each 32-atom block copies
the rows of its neighbouring 32-atom blocks into shared memory with bulk
asynchronous copies and reads its neighbours from there.  The pairs and the
order of the sums are those of the global-memory kernels, so the mutual
field is bit-identical, and so are whole solves at 8 lanes per atom (at 4
lanes the staged preconditioner groups the CG dot products' partial sums by
32 atoms instead of 64, so the dipoles agree to rounding of those sums);
blocks with more neighbouring blocks than the staging capacity (the NaCl box
has some) read from global memory in the same launch.  No copy may time
out."""
import numpy as np
import pytest

from gpu_util import cpu, engine_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,lanes", [("water648", 8), ("water12288", 8), ("water12288", 4), ("nacl23142", 8),
                                        ("nacl23142", 4)])
def test_staged_kernels_bit_identical(gpu_lib, tg, name, lanes):
    s = tg.systems.make_config(name)
    a = engine_for(s)
    a.pair_lanes(lanes)
    a.pair_staging(False)
    b = engine_for(s)
    b.pair_lanes(lanes)
    b.pair_staging(True)
    rng = np.random.default_rng(12)
    u, up = rng.normal(size=(s.n, 3)) * 0.05, rng.normal(size=(s.n, 3)) * 0.05
    for x, y in zip(a.ufield(u, up), b.ufield(u, up)):
        assert np.array_equal(cpu(x), cpu(y))
    ua, pa, _ = a.induce()
    ub, pb, _ = b.induce()
    print(name, lanes, "iterations", a.stats()[0], b.stats()[0])
    assert a.stats()[0] == b.stats()[0]
    if lanes == 8:
        assert np.array_equal(cpu(ua), cpu(ub)) and np.array_equal(cpu(pa), cpu(pb))
    else:
        scale = np.abs(cpu(ua)).max()
        assert np.abs(cpu(ua) - cpu(ub)).max() < 1e-5 * scale and np.abs(cpu(pa) - cpu(pb)).max() < 1e-5 * scale
    assert b.copy_error() == 0


def test_staged_predictor_trajectory(gpu_lib, tg):
    """Graph-captured solves with the ASPC start over a trajectory (list
    reuse and rebuilds): staged and global kernels agree to the bit."""
    s = tg.systems.make_config("water12288")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    a.pair_staging(False)
    b = engine_for(s, predictor=1)
    b.pair_staging(True)
    for k in range(22):
        x = tr.frame(k)
        ua, pa, _ = a.induce_host(x)
        ub, pb, _ = b.induce_host(x)
        assert a.stats()[0] == b.stats()[0], k
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb), k
    assert b.copy_error() == 0
