"""CUDA induce() (PCG) against the FP64 oracle and the reference's known
answers.  Both solves stop at an RMS residual below poleps (1e-6 Debye);
the dipoles must agree to DIPOLE_RMS_DEBYE RMS."""
import numpy as np
import pytest

import lf_fixture as L
from gpu_util import cpu, engine_for, rms_err

pytestmark = pytest.mark.gpu
DIPOLE_RMS_DEBYE = 2.0e-5
DIPOLE_MAX_DEBYE = 2.0e-4
GOLDEN_MARGIN = 1.0e-4


@pytest.mark.parametrize("ewald", [0, 1], ids=["nonewald", "pme"])
def test_localframe_induce(gpu_lib, oracle, tg, ewald):
    s, fx = L.system(ewald)
    e = engine_for(s)
    ud, up, rc = e.induce()
    assert rc == 0
    it, eps, st = e.stats()
    assert eps < s.settings["poleps"] and 3 <= it < 100
    D = tg.units.DEBYE
    ex = L.expected(fx, ewald)["induce"]
    assert np.abs(cpu(ud) * D - ex["ref_ud_debye"]).max() < GOLDEN_MARGIN
    assert np.abs(cpu(up) * D - ex["ref_up_debye"]).max() < GOLDEN_MARGIN
    ou, op, *_ = oracle.OracleSystem(s).induce()
    assert rms_err(cpu(ud) * D, ou * D) < DIPOLE_RMS_DEBYE


@pytest.mark.parametrize("name", ["water648", "nacl23142"])
def test_water_induce(gpu_lib, oracle, tg, name):
    s = tg.systems.make_config(name)
    e = engine_for(s)
    ud, up, rc = e.induce()
    assert rc == 0
    it, eps, st = e.stats()
    ou, op, _, _, oit, oeps = oracle.OracleSystem(s).induce()
    D = tg.units.DEBYE
    print(name, "gpu iters", it, "eps", eps, "oracle iters", oit, "eps", oeps)
    assert eps < 1e-6 and abs(it - oit) <= 2
    assert rms_err(cpu(ud) * D, ou * D) < DIPOLE_RMS_DEBYE
    assert rms_err(cpu(up) * D, op * D) < DIPOLE_RMS_DEBYE
    assert np.abs(cpu(ud) - ou).max() * D < DIPOLE_MAX_DEBYE


def test_induce_host_entry_matches_device_entry(gpu_lib, tg):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    ud, up, _ = e.induce()
    hd, hp, rc = e.induce_host(s.xyz)
    assert rc == 0
    assert np.array_equal(cpu(ud).astype(np.float32), hd.astype(np.float32))


def test_induce_bit_reproducible(gpu_lib, tg):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    a = cpu(e.induce()[0])
    b = cpu(e.induce()[0])
    assert np.array_equal(a, b)


def test_not_converged_status(gpu_lib, tg):
    """politer = 1 forces the reference's non-convergence error path."""
    abi = __import__("importlib").import_module("tinker-gpu_gb300.abi")
    s = tg.systems.make_config("water648")
    e = abi.Engine(s, politer=1)
    e.prepare()
    _, _, rc = e.induce()
    assert rc == abi.T9GB_NOT_CONVERGED


def test_aspc_predictor_trajectory(gpu_lib, oracle, tg):
    """ASPC guess after 16 saved steps: fewer iterations, same answer."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    plain = engine_for(s)
    pred = engine_for(s, predictor=1)
    its_plain, its_pred = [], []
    for step in range(20):
        x = tr.frame(step)
        ud0, _, _ = plain.induce_host(x)
        its_plain.append(plain.stats()[0])
        ud1, _, rc = pred.induce_host(x)
        assert rc == 0
        its_pred.append(pred.stats()[0])
    D = tg.units.DEBYE
    assert rms_err(ud1 * D, ud0 * D) < DIPOLE_RMS_DEBYE
    assert np.mean(its_pred[17:]) < np.mean(its_plain[17:])


def test_graph_matches_stepwise(gpu_lib, tg):
    """The whole-induce CUDA graph (device-side loop) and the host-driven
    loop give bit-identical dipoles and the same iteration count."""
    s = tg.systems.make_config("water648")
    a = engine_for(s)
    b = engine_for(s)
    b.use_graph(False)
    ua, pa, _ = a.induce()
    ub, pb, _ = b.induce()
    assert a.stats()[0] == b.stats()[0]
    assert np.array_equal(cpu(ua), cpu(ub)) and np.array_equal(cpu(pa), cpu(pb))


def test_graph_predictor_steps_match_stepwise(gpu_lib, tg):
    """ASPC bookkeeping lives on the device: graph and stepwise runs agree
    step by step, including after the predictor switches on."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    b = engine_for(s, predictor=1)
    b.use_graph(False)
    for step in range(18):
        x = tr.frame(step)
        ua, _, _ = a.induce_host(x)
        ub, _, _ = b.induce_host(x)
        assert a.stats()[0] == b.stats()[0]
        assert np.array_equal(ua, ub)


def test_gear_predictor_trajectory(gpu_lib, oracle, tg):
    """Gear guess after 6 saved steps: fewer iterations than alpha E, the
    converged answer unchanged; graph and host-driven loops agree."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    plain = engine_for(s)
    gear = engine_for(s, predictor=2)
    step = engine_for(s, predictor=2)
    step.use_graph(False)
    its_plain, its_gear = [], []
    for k in range(12):
        x = tr.frame(k)
        ud0, _, _ = plain.induce_host(x)
        its_plain.append(plain.stats()[0])
        ud1, _, rc = gear.induce_host(x)
        assert rc == 0
        its_gear.append(gear.stats()[0])
        ud2, _, _ = step.induce_host(x)
        assert np.array_equal(ud1, ud2) and gear.stats()[0] == step.stats()[0]
    print("iterations plain", its_plain, "gear", its_gear)
    D = tg.units.DEBYE
    assert rms_err(ud1 * D, ud0 * D) < DIPOLE_RMS_DEBYE
    assert its_gear[:6] == its_plain[:6]
    assert np.mean(its_gear[7:]) < np.mean(its_plain[7:])


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_coordinates_rejected(gpu_lib, tg, bad):
    """A non-finite coordinate is refused before any copy or launch; the
    context keeps working and gives the same dipoles as before."""
    import importlib

    abi = importlib.import_module("tinker-gpu_gb300.abi")
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    ref, _, _ = e.induce_host(s.xyz)
    x = s.xyz.copy()
    x[100, 1] = bad
    with pytest.raises(abi.T9Error) as err:
        e.induce_host(x)
    assert err.value.code == abi.T9GB_BAD_ARG
    again, _, _ = e.induce_host(s.xyz)
    assert np.array_equal(ref, again)


def test_reused_list_keeps_every_pair_within_cutoff(gpu_lib, oracle, tg):
    """Non-Ewald multipoles with a 7 A cutoff, where a pair near the cutoff
    carries kcal/mol: after frames whose motion stays under half the list
    buffer (no rebuild), the energy still matches the oracle, which takes
    every pair within the cutoff at the current positions."""
    s = tg.systems.make_config("water648")
    st = dict(s.settings)
    st.update(use_ewald=0, ewald_cutoff=7.0, nfft=(0, 0, 0), aewald=0.0)
    s.settings = st
    tr = tg.systems.Trajectory(s)
    e = engine_for(s)
    for k in range(0, 31, 5):
        x = tr.frame(k)
        e.set_xyz(x)
        e.mpole_init()
        en, _ = e.empole_energy()
    _, parts = oracle.OracleSystem(s, x).empole_energy()
    eo = parts.sum()
    print("empole", en, "oracle", eo)
    assert abs(en - eo) < 1e-5 * np.abs(parts).sum() + 1e-4


@pytest.mark.parametrize("mask", [0, 3, 7])
def test_pcg_fusion_variants_agree(gpu_lib, tg, mask):
    """Every kernel-fusion setting of the CG iteration solves the same
    system: dipoles equal to rounding of the reordered partial sums, over a
    predictor trajectory (the default fusion is the reference)."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    b = engine_for(s, predictor=1)
    b.pcg_fusion(mask)
    for step in range(18):
        x = tr.frame(step)
        ua, pa, _ = a.induce_host(x)
        ub, pb, _ = b.induce_host(x)
        assert abs(a.stats()[0] - b.stats()[0]) <= 1
        assert np.abs(ua - ub).max() < 1e-6 and np.abs(pa - pb).max() < 1e-6


def test_dipole_grid_range_fallback(gpu_lib, tg):
    """The dipole grids pack d and p as 32-bit fixed point; dipoles large
    enough to reach the packing guard make the context widen the range and
    recompute, so the mutual field stays linear in the dipoles."""
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    rng = np.random.default_rng(3)
    u = rng.normal(scale=0.1, size=(s.n, 3))
    f1, p1 = e.ufield(u, -u)
    big = 1000.0
    f2, p2 = e.ufield(big * u, -big * u)
    f1, p1, f2, p2 = (cpu(t) for t in (f1, p1, f2, p2))
    scale = np.abs(f1).max()
    assert np.abs(f2 / big - f1).max() < 1e-4 * scale
    assert np.abs(p2 / big - p1).max() < 1e-4 * scale
    # the widened context keeps solving
    ud, _, _ = e.induce()
    assert np.isfinite(cpu(ud)).all()


def test_predicted_start_overlap_is_bit_identical(gpu_lib, tg):
    """With the predictor's ring full the guess's field runs beside the
    permanent field (fusion bit 3): the same kernels and sums, so the same
    bits as the start in order; a reset of the predictor (a new neighbour
    order) falls back to the plain start and refills the ring."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    b = engine_for(s, predictor=1)
    b.pcg_fusion(1)
    for step in range(40):
        x = tr.frame(step)
        if step == 24:
            for e in (a, b):
                e.set_xyz(x)
                e.nblist_build()  # new spatial order: the predictor starts over
        ua, pa, _ = a.induce_host(x)
        ub, pb, _ = b.induce_host(x)
        assert a.stats()[0] == b.stats()[0], step
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb), step


@pytest.mark.parametrize("name", ["water648", "water12288"])
def test_side_gather_bit_identical(gpu_lib, tg, name):
    """Fusion bit 5 moves the CG direction's gather behind the transform on
    the reciprocal stream (recip + self stored apart, added to the
    real-space field by the Ap kernel), bit 6 keeps that chain on the main
    stream and the real-space field on the side stream: the same operands in
    the same order, so the same bits as the gather that adds itself, in the
    graph and in the host-driven loop, over a predictor trajectory."""
    s = tg.systems.make_config(name)
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    a.pcg_fusion(25)
    others = []
    for mask, graph in ((25 | 32, True), (25 | 32, False), (25 | 32 | 64, True), (25 | 32 | 64, False)):
        e = engine_for(s, predictor=1)
        e.pcg_fusion(mask)
        e.use_graph(graph)
        others.append(e)
    for step in range(20):
        x = tr.frame(step)
        ua, pa, _ = a.induce_host(x)
        for e in others:
            ub, pb, rc = e.induce_host(x)
            assert rc == 0
            assert a.stats()[0] == e.stats()[0], step
            assert np.array_equal(ua, ub) and np.array_equal(pa, pb), step


@pytest.mark.parametrize("name", ["water648", "water12288"])
def test_programmatic_dependent_launch_bit_identical(gpu_lib, tg, name):
    """Fusion bit 4 launches the PCG loop's kernels as programmatic
    dependents (each waits for its predecessor at its start): the same
    kernels and sums, so the same bits as plain launches, in the graph and
    in the host-driven loop, over a predictor trajectory."""
    s = tg.systems.make_config(name)
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    a.pcg_fusion(9)
    b = engine_for(s, predictor=1)
    b.pcg_fusion(9 | 16)
    c = engine_for(s, predictor=1)
    c.pcg_fusion(9 | 16)
    c.use_graph(False)
    for step in range(20):
        x = tr.frame(step)
        ua, pa, _ = a.induce_host(x)
        ub, pb, rc = b.induce_host(x)
        uc, pc, _ = c.induce_host(x)
        assert rc == 0
        assert a.stats()[0] == b.stats()[0] == c.stats()[0], step
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb), step
        assert np.array_equal(ua, uc) and np.array_equal(pa, pc), step


def test_learned_extrapolation(gpu_lib, oracle, tg):
    """The learned extrapolation of the ASPC ring (online least squares over
    the last 7 frames): the dipoles still meet the oracle's, the start needs
    no more iterations than ASPC's on a trajectory, graph and host-driven
    loop agree bit for bit, and orders outside 2..8 or a context without
    ASPC are rejected."""
    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=1)
    b = engine_for(s, predictor=1)
    b.learn_extrapolation(7)
    c = engine_for(s, predictor=1)
    c.learn_extrapolation(7)
    c.use_graph(False)
    ia, ib, hist = [], [], []
    for step in range(40):
        x = tr.frame(step)
        ua, pa, _ = a.induce_host(x)
        ub, pb, rc = b.induce_host(x)
        uc, pc, _ = c.induce_host(x)
        assert rc == 0
        assert np.array_equal(ub, uc) and np.array_equal(pb, pc), step
        hist.append(np.concatenate([ub, pb]))
        if step >= 24:
            ia.append(a.stats()[0])
            ib.append(b.stats()[0])
    print("iterations ASPC", np.mean(ia), "learned extrapolation", np.mean(ib))
    assert np.mean(ib) <= np.mean(ia)
    # a fit after every solve from the eighth on (7 ring frames and the new
    # one), none rejected; the coefficients reproduce a constant frame
    fb, rb, cb = b.learn_extrapolation_state()
    fc, rc_, cc = c.learn_extrapolation_state()
    assert (fb, rb) == (fc, rc_) == (33, 0)
    assert np.array_equal(cb, cc) and not cb[7:].any()
    assert abs(float(cb.sum()) - 1.0) < 0.05, cb
    # the same online fit restated in FP64 over the returned dipoles (the
    # ring holds exactly those values; the device sums products in FP32 and
    # solves in FP32: 3.6e-4 of the largest coefficient measured)
    from oracle import learn_oracle as LO

    ref, nfit = LO.lx_ring_coefficients(hist, 7)
    err = float(np.abs(cb - ref).max())
    print("ring coefficients", cb[:7], "FP64 restatement", ref[:7], "max error", err)
    assert nfit == 33 and err < 1e-3 * max(1.0, float(np.abs(ref).max()))
    assert a.learn_extrapolation_state()[:2] == (0, 0) and not a.learn_extrapolation_state()[2].any()
    ou, op, *_ = oracle.OracleSystem(s, xyz=tr.frame(39)).induce()
    D = tg.units.DEBYE
    assert rms_err(ub * D, ou * D) < DIPOLE_RMS_DEBYE and rms_err(pb * D, op * D) < DIPOLE_RMS_DEBYE
    abi = gpu_lib
    for bad in (1, 9, -1):
        with pytest.raises(abi.T9Error):
            b.learn_extrapolation(bad)
    d = engine_for(s, predictor=0)
    with pytest.raises(abi.T9Error):
        d.learn_extrapolation(7)


def test_learned_extrapolation_gear(gpu_lib, oracle, tg):
    """The learned extrapolation over Gear's ring of 6 frames (order 5): no
    more iterations than Gear's own start, the oracle's dipoles, coefficients
    as the FP64 restatement fits them; order 6 does not fit in the ring."""
    from oracle import learn_oracle as LO

    s = tg.systems.make_config("water648")
    tr = tg.systems.Trajectory(s)
    a = engine_for(s, predictor=2)
    b = engine_for(s, predictor=2)
    b.learn_extrapolation(5)
    ia, ib, hist = [], [], []
    for step in range(40):
        x = tr.frame(step)
        a.induce_host(x)
        ub, pb, rc = b.induce_host(x)
        assert rc == 0
        hist.append(np.concatenate([ub, pb]))
        if step >= 16:
            ia.append(a.stats()[0])
            ib.append(b.stats()[0])
    print("iterations Gear", np.mean(ia), "learned extrapolation", np.mean(ib))
    assert np.mean(ib) <= np.mean(ia)
    ou, op, *_ = oracle.OracleSystem(s, xyz=tr.frame(39)).induce()
    D = tg.units.DEBYE
    assert rms_err(ub * D, ou * D) < DIPOLE_RMS_DEBYE and rms_err(pb * D, op * D) < DIPOLE_RMS_DEBYE
    fits, rej, cb = b.learn_extrapolation_state()
    ref, nfit = LO.lx_ring_coefficients(hist, 5)
    err = float(np.abs(cb - ref).max())
    print("ring coefficients", cb[:5], "FP64 restatement", ref[:5], "max error", err)
    assert (fits, rej) == (nfit, 0) == (35, 0)
    assert err < 1e-3 * max(1.0, float(np.abs(ref).max()))
    with pytest.raises(gpu_lib.T9Error):
        b.learn_extrapolation(6)
