"""Learned initial guess on the GPU: descriptors, BF16 tensor-core network
gradients and AdamW against the CPU oracle, the residual-based fallback, graph
vs stepwise determinism, and the gain of the trained network over the plain
(alpha E) guess on a water trajectory."""
import numpy as np
import pytest

from gpu_util import cpu, engine_for, rms_err

pytestmark = pytest.mark.gpu

FEATURE_TOL = 5e-4     # max |gpu - oracle| per column / max |oracle| of that column
NET_TOL = 2e-3         # ||gpu - oracle(bf16 emulated)|| / ||oracle||
NET_TOL_FP64 = 3e-2    # ||gpu - oracle(fp64)|| / ||oracle||: the BF16 error itself
DIPOLE_RMS_DEBYE = 2.0e-5


@pytest.fixture(scope="module")
def LO():
    from oracle import learn_oracle

    return learn_oracle


def test_features_match_oracle(gpu_lib, oracle, tg, LO):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    e.learn_config(1)
    e.induce()
    X = e.learn_features()
    fd, fp = oracle.OracleSystem(s).dfield()
    Xo = LO.features(s, s.xyz, fd, fp, oracle.frames(s))
    scale = np.maximum(np.abs(Xo).max(axis=0), 1e-12)
    err = (np.abs(X - Xo).max(axis=0) / scale)
    print("worst feature column", int(err.argmax()), float(err.max()))
    assert err.max() < FEATURE_TOL


def test_network_gradient_matches_oracle(gpu_lib, tg, LO):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    e.learn_reset(seed=7)
    w = e.learn_weights().astype(np.float64)
    rng = np.random.default_rng(8)
    rows = 1000
    x = rng.normal(size=(rows, 32)).astype(np.float32)
    t = rng.normal(size=(rows, 3)).astype(np.float32)
    y, g, loss = e.learn_eval(x, t)
    yo, lo, go = LO.loss_grad(w, x.astype(np.float64), t.astype(np.float64), bf=True)
    _, _, g64 = LO.loss_grad(w, x.astype(np.float64), t.astype(np.float64), bf=False)
    assert np.linalg.norm(y - yo) < NET_TOL * np.linalg.norm(yo)
    assert abs(loss - lo) < NET_TOL * lo
    assert np.linalg.norm(g - go) < NET_TOL * np.linalg.norm(go)
    assert np.linalg.norm(g - g64) < NET_TOL_FP64 * np.linalg.norm(g64)
    for name, (a, b) in zip(["W1", "b1", "W2", "b2", "W3", "b3"], zip(LO.unpack(g).values(), LO.unpack(go).values())):
        assert np.linalg.norm(a - b) <= NET_TOL * np.linalg.norm(b) + 1e-9, name
    # columns 3-7 of the output layer are padding
    assert np.all(LO.unpack(g)["W3"][:, 3:] == 0) and np.all(LO.unpack(g)["b3"][3:] == 0)


def test_adamw_matches_oracle(gpu_lib, tg, LO):
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    e.learn_config(0, lr=1e-3, weight_decay=1e-2)
    e.learn_reset(seed=9)
    w0 = e.learn_weights().astype(np.float64)
    rng = np.random.default_rng(10)
    x = rng.normal(size=(300, 32)).astype(np.float32)
    t = rng.normal(size=(300, 3)).astype(np.float32)
    m = np.zeros_like(w0)
    v = np.zeros_like(w0)
    w_ref = w0.copy()
    for step in range(1, 4):
        _, g, _ = e.learn_eval(x, t)
        e.learn_adamw()
        w_ref, m, v = LO.adamw(w_ref, g.astype(np.float64), m, v, step, lr=1e-3, wd=1e-2)
        w = e.learn_weights().astype(np.float64)
        assert np.abs(w - w_ref).max() < 2e-6 * max(1.0, np.abs(w_ref).max())
        w_ref = w  # continue from the device state (FP32 master weights)
    assert np.all(w[LO.trainable_mask() == 0] == 0)


def _run(e, traj, steps, mode, record=None):
    e.learn_config(mode)
    for k in steps:
        e.induce_host(traj.frame(k))
        if record is not None:
            it, eps, st = e.stats()
            record.append((it, eps, st) + e.learn_stats())


def test_learned_guess_cuts_iterations(gpu_lib, oracle, tg):
    """Train online on 300 frames, then solve 20 new frames twice: with the
    plain alpha E guess and from the learned guess (no predictor history)."""
    s = tg.systems.make_config("water648")
    traj = tg.systems.Trajectory(s)
    e = engine_for(s)
    e.learn_reset(seed=1)
    _run(e, traj, range(300), 1)
    plain, learned = [], []
    _run(e, traj, range(300, 320), 2, learned)
    # same frames, plain guess, on a second engine without a network
    _run(engine_for(s), traj, range(300, 320), 0, plain)
    it_p = np.mean([r[0] for r in plain])
    it_l = np.mean([r[0] for r in learned])
    eps0_p = np.mean([r[4] for r in learned])
    eps0_l = np.mean([r[5] for r in learned])
    used = np.mean([r[3] == 3 for r in learned])
    print(f"iterations plain {it_p:.2f} learned {it_l:.2f}; start residual plain {eps0_p:.4g} learned {eps0_l:.4g} D;"
          f" learned start taken in {used:.0%} of solves")
    assert all(r[2] == 0 and r[1] < 1e-6 for r in plain + learned)
    assert eps0_l < 0.6 * eps0_p
    assert used > 0.9
    assert it_l < it_p
    # the learned start changes the path, not the answer
    xyz = traj.frame(319)
    ou, op, *_ = oracle.OracleSystem(s, xyz).induce()
    ud, up, _ = e.induce_host(xyz)
    D = tg.units.DEBYE
    assert rms_err(ud * D, ou * D) < DIPOLE_RMS_DEBYE
    assert rms_err(up * D, op * D) < DIPOLE_RMS_DEBYE


def test_fallback_rejects_a_bad_network(gpu_lib, tg, LO):
    """A network with huge weights gives a far worse start: the solve must
    keep the plain guess and converge exactly as without the network."""
    s = tg.systems.make_config("water648")
    traj = tg.systems.Trajectory(s)
    e = engine_for(s)
    e.learn_reset(seed=3)
    _run(e, traj, range(3), 1)  # fixes the feature statistics and target scale
    w = e.learn_weights()
    e.learn_weights(w * 40.0)
    rec = []
    _run(e, traj, [10], 2, rec)
    # the same frames without a network (same neighbour-list history)
    ref = engine_for(s)
    _run(ref, traj, [0, 1, 2, 10, 10], 0)
    ud_ref, up_ref, _ = ref.induce_host(traj.frame(10))
    ud, up, _ = e.induce_host(traj.frame(10))
    it, eps, st, choice, eps0_p, eps0_l, _, compared = rec[0]
    assert compared == 1 and choice == 0 and eps0_l > eps0_p
    assert np.array_equal(ud, ud_ref) and np.array_equal(up, up_ref)


def test_probe_policy(gpu_lib, tg):
    """probe_every = 4: the comparison runs on every 4th solve; the solves in
    between start from the learned guess without computing the plain
    residual and give the same bits as a solve that compares and picks it
    (two engines with the same history, probe 4 and probe 1)."""
    s = tg.systems.make_config("water648")
    traj = tg.systems.Trajectory(s)
    engines = []
    for probe in (4, 1):
        e = engine_for(s)
        e.learn_reset(seed=2)
        _run(e, traj, range(100), 1)
        e.learn_policy(probe)
        e.learn_config(2)
        engines.append(e)
    rec, sol = [[], []], [[], []]
    for k in range(100, 106):
        for j, e in enumerate(engines):
            sol[j].append(e.induce_host(traj.frame(k))[:2])
            rec[j].append(e.learn_stats())
    assert [r[4] for r in rec[0]] == [1, 0, 0, 0, 1, 0]
    assert [r[4] for r in rec[1]] == [1] * 6
    assert all(r[0] == 3 for r in rec[0] + rec[1])
    for k in range(6):
        assert np.array_equal(sol[0][k][0], sol[1][k][0]) and np.array_equal(sol[0][k][1], sol[1][k][1])


def test_learned_graph_matches_stepwise(gpu_lib, tg):
    """Training and the learned start inside the induce() graph give the same
    bits as the same kernels launched one by one."""
    s = tg.systems.make_config("water648")
    traj = tg.systems.Trajectory(s)
    out = []
    for graph in (True, False):
        e = engine_for(s, predictor=1)
        e.use_graph(graph)
        e.learn_reset(seed=5)
        _run(e, traj, range(6), 1)
        _run(e, traj, range(6, 10), 3)
        ud, up, _ = e.induce_host(traj.frame(10))
        out.append((ud, up, e.learn_weights(), e.learn_stats()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
    assert out[0][3] == out[1][3]


def test_tensor_core_forward_matches_oracle(gpu_lib, tg, LO):
    """The fused tcgen05 forward and backward passes (the default;
    tensor-memory accumulators, one CTA per 128 rows, a partial last tile
    here) give the network outputs, loss and gradient within the same bar as
    the mma.sync path, and close to it."""
    s = tg.systems.make_config("water648")
    rng = np.random.default_rng(8)
    rows = 1000
    x = rng.normal(size=(rows, 32)).astype(np.float32)
    t = rng.normal(size=(rows, 3)).astype(np.float32)
    # two contexts with the same weights, so neither reads the other's outputs
    ref = engine_for(s)
    ref.learn_tensor_path(0)
    ref.learn_reset(seed=7)
    y0, g0, l0 = ref.learn_eval(x, t)
    e = engine_for(s)
    e.learn_reset(seed=7)
    e.learn_tensor_path(1)
    w = e.learn_weights().astype(np.float64)
    y, g, loss = e.learn_eval(x, t)
    assert e.copy_error() == 0
    # a second batch through the same context: new outputs, not the last call's
    y2, _, _ = e.learn_eval(-x, t)
    assert not np.array_equal(y2, y)
    yo2, _, _ = LO.loss_grad(w, -x.astype(np.float64), t.astype(np.float64), bf=True)
    assert np.linalg.norm(y2 - yo2) < NET_TOL * np.linalg.norm(yo2)
    yo, lo, go = LO.loss_grad(w, x.astype(np.float64), t.astype(np.float64), bf=True)
    print("tcgen05 vs mma.sync: y", float(np.linalg.norm(y - y0) / np.linalg.norm(y0)),
          "vs oracle", float(np.linalg.norm(y - yo) / np.linalg.norm(yo)))
    assert np.linalg.norm(y - yo) < NET_TOL * np.linalg.norm(yo)
    assert abs(loss - lo) < NET_TOL * lo
    assert np.linalg.norm(g - go) < NET_TOL * np.linalg.norm(go)
    assert np.linalg.norm(y - y0) < NET_TOL * np.linalg.norm(y0)
    # backward: every parameter block against the oracle and the mma.sync path
    print("tcgen05 vs mma.sync: g", float(np.linalg.norm(g - g0) / np.linalg.norm(g0)))
    assert abs(loss - l0) < NET_TOL * l0
    for name, a, b, c in zip(["W1", "b1", "W2", "b2", "W3", "b3"], LO.unpack(g).values(), LO.unpack(go).values(),
                             LO.unpack(g0).values()):
        assert np.linalg.norm(a - b) <= NET_TOL * np.linalg.norm(b) + 1e-9, name
        assert np.linalg.norm(a - c) <= NET_TOL * np.linalg.norm(c) + 1e-9, name
    assert np.all(LO.unpack(g)["W3"][:, 3:] == 0) and np.all(LO.unpack(g)["b3"][3:] == 0)


@pytest.mark.parametrize("rows", [1, 77, 128, 1300])
def test_tensor_core_backward_tiles(gpu_lib, tg, LO, rows):
    """Partial, single and many 128-row tiles of the fused backward pass
    against the oracle (BF16 rounding emulated)."""
    s = tg.systems.make_config("water648")
    rng = np.random.default_rng(rows)
    x = rng.normal(size=(rows, 32)).astype(np.float32)
    t = rng.normal(size=(rows, 3)).astype(np.float32)
    e = engine_for(s)
    e.learn_reset(seed=3)
    e.learn_tensor_path(1)
    w = e.learn_weights().astype(np.float64)
    y, g, loss = e.learn_eval(x, t)
    assert e.copy_error() == 0
    yo, lo, go = LO.loss_grad(w, x.astype(np.float64), t.astype(np.float64), bf=True)
    assert abs(loss - lo) < NET_TOL * lo
    assert np.linalg.norm(g - go) < NET_TOL * np.linalg.norm(go)


def test_tensor_core_learned_solve(gpu_lib, oracle, tg):
    """Training and the learned start with the tcgen05 forward pass: the
    solve still converges to the oracle's dipoles."""
    s = tg.systems.make_config("water648")
    e = engine_for(s)
    e.learn_tensor_path(1)
    e.learn_reset(seed=1)
    e.learn_config(3)
    for _ in range(3):
        ud, up, rc = e.induce_host(s.xyz)
    assert rc == 0 and e.copy_error() == 0
    ou, op, *_ = oracle.OracleSystem(s).induce()
    D = tg.units.DEBYE
    assert rms_err(ud * D, ou * D) < DIPOLE_RMS_DEBYE and rms_err(up * D, op * D) < DIPOLE_RMS_DEBYE


def test_network_beside_learned_extrapolation(gpu_lib, oracle, tg):
    """Both learned starts on one ASPC context: the network trains and is
    compared with the plain start, which is now the learned extrapolation of
    the ring; the graph and the host-driven loop agree bit for bit, every
    solve converges, the dipoles meet the oracle and no fit is rejected."""
    s = tg.systems.make_config("water648")
    traj = tg.systems.Trajectory(s)
    out = []
    for graph in (True, False):
        e = engine_for(s, predictor=1)
        e.use_graph(graph)
        e.learn_extrapolation(8)
        e.learn_reset(seed=3)
        rec = []
        _run(e, traj, range(20), 1, rec)
        _run(e, traj, range(20, 30), 3, rec)
        assert all(r[2] == 0 and r[1] < 1e-6 for r in rec)
        ud, up, _ = e.induce_host(traj.frame(30))
        fits, rej, coef = e.learn_extrapolation_state()
        assert fits == 23 and rej == 0
        out.append((ud, up, coef, e.learn_weights()))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    ou, op, *_ = oracle.OracleSystem(s, traj.frame(30)).induce()
    D = tg.units.DEBYE
    assert rms_err(out[0][0] * D, ou * D) < DIPOLE_RMS_DEBYE
    assert rms_err(out[0][1] * D, op * D) < DIPOLE_RMS_DEBYE
