"""The learned-guess oracle (oracle/learn_oracle.py) pinned on the CPU:
its FP64 gradient against torch autograd, its AdamW against
torch.optim.AdamW, its BF16 rounding against torch's float -> bfloat16
conversion, and the descriptors' rotation/translation invariance."""
import dataclasses

import numpy as np
import pytest
import torch

from oracle import learn_oracle as LO


def _torch_net(w):
    P = LO.unpack(w)
    net = torch.nn.Sequential(torch.nn.Linear(32, 64), torch.nn.SiLU(), torch.nn.Linear(64, 64), torch.nn.SiLU(),
                              torch.nn.Linear(64, 8)).double()
    with torch.no_grad():
        for lin, (W, b) in zip((net[0], net[2], net[4]), (("W1", "b1"), ("W2", "b2"), ("W3", "b3"))):
            lin.weight.copy_(torch.tensor(P[W].T))
            lin.bias.copy_(torch.tensor(P[b]))
    return net


def _grad_of(net):
    g = {}
    for lin, (W, b) in zip((net[0], net[2], net[4]), (("W1", "b1"), ("W2", "b2"), ("W3", "b3"))):
        g[W] = lin.weight.grad.numpy().T
        g[b] = lin.bias.grad.numpy()
    return LO.pack(g)


def _random_weights(rng):
    w = rng.normal(scale=0.2, size=LO.NPARAM)
    return w * LO.trainable_mask()


def test_fp64_gradient_matches_autograd():
    rng = np.random.default_rng(3)
    w = _random_weights(rng)
    x = rng.normal(size=(50, 32))
    t = rng.normal(size=(50, 3))
    y, loss, g = LO.loss_grad(w, x, t, bf=False)
    net = _torch_net(w)
    out = net(torch.tensor(x))[:, :3]
    tl = ((out - torch.tensor(t)) ** 2).mean()
    tl.backward()
    assert abs(loss - tl.item()) < 1e-12 * max(1.0, abs(loss))
    assert np.abs(y - out.detach().numpy()).max() < 1e-12
    gt = _grad_of(net) * LO.trainable_mask()
    assert np.abs(g - gt).max() < 1e-12 * max(1.0, np.abs(gt).max())


def test_bf16_gradient_close_to_fp64():
    rng = np.random.default_rng(4)
    w = _random_weights(rng)
    x = rng.normal(size=(200, 32))
    t = rng.normal(size=(200, 3))
    _, _, g64 = LO.loss_grad(w, x, t, bf=False)
    _, _, g16 = LO.loss_grad(w, x, t, bf=True)
    assert np.linalg.norm(g16 - g64) < 3e-2 * np.linalg.norm(g64)


def test_adamw_matches_torch():
    rng = np.random.default_rng(5)
    w = _random_weights(rng)
    mask = LO.trainable_mask() > 0
    p = torch.nn.Parameter(torch.tensor(w[mask]))
    opt = torch.optim.AdamW([p], lr=1e-3, weight_decay=1e-2, betas=(0.9, 0.999), eps=1e-8)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    ww = w.copy()
    for step in range(1, 4):
        g = rng.normal(size=w.shape) * LO.trainable_mask()
        p.grad = torch.tensor(g[mask])
        opt.step()
        ww, m, v = LO.adamw(ww, g, m, v, step)
    assert np.abs(ww[mask] - p.detach().numpy()).max() < 1e-13
    assert np.all(ww[~mask] == w[~mask])


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(6)
    a = np.concatenate([rng.normal(size=5000), rng.normal(size=5000) * 1e-3, [0.0, 1.0, 1.0 + 2.0 ** -8, -3.0]])
    a = a.astype(np.float32)
    ref = torch.tensor(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(LO.bf16(a), ref)


def _cluster(tg, nmol=40):
    """A non-periodic cut of the 648-atom water box (first nmol molecules)."""
    s = tg.systems.make_config("water648")
    na = 3 * nmol
    keep = (s.excl_ik[:, 0] < na) & (s.excl_ik[:, 1] < na)
    fr = s.frames[:na].copy()
    return dataclasses.replace(s, xyz=s.xyz[:na].copy(), types=s.types[:na], frames=fr, pole=s.pole[:na],
                               polarity=s.polarity[:na], thole=s.thole[:na], pdamp=s.pdamp[:na],
                               excl_ik=s.excl_ik[keep], excl_scale=s.excl_scale[keep], box=None,
                               mol_start=None, mol_size=None)


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q *= np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def test_features_rotation_translation_invariant(tg, oracle):
    s = _cluster(tg)
    rng = np.random.default_rng(7)
    n = s.n
    fd = rng.normal(size=(n, 3)) * 0.1
    fp = rng.normal(size=(n, 3)) * 0.1
    X = LO.features(s, s.xyz, fd, fp, oracle.frames(s, s.xyz))
    R = _random_rotation(rng)
    xyz2 = s.xyz @ R.T + np.array([3.0, -7.0, 11.0])
    X2 = LO.features(s, xyz2, fd @ R.T, fp @ R.T, oracle.frames(s, xyz2))
    assert np.abs(X - X2).max() < 1e-9 * max(1.0, np.abs(X).max())
    # every atom of the cut sees partners within 6 A
    assert (X[:, 4:11].sum(axis=1) > 0).all()


def test_features_two_atoms_by_hand(tg):
    """Two bare atoms 2.5 A apart along z: radial and polarizability sums by hand."""
    s = _cluster(tg, nmol=1)
    s = dataclasses.replace(s, xyz=np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.5]]), types=s.types[:2],
                            frames=np.array([[0, 0, 0, 0], [0, 0, 0, 0]], dtype=np.int32), pole=s.pole[:2],
                            polarity=s.polarity[:2], thole=s.thole[:2], pdamp=s.pdamp[:2],
                            excl_ik=np.zeros((0, 2), dtype=np.int32), excl_scale=np.zeros((0, 4)))
    F = np.repeat(np.eye(3)[None], 2, axis=0)
    z = np.zeros((2, 3))
    X = LO.features(s, s.xyz, z, z, F)
    r = 2.5
    fc = 0.5 * (np.cos(np.pi * r / 6) + 1)
    for j in range(7):
        mu = 1 + 5.0 * j / 6
        assert X[0, 4 + j] == pytest.approx(fc * np.exp(-((r - mu) ** 2) / 0.5))
    for j in range(5):
        mu = 1 + 1.25 * j
        assert X[0, 21 + j] == pytest.approx(s.polarity[1] * fc * np.exp(-((r - mu) ** 2) / 0.72))
    # charge-direction feature points from atom 0 to atom 1 (+z)
    q1 = s.pole[1, 0]
    assert X[0, 17] == pytest.approx(q1 * fc * np.exp(-((r - 2.0) ** 2) / 2.0))
    assert X[1, 17] == pytest.approx(-s.pole[0, 0] * fc * np.exp(-((r - 2.0) ** 2) / 2.0))


def test_lx_ring_coefficients_polynomial():
    """The restated online fit of the ring extrapolation: frames that follow
    polynomials of degree K - 1 in time are extrapolated exactly by
    c_j = (-1)^j C(K, j + 1) (the K-th difference vanishes), one fit after
    each frame from the (K + 1)-th on; the coefficients sum to 1."""
    from math import comb

    rng = np.random.default_rng(3)
    for K in (2, 4, 6):
        P = rng.normal(size=(K, 300))
        frames = [sum(P[d] * (0.1 * t) ** d for d in range(K)) for t in range(K + 20)]
        c, nfit = LO.lx_ring_coefficients(frames, K, ridge=0.0)
        want = np.zeros(16)
        want[:K] = [(-1) ** j * comb(K, j + 1) for j in range(K)]
        assert nfit == 20
        assert np.abs(c - want).max() < 1e-6 * comb(K, K // 2), (K, c[:K])
        assert c.sum() == pytest.approx(1.0, abs=1e-8)
