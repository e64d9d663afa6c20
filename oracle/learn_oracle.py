"""numpy restatement of the learned initial guess (descriptors, network,
AdamW) used to check the CUDA kernels.

TEST INFRASTRUCTURE ONLY: imported by tests/ and bench.py's checks, never by
the product library.  The learned guess has no counterpart in the reference
(its guesses are alpha*E, src/cu/amoeba/induce.cu pcgUdirV2, and the
predictors of src/amoeba/induce.cpp:29-69), so this module states the
project's own definition:

  features (32 per atom and dipole set, in the atom's local multipole frame)
    0-2   direct field E;  3  polarizability
    4-10  sum_k fc g(r; 1 + 5j/6, 0.5)          11-14 sum_k q_k fc g(r; 1.5(j+1), 0.75)
    15-20 sum_k q_k fc g(r; mu, 1) r_hat, mu = 2, 4.5
    21-25 sum_k alpha_k fc g(r; 1 + 1.25j, 0.6)
    26-31 sum_k u_ik (-T_ik^Thole)(alpha_k E_k), split at r = 3.5 A
  over partners within 6 A, fc = (1 + cos(pi r / 6)) / 2,
  g(r; mu, s) = exp(-(r - mu)^2 / (2 s^2)).  The Thole damping is the
  reference's damp_thole3 (include/seq/damp.h:26-44).

  network 32 -> 64 SiLU -> 64 SiLU -> 3, loss mean((y - t)^2); the CUDA path
  rounds inputs, weights, hidden activations and the back-propagated output
  and pre-activation gradients to BF16 and accumulates in FP32; bf16=True
  reproduces those rounding points.

  AdamW (Loshchilov & Hutter 2019) with beta 0.9 / 0.999, eps 1e-8.
"""
import numpy as np

NFEAT, NHID, NOUT, NOUT_PAD = 32, 64, 3, 8
SIZES = [("W1", (NFEAT, NHID)), ("b1", (NHID,)), ("W2", (NHID, NHID)), ("b2", (NHID,)), ("W3", (NHID, NOUT_PAD)),
         ("b3", (NOUT_PAD,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)
DESC_CUT = 6.0


def unpack(w):
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = np.asarray(w[o:o + k], dtype=np.float64).reshape(shape)
        o += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def trainable_mask():
    """1 for parameters the optimiser updates (output columns 3-7 stay 0)."""
    m = {name: np.ones(shape) for name, shape in SIZES}
    m["W3"][:, NOUT:] = 0
    m["b3"][NOUT:] = 0
    return pack(m)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(w, x, bf=True):
    """Returns (y [rows][3], cache)."""
    P = unpack(w)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    W1, W2, W3 = r(P["W1"]), r(P["W2"]), r(P["W3"])
    X = r(x)
    Z1 = X @ W1 + P["b1"]
    H1 = r(_silu(Z1))
    Z2 = H1 @ W2 + P["b2"]
    H2 = r(_silu(Z2))
    Y = H2 @ W3 + P["b3"]
    return Y[:, :NOUT], dict(X=X, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Y=Y, W1=W1, W2=W2, W3=W3, bf=bf)


def loss_grad(w, x, t, bf=True):
    """(y, loss, gradient in the packed layout)."""
    y, c = forward(w, x, bf)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    rows = x.shape[0]
    d = y - t
    loss = float((d ** 2).sum() / (rows * NOUT))
    dYf = np.zeros((rows, NOUT_PAD))
    dYf[:, :NOUT] = 2.0 * d / (rows * NOUT)
    dY = r(dYf)
    g = {}
    g["W3"] = c["H2"].T @ dY
    g["b3"] = dYf.sum(axis=0)
    dZ2f = (dY @ c["W3"].T) * _silu_grad(c["Z2"])
    dZ2 = r(dZ2f)
    g["W2"] = c["H1"].T @ dZ2
    g["b2"] = dZ2f.sum(axis=0)
    dZ1f = (dZ2 @ c["W2"].T) * _silu_grad(c["Z1"])
    dZ1 = r(dZ1f)
    g["W1"] = c["X"].T @ dZ1
    g["b1"] = dZ1f.sum(axis=0)
    return y, loss, pack(g)


def adamw(w, g, m, v, step, lr=1e-3, wd=1e-2, beta1=0.9, beta2=0.999, eps=1e-8):
    """One AdamW step on the trainable parameters; returns (w, m, v)."""
    mask = trainable_mask() > 0
    w, m, v = np.array(w, dtype=np.float64), np.array(m, dtype=np.float64), np.array(v, dtype=np.float64)
    m[mask] = beta1 * m[mask] + (1 - beta1) * g[mask]
    v[mask] = beta2 * v[mask] + (1 - beta2) * g[mask] ** 2
    c1, c2 = 1 - beta1 ** step, 1 - beta2 ** step
    w[mask] -= lr * ((m[mask] / c1) / (np.sqrt(v[mask] / c2) + eps) + wd * w[mask])
    return w, m, v


# ---------------------------------------------------------------------------
# descriptors


def _pairs(xyz, box, cut):
    """All i < k within cut (minimum image for a periodic box): (i, k, d = x_k - x_i)."""
    from scipy.spatial import cKDTree

    if box is not None:
        L = np.asarray(box, dtype=np.float64)
        tree = cKDTree(np.mod(xyz, L), boxsize=L)
    else:
        tree = cKDTree(xyz)
    pr = tree.query_pairs(cut, output_type="ndarray")
    i, k = pr[:, 0], pr[:, 1]
    d = xyz[k] - xyz[i]
    if box is not None:
        d -= L * np.round(d / L)
    return i, k, d


def _gauss(r, mu, s):
    return np.exp(-((r - mu) ** 2) / (2 * s * s))


def features(system, xyz, field_d, field_p, frames):
    """Raw features [2n][32] (d rows, then p rows) for the given coordinates,
    direct fields [n][3] and local frames [n][3][3]."""
    n = system.n
    xyz = np.asarray(xyz, dtype=np.float64)
    alpha = np.asarray(system.polarity, dtype=np.float64)
    q = np.asarray(system.pole, dtype=np.float64)[:, 0]
    thole = np.asarray(system.thole, dtype=np.float64)
    pdamp = np.asarray(system.pdamp, dtype=np.float64)
    ud = alpha[:, None] * field_d
    up = alpha[:, None] * field_p
    i, k, d = _pairs(xyz, system.box, DESC_CUT)
    uscale = np.ones(len(i))
    if len(system.excl_ik):
        key = {}
        for (a, b), sc in zip(np.asarray(system.excl_ik), np.asarray(system.excl_scale)):
            key[(min(a, b), max(a, b))] = sc[3]
        for m in range(len(i)):
            s = key.get((min(i[m], k[m]), max(i[m], k[m])))
            if s is not None:
                uscale[m] = s
    r = np.linalg.norm(d, axis=1)
    fc = 0.5 * (np.cos(np.pi * r / DESC_CUT) + 1)
    pg = np.minimum(thole[i], thole[k])
    damp = pdamp[i] * pdamp[k]
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(damp != 0, -pg * (r / np.where(damp != 0, damp, 1)) ** 3, -1e16)
    ex = np.exp(a)
    s3 = 1 - ex
    s5 = 1 - ex * (1 - a)
    rr3 = uscale * s3 / r ** 3
    rr5 = 3 * uscale * s5 / r ** 5
    acc = np.zeros((n, 34))
    for src, dst, dd in ((k, i, d), (i, k, -d)):
        for j in range(7):
            np.add.at(acc[:, j], dst, fc * _gauss(r, 1 + 5.0 * j / 6, 0.5))
        for j in range(4):
            np.add.at(acc[:, 7 + j], dst, q[src] * fc * _gauss(r, 1.5 * (j + 1), 0.75))
        for s_, mu in enumerate((2.0, 4.5)):
            h = q[src] * fc * _gauss(r, mu, 1.0) / r
            for c in range(3):
                np.add.at(acc[:, 11 + 3 * s_ + c], dst, h * dd[:, c])
        for j in range(5):
            np.add.at(acc[:, 17 + j], dst, alpha[src] * fc * _gauss(r, 1 + 1.25 * j, 0.6))
        near = r < 3.5
        for off, u in ((22, ud), (28, up)):
            uk = u[src]
            c = rr5 * (dd * uk).sum(axis=1)
            f = c[:, None] * dd - rr3[:, None] * uk
            for comp in range(3):
                np.add.at(acc[:, off + comp], dst[near], f[near, comp])
                np.add.at(acc[:, off + 3 + comp], dst[~near], f[~near, comp])
    loc = lambda v: np.einsum("nab,nb->na", frames, v)
    out = np.zeros((2, n, NFEAT))
    for sysi, (E, off) in enumerate(((field_d, 22), (field_p, 28))):
        x = out[sysi]
        x[:, 0:3] = loc(E)
        x[:, 3] = alpha
        x[:, 4:11] = acc[:, 0:7]
        x[:, 11:15] = acc[:, 7:11]
        x[:, 15:18] = loc(acc[:, 11:14])
        x[:, 18:21] = loc(acc[:, 14:17])
        x[:, 21:26] = acc[:, 17:22]
        x[:, 26:29] = loc(acc[:, off:off + 3])
        x[:, 29:32] = loc(acc[:, off + 3:off + 6])
    return out.reshape(2 * n, NFEAT)


def targets(system, uind, uinp, field_d, field_p, frames, tscale):
    """Training targets [2n][3]: F (u - alpha E) / (alpha tscale)."""
    alpha = np.asarray(system.polarity, dtype=np.float64)[:, None]
    td = np.einsum("nab,nb->na", frames, (uind - alpha * field_d) / alpha) / tscale
    tp = np.einsum("nab,nb->na", frames, (uinp - alpha * field_p) / alpha) / tscale
    return np.concatenate([td, tp])


def guess(system, y, field_d, field_p, frames, tscale):
    """Dipoles alpha E + alpha F^T y tscale from network outputs y [2n][3]."""
    n = system.n
    alpha = np.asarray(system.polarity, dtype=np.float64)[:, None]
    g = np.einsum("nab,na->nb", frames, y[:n]) * tscale
    gp = np.einsum("nab,na->nb", frames, y[n:]) * tscale
    return alpha * (field_d + g), alpha * (field_p + gp)


def lx_ring_coefficients(frames, order, lam=0.99, ridge=1e-6):
    """The learned extrapolation of the predictor ring, restated in FP64.

    frames: the converged dipoles of consecutive solves (any shape; the d and
    p sets of one solve together), oldest first.  After every solve t >= order
    the newest frame y = u_t and the `order` frames before it give the samples
    y ~ sum_k a_k D^k u_{t-1} over every element, D^k u_{t-1} =
    sum_j (-1)^j C(k, j) u_{t-1-j} the k-th backward difference.  The normal
    equations accumulate with forgetting factor lam (N <- lam N + D^T D,
    r <- lam r + D^T y); each fit solves the Jacobi-scaled system plus ridge on
    its diagonal.  Returns the 16 ring coefficients by frame age (0 the newest;
    zero beyond the order) after the last fit, c_j = sum_k a_k (-1)^j C(k, j),
    and the number of fits."""
    from math import comb

    K = order
    U = [np.asarray(f, dtype=np.float64).ravel() for f in frames]
    N = np.zeros((K, K))
    r = np.zeros(K)
    coef = np.zeros(16)
    fits = 0
    S = np.array([[(-1) ** j * comb(k, j) for j in range(K)] for k in range(K)], dtype=np.float64)
    for t in range(K, len(U)):
        prev = np.stack([U[t - 1 - j] for j in range(K)], 1)   # [m][K], ages 0..K-1
        D = prev @ S.T                                          # [m][K], differences 0..K-1
        N = lam * N + D.T @ D
        r = lam * r + D.T @ U[t]
        sc = 1.0 / np.sqrt(np.diag(N))
        z = np.linalg.solve(N * np.outer(sc, sc) + ridge * np.eye(K), r * sc)
        a = z * sc
        coef[:K] = S.T @ a
        fits += 1
    return coef, fits
