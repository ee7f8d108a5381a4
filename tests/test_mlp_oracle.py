"""CPU checks of the FP64 radiance-cache oracle (oracle/rr_mlp.c): its
gradient equals finite differences of the loss (with the denominators held
at the unperturbed prediction, as the relative-L2 loss prescribes), and its
BF16 emulation stays close to the exact computation."""
import numpy as np

from oracle import orc

NP = 4 * 64 * 64 + 64 * 16


def random_problem(B=64, seed=0):
    rng = np.random.default_rng(seed)
    W = np.concatenate([rng.uniform(-0.2, 0.2, 4 * 4096), rng.uniform(-0.27, 0.27, 1024)]).astype(np.float32)
    p = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    n = rng.normal(size=(B, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    alb = rng.uniform(0.2, 0.8, (B, 3)).astype(np.float32)
    X = orc.mlp_encode(p, n, alb, np.array([-1, -1, -1], np.float32), np.array([1, 1, 1], np.float32))
    T = rng.uniform(0, 2, (B, 3)).astype(np.float32)
    return W, X.astype(np.float32), T


def test_encoding_layout():
    X = orc.mlp_encode(np.array([[0.5, 0.25, 1.0]], np.float32), np.array([[0, 0, 1]], np.float32),
                       np.array([[0.2, 0.4, 0.6]], np.float32), np.zeros(3, np.float32), np.full(3, 2, np.float32))
    u = [0.25, 0.125, 0.5]
    for j in range(3):
        for k in range(8):
            assert abs(X[0, 16 * j + 2 * k] - np.sin(2 ** k * np.pi * u[j])) < 1e-12
            assert abs(X[0, 16 * j + 2 * k + 1] - np.cos(2 ** k * np.pi * u[j])) < 1e-12
    np.testing.assert_allclose(X[0, 48:55], [0, 0, 1, 0.2, 0.4, 0.6, 1], atol=1e-7)
    assert np.all(X[0, 55:] == 0)


def test_gradient_matches_finite_differences():
    W, X, T = random_problem()
    dW, loss, Y0 = orc.mlp_grad(W, X, T, bf16=False)
    B = X.shape[0]
    den = Y0.astype(np.float64) ** 2 + 0.01
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.integers(0, 4096, 4) + 4096 * l for l in range(4)] + [16384 + rng.integers(0, 1024, 4)])
    for i in idx:
        h = 1e-3
        Wp, Wm = W.astype(np.float64).copy(), W.astype(np.float64).copy()
        Wp[i] += h
        Wm[i] -= h
        _, _, Yp = orc.mlp_grad(Wp.astype(np.float32), X, T, bf16=False)
        _, _, Ym = orc.mlp_grad(Wm.astype(np.float32), X, T, bf16=False)
        Lp = (((Yp - T) ** 2) / den).sum() / B
        Lm = (((Ym - T) ** 2) / den).sum() / B
        fd = (Lp - Lm) / (float(np.float32(W[i] + h)) - float(np.float32(W[i] - h)))
        assert abs(fd - dW[i]) <= 2e-3 * max(1.0, abs(dW[i])) + 2e-5, (i, fd, dW[i])


def test_bf16_emulation_close_to_exact():
    W, X, T = random_problem(B=256, seed=3)
    d64, l64, _ = orc.mlp_grad(W, X, T, bf16=False)
    d16, l16, _ = orc.mlp_grad(W, X, T, bf16=True)
    for l in range(5):
        a, b = (slice(4096 * l, 4096 * (l + 1)) if l < 4 else slice(16384, NP)), None
        rel = np.linalg.norm(d16[a] - d64[a]) / np.linalg.norm(d64[a])
        assert rel < 0.12, (l, rel)   # BF16 rounding of activations and deltas
    assert abs(l16 - l64) < 0.02 * l64
    assert orc.lib().orc_bf16(1.0 + 2 ** -9) == 1.0            # ties to even
    assert orc.lib().orc_bf16(1.0 + 3 * 2 ** -9) == 1.0 + 2 ** -7


# ------------------------------------------------------------ hash grid
HT = 1 << 14


def hash_problem(B=48, seed=5):
    rng = np.random.default_rng(seed)
    W = np.concatenate([rng.uniform(-0.2, 0.2, 4 * 4096), rng.uniform(-0.27, 0.27, 1024)]).astype(np.float32)
    table = rng.uniform(-0.5, 0.5, 16 * HT * 2).astype(np.float32)
    p = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    n = rng.normal(size=(B, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    alb = rng.uniform(0.2, 0.8, (B, 3)).astype(np.float32)
    t = rng.uniform(0, 2, (B, 3)).astype(np.float32)
    lo = np.full(3, -1, np.float32)
    ie = np.full(3, 0.5, np.float32)
    return W, table, orc.hashgrid_res(), lo, ie, p, n, alb, t


def test_hashgrid_resolutions():
    r = orc.hashgrid_res()
    assert r[0] == 16 and r[-1] in (1023, 1024) and np.all(np.diff(r) > 0)
    b = (1024 / 16) ** (1 / 15)
    np.testing.assert_array_equal(r, np.floor(16 * b ** np.arange(16)).astype(np.int32))


def test_hash_encoding_interpolates_a_linear_table():
    """On densely indexed levels a table holding (ix, iy) at each lattice
    point encodes to (u_x N, u_y N): trilinear interpolation is exact on a
    linear field."""
    res = orc.hashgrid_res()
    table = np.zeros(16 * HT * 2, np.float32)
    dense = [l for l in range(16) if (res[l] + 1) ** 3 <= HT]
    assert dense == [0, 1]
    for l in dense:
        n1 = res[l] + 1
        iz, iy, ix = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
        idx = (ix + iy * n1 + iz * n1 * n1).ravel()
        table[(l * HT + idx) * 2] = ix.ravel()
        table[(l * HT + idx) * 2 + 1] = iy.ravel()
    rng = np.random.default_rng(2)
    p = rng.uniform(-1, 1, (20, 3)).astype(np.float32)
    lo = np.full(3, -1, np.float32)
    ie = np.full(3, 0.5, np.float32)
    X = orc.mlp_encode_hash(p, np.zeros((20, 3)), np.zeros((20, 3)), lo, ie, table, res, HT)
    u = (p - lo) * ie
    for l in dense:
        np.testing.assert_allclose(X[:, 2 * l], u[:, 0] * res[l], atol=1e-4)
        np.testing.assert_allclose(X[:, 2 * l + 1], u[:, 1] * res[l], atol=1e-4)
    np.testing.assert_allclose(X[:, 62], 1.0)
    np.testing.assert_allclose(X[:, 32], np.sin(np.pi * u[:, 0].astype(np.float64)), atol=1e-6)


def test_hash_table_gradient_matches_finite_differences():
    W, table, res, lo, ie, p, n, alb, t = hash_problem()
    dW, dT, loss, Y0 = orc.mlp_grad_hash(W, table, res, HT, lo, ie, p, n, alb, t, bf16=False)
    B = p.shape[0]
    den = Y0.astype(np.float64) ** 2 + 0.01
    touched = np.nonzero(dT)[0]
    assert touched.size > 1000
    rng = np.random.default_rng(3)
    errs = []
    for i in rng.choice(touched, 12, replace=False):
        h = 1e-3
        tp, tm = table.copy(), table.copy()
        tp[i] += h
        tm[i] -= h
        _, _, _, Yp = orc.mlp_grad_hash(W, tp, res, HT, lo, ie, p, n, alb, t, bf16=False)
        _, _, _, Ym = orc.mlp_grad_hash(W, tm, res, HT, lo, ie, p, n, alb, t, bf16=False)
        Lp = (((Yp - t) ** 2) / den).sum() / B
        Lm = (((Ym - t) ** 2) / den).sum() / B
        fd = (Lp - Lm) / (float(tp[i]) - float(tm[i]))
        errs.append(abs(fd - dT[i]) / abs(dT[i]))
    # relu kinks inside +-h can move a few; the bulk agrees to FD precision
    assert np.median(errs) < 1e-3 and max(errs) < 0.1, errs
