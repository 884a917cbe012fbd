"""The learned preconditioner's CPU oracle (oracle/mpnn_ref.py) on its own:
analytic gradients against central finite differences (block-Jacobi and
SSOR contexts), the losses against their definitions, the BF16 rounding
helper against known values, and the blocks' SPD property."""
import numpy as np

from oracle import mpnn_ref as R


def tiny_graph(n=24, seed=0):
    rng = np.random.default_rng(seed)
    rows = [sorted({i, (i + 1) % n, (i - 1) % n, int(rng.integers(n))}) for i in range(n)]
    rp = np.cumsum([0] + [len(r) for r in rows])
    cols = np.concatenate(rows)
    return rp, cols


def spd(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(2 * n, 2 * n))
    return A @ A.T + 2 * n * np.eye(2 * n)


def test_param_count():
    assert R.N_PARAMS == 26051


import pytest


@pytest.mark.parametrize("ssor", [False, True])
def test_gradient_matches_finite_differences(ssor):
    n = 24
    rp, cols = tiny_graph(n)
    rng = np.random.default_rng(1)
    f = rng.normal(size=(n, R.F_IN))
    K = spd(n, 2)
    Kd = np.stack([K[2 * i:2 * i + 2, 2 * i:2 * i + 2] for i in range(n)])
    e = rng.normal(size=2 * n)
    v = rng.normal(size=2 * n)
    r = K @ e
    th = rng.normal(0, 0.3, R.N_PARAMS)
    args = (f, rp, cols, K, Kd, r, e, v)
    loss, g, _ = R.loss_and_grad(th, *args, ssor=ssor)
    assert np.isfinite(loss)
    idx = rng.choice(R.N_PARAMS, 60, replace=False)
    h = 1e-6
    for k in idx:
        tp, tm = th.copy(), th.copy()
        tp[k] += h
        tm[k] -= h
        fd = (R.loss_and_grad(tp, *args, ssor=ssor)[0] - R.loss_and_grad(tm, *args, ssor=ssor)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-5 * max(1.0, abs(g).max()), (k, fd, g[k])


def test_loss_is_log_rayleigh_ratio():
    """With c = 0 (block Jacobi) the loss is log R(v) - log R(e) computed directly."""
    n = 10
    rp, cols = tiny_graph(n)
    rng = np.random.default_rng(4)
    K = spd(n, 5)
    Kd = np.stack([K[2 * i:2 * i + 2, 2 * i:2 * i + 2] for i in range(n)])
    th = np.zeros(R.N_PARAMS)
    e, v = rng.normal(size=2 * n), rng.normal(size=2 * n)
    loss, _, c = R.loss_and_grad(th, rng.normal(size=(n, R.F_IN)), rp, cols, K, Kd, K @ e, e, v)
    Binv = np.zeros((2 * n, 2 * n))
    for i in range(n):
        Binv[2 * i:2 * i + 2, 2 * i:2 * i + 2] = Kd[i]
    Rq = lambda x: (x @ K @ x) / (x @ Binv @ x)
    assert abs(loss - (np.log(Rq(v)) - np.log(Rq(e)))) < 1e-12


def test_ssor_loss_is_log_rayleigh_ratio():
    """SSOR context with c = 0: Q(x) = x.M x, M = (D + L) D^-1 (D + U) with
    D the diagonal blocks, L / U the lower / upper node-block parts."""
    n = 10
    rp, cols = tiny_graph(n)
    rng = np.random.default_rng(6)
    K = spd(n, 7)
    Kd = np.stack([K[2 * i:2 * i + 2, 2 * i:2 * i + 2] for i in range(n)])
    th = np.zeros(R.N_PARAMS)
    e, v = rng.normal(size=2 * n), rng.normal(size=2 * n)
    loss, _, _ = R.loss_and_grad(th, rng.normal(size=(n, R.F_IN)), rp, cols, K, Kd, K @ e, e, v, ssor=True)
    blk = np.kron(np.eye(n), np.ones((2, 2))) > 0
    D = np.where(blk, K, 0.0)
    Lo = np.where(blk, 0.0, np.tril(K))
    Up = np.where(blk, 0.0, np.triu(K))
    Mm = (D + Lo) @ np.linalg.inv(D) @ (D + Up)
    Rq = lambda x: (x @ K @ x) / (x @ Mm @ x)
    assert abs(loss - (np.log(Rq(v)) - np.log(Rq(e)))) < 1e-10


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -3.0 + 2 ** -7 + 2 ** -8, 65504.0, 1e-3])
    want = np.array([1.0, 1.0, 1.0 + 2 ** -7, -3.0 + 2 ** -6, 65536.0, 0.00099945068359375])
    np.testing.assert_array_equal(R.bf16(x), want)


def test_blocks_are_spd_for_any_output():
    rng = np.random.default_rng(3)
    c = R.C_SCALE * np.tanh(rng.normal(0, 10, (1000, 3)))
    A = rng.normal(size=(1000, 2, 2))
    Kd = A @ np.transpose(A, (0, 2, 1)) + 0.1 * np.eye(2) * np.exp(rng.normal(0, 3, (1000, 1, 1)))
    B = R.blocks(c, Kd)
    ev = np.linalg.eigvalsh(B)
    assert (ev > 0).all()
    # c = 0: block Jacobi
    np.testing.assert_allclose(R.blocks(0 * c, Kd), np.linalg.inv(Kd), rtol=1e-12)
