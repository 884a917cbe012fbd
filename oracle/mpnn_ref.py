"""CPU restatement of the learned block preconditioner (TEST INFRASTRUCTURE ONLY).

The network of bfm_gb300/csrc/mpnn.cu in float64 numpy, forward and analytic
backward, used by tests/test_gpu_learned.py to check the GPU kernels'
features, activations, blocks, loss and gradients.  It has no counterpart in the
reference (libbfm has no learned part); it is the oracle of this build's own
additive feature.

Network (parameters in this order, FP32 masters, BF16 copies on the GPU):
    h0 = relu(W0 f + b0)                       W0: 64 x 16
    h_l = relu(W_l [h_{l-1}, m_{l-1}] + b_l)   W_l: 64 x 128, l = 1..3
          m = mean of h over the node's row of the node graph (itself included)
    o = Wo h3 + bo                             Wo: 3 x 64
    c = 0.45 tanh(o)
    B_i = K_ii^-1 + L_i C_i L_i^T,  L_i L_i^T = K_ii^-1 (Cholesky),  C_i = [[c0, c1], [c1, c2]]
          (K_ii: the node's 2x2 diagonal block; c = 0 is block Jacobi)
Loss of one (residual r = K e, error e) pair with a power vector v of B K:
    L = log R(v) - log R(e),  R(x) = (x.K x) / (x.B^-1 x)
the log of a condition-number estimate of the preconditioned operator.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

F_IN, H = 16, 64
SHAPES = [(H, F_IN), (H,), (H, 2 * H), (H,), (H, 2 * H), (H,), (H, 2 * H), (H,), (3, H), (3,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)
C_SCALE = 0.45


def unpack(theta: np.ndarray):
    out, k = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(theta[k:k + n].reshape(s))
        k += n
    return out


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), through float32, as
    __float2bfloat16 does on the GPU."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _id(x):
    return x


def mean_agg(rp, cols, h):
    deg = np.diff(rp).astype(np.float64)
    m = np.zeros_like(h)
    rows = np.repeat(np.arange(len(deg)), np.diff(rp))
    np.add.at(m, rows, h[cols])
    return m / deg[:, None]


def mean_agg_T(rp, cols, dm):
    """adjoint of mean_agg: dh[j] = sum over rows i containing j of dm[i]/deg[i]"""
    deg = np.diff(rp).astype(np.float64)
    rows = np.repeat(np.arange(len(deg)), np.diff(rp))
    dh = np.zeros_like(dm)
    np.add.at(dh, cols, dm[rows] / deg[rows, None])
    return dh


def forward(theta, f, rp, cols, emulate=False):
    """c (n, 3) and the activations.  emulate=True rounds to BF16 where the
    GPU stores BF16 (weights of the dense layers, activations, aggregates);
    the head and every accumulation stay in full precision."""
    r = bf16 if emulate else _id
    W0, b0, W1, b1, W2, b2, W3, b3, Wo, bo = unpack(theta)
    hs = [r(np.maximum(f @ r(W0).T + b0, 0.0))]
    xs = []
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        x = np.concatenate([hs[-1], r(mean_agg(rp, cols, hs[-1]))], 1)
        xs.append(x)
        hs.append(r(np.maximum(x @ r(W).T + b, 0.0)))
    o = hs[-1] @ Wo.T + bo
    c = C_SCALE * np.tanh(o)
    return c, dict(hs=hs, xs=xs, o=o)


def chol_inv(Kd):
    """L (n, 2, 2) lower triangular with L L^T = Kd^-1 for SPD 2x2 blocks Kd."""
    k00, k01, k11 = Kd[:, 0, 0], Kd[:, 0, 1], Kd[:, 1, 1]
    det = k00 * k11 - k01 * Kd[:, 1, 0]
    L = np.zeros_like(Kd)
    L[:, 0, 0] = np.sqrt(k11 / det)
    L[:, 1, 0] = -k01 / np.sqrt(det * k11)
    L[:, 1, 1] = 1.0 / np.sqrt(k11)
    return L


def blocks(c, Kd):
    """B_i as (n, 2, 2) from c (n, 3) and the diagonal blocks Kd (n, 2, 2)"""
    L = chol_inv(Kd)
    C = np.zeros_like(Kd)
    C[:, 0, 0], C[:, 0, 1], C[:, 1, 0], C[:, 1, 1] = c[:, 0], c[:, 1], c[:, 1], c[:, 2]
    return np.linalg.inv(Kd) + L @ C @ np.transpose(L, (0, 2, 1))


def binv_quad(L, c, x2):
    """Per node u = L^-1 x, w = (I + C)^-1 u; returns (sum of u.w, w)."""
    u0 = x2[:, 0] / L[:, 0, 0]
    u1 = (x2[:, 1] - L[:, 1, 0] * u0) / L[:, 1, 1]
    det = (1 + c[:, 0]) * (1 + c[:, 2]) - c[:, 1] ** 2
    w0 = ((1 + c[:, 2]) * u0 - c[:, 1] * u1) / det
    w1 = (-c[:, 1] * u0 + (1 + c[:, 0]) * u1) / det
    return float(u0 @ w0 + u1 @ w1), np.stack([w0, w1], 1)


def b_quad(L, c, u2):
    """Per node s = L^T u, s.(I + C) s; returns (sum, s)."""
    s0 = L[:, 0, 0] * u2[:, 0] + L[:, 1, 0] * u2[:, 1]
    s1 = L[:, 1, 1] * u2[:, 1]
    q = s0 * s0 + s1 * s1 + c[:, 0] * s0 * s0 + 2 * c[:, 1] * s0 * s1 + c[:, 2] * s1 * s1
    return float(q.sum()), np.stack([s0, s1], 1)


def lu_split(K, n):
    """Strictly lower- and upper-node-block parts of K (scalar CSR, 2 DOFs per
    node): in a colour-major order, the lower- and higher-colour couplings."""
    Kc = sp.coo_matrix(K)
    rn, cn = Kc.row // 2, Kc.col // 2
    mk = lambda m: sp.csr_matrix((Kc.data[m], (Kc.row[m], Kc.col[m])), shape=K.shape)
    return mk(cn < rn), mk(cn > rn)


def loss_and_grad(theta, f, rp, cols, K, Kd, r, e, v, emulate=False, ssor=False):
    """Loss log R(v) - log R(e), R(x) = (x.Kx) / Q(x), and d loss / d theta
    (float64); r = K e; emulate as in forward (the back-propagated signal
    entering each dense layer's GEMMs is BF16 too).  Q(x) = x.B^-1 x for the
    block preconditioner B; with ssor (K in colour-major order, B the SSOR
    relaxation block inverses) Q(x) = x.M x with
    M = (B^-1 + L) B (B^-1 + U): per node x_i.B_i^-1 x_i + u_i.B_i u_i,
    u = U x, plus 2 x.L x (bfm_gb300/csrc/mpnn.cu, k_loss_terms)."""
    q = bf16 if emulate else _id
    c, cache = forward(theta, f, rp, cols, emulate)
    n = len(c)
    L = chol_inv(Kd)
    Qv, wv = binv_quad(L, c, v.reshape(n, 2))
    Qe, we = binv_quad(L, c, e.reshape(n, 2))
    dc = np.stack([wv[:, 0] ** 2 / Qv - we[:, 0] ** 2 / Qe,
                   2 * (wv[:, 0] * wv[:, 1] / Qv - we[:, 0] * we[:, 1] / Qe),
                   wv[:, 1] ** 2 / Qv - we[:, 1] ** 2 / Qe], 1)
    if ssor:
        Lo, Up = lu_split(K, n)
        qv2, sv = b_quad(L, c, (Up @ v).reshape(n, 2))
        qe2, se = b_quad(L, c, (Up @ e).reshape(n, 2))
        Qv = Qv + qv2 + 2 * v @ (Lo @ v)
        Qe = Qe + qe2 + 2 * e @ (Lo @ e)
        dc = np.stack([wv[:, 0] ** 2 - sv[:, 0] ** 2, 2 * (wv[:, 0] * wv[:, 1] - sv[:, 0] * sv[:, 1]),
                       wv[:, 1] ** 2 - sv[:, 1] ** 2], 1) / Qv - \
            np.stack([we[:, 0] ** 2 - se[:, 0] ** 2, 2 * (we[:, 0] * we[:, 1] - se[:, 0] * se[:, 1]),
                      we[:, 1] ** 2 - se[:, 1] ** 2], 1) / Qe
    loss = np.log(v @ (K @ v)) - np.log(Qv) - np.log(e @ r) + np.log(Qe)
    do = dc * C_SCALE * (1.0 - np.tanh(cache["o"]) ** 2)
    W0, b0, W1, b1, W2, b2, W3, b3, Wo, bo = unpack(theta)
    grads = [None] * 10
    grads[8] = do.T @ cache["hs"][3]
    grads[9] = do.sum(0)
    dh = do @ Wo
    for li, (W, gi) in zip((2, 1, 0), ((W3, 6), (W2, 4), (W1, 2))):
        dpre = q(dh * (cache["hs"][li + 1] > 0))
        grads[gi] = dpre.T @ cache["xs"][li]
        grads[gi + 1] = dpre.sum(0)
        dx = dpre @ q(W)
        dh = dx[:, :H] + mean_agg_T(rp, cols, dx[:, H:])
    dpre = q(dh * (cache["hs"][0] > 0))
    grads[0] = dpre.T @ f
    grads[1] = dpre.sum(0)
    return loss, np.concatenate([g.reshape(-1) for g in grads]), c


def features(p, rp, cols, vals, b):
    """Input features (n, 16) of the network for a meshgen.Problem with its
    assembled 2x2-block CSR operator (rp, cols, vals (nb, 2, 2)) and load
    vector b (2n): the restatement of k_feat1/k_feat2 in
    bfm_gb300/csrc/mpnn.cu, in float64."""
    n = p.n_nodes
    eE = p.elem_E if p.elem_E is not None else np.full(p.n_elems, p.E)
    enu = p.elem_nu if p.elem_nu is not None else np.full(p.n_elems, p.nu)
    le = np.log10(eE)
    cnt = np.bincount(p.elems.reshape(-1), minlength=n).astype(np.float64)
    ids = p.elems.reshape(-1)
    le_rep = np.repeat(le, p.kind)
    nu_rep = np.repeat(enu, p.kind)
    node_le = np.bincount(ids, le_rep, minlength=n)
    node_nu = np.bincount(ids, nu_rep, minlength=n)
    has = cnt > 0
    node_le = np.where(has, node_le / np.maximum(cnt, 1), np.log10(p.E))
    node_nu = np.where(has, node_nu / np.maximum(cnt, 1), p.nu)
    lmin = np.full(n, np.inf)
    lmax = np.full(n, -np.inf)
    np.minimum.at(lmin, ids, le_rep)
    np.maximum.at(lmax, ids, le_rep)
    contrast = np.where(has, lmin - lmax, 0.0)
    deg = np.diff(rp)
    rows = np.repeat(np.arange(n), deg)
    nb_mean = np.bincount(rows, node_le[cols], minlength=n) / deg
    dk = np.zeros((n, 2, 2))
    diag = rows == cols
    dk[rows[diag]] = vals[diag]
    k00, k01, k11 = dk[:, 0, 0], dk[:, 0, 1], dk[:, 1, 1]
    b2 = b.reshape(n, 2)
    z0 = np.where(k00 != 0, b2[:, 0] / np.where(k00 != 0, k00, 1), 0.0)
    z1 = np.where(k11 != 0, b2[:, 1] / np.where(k11 != 0, k11, 1), 0.0)
    rms = np.sqrt((z0 @ z0 + z1 @ z1) / (2.0 * max(n, 1)))
    rms = rms if rms > 0 else 1.0
    z0, z1 = z0 / rms, z1 / rms
    dirx = np.zeros(n, bool)
    diry = np.zeros(n, bool)
    for kind, _, mask in p.conds:
        if kind == 0:
            dirx |= mask
        elif kind == 1:
            diry |= mask
    pos = (k00 > 0) & (k11 > 0)
    f = np.zeros((n, F_IN))
    f[:, 0] = node_le - nb_mean
    f[:, 1] = (node_nu - 0.3) * 10.0
    f[:, 2] = dirx
    f[:, 3] = diry
    f[:, 4] = deg / 9.0
    f[:, 5] = z0
    f[:, 6] = z1
    f[:, 7] = np.where(pos, np.log10(np.where(pos, k00 / np.where(pos, k11, 1), 1)), 0.0)
    f[:, 8] = np.where(pos, k01 / np.sqrt(np.where(pos, k00 * k11, 1)), 0.0)
    f[:, 9] = np.abs(z0) + np.abs(z1)
    f[:, 10] = contrast
    return f
