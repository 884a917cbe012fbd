"""Learned block preconditioner on the GPU: features, forward pass, loss and
gradients of the tensor-core kernels against the float64 oracle
(oracle/mpnn_ref.py, with the GPU's BF16 rounding points emulated) in the
block-Jacobi and the SSOR contexts, Adam training, the solve with the learned
blocks, the Jacobi fallback, and what a trained network gains over
Jacobi-PCG."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg  # noqa: F401 (sp.linalg)

import bfm_gb300
from bfm_gb300 import learned as LN, meshgen as M
from oracle import mpnn_ref as R

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def soft_plate(nx=48, ny=12, seed=11):
    """P1 plate, left edge clamped, traction on the right edge, gravity,
    per-element E log-uniform in [1e9, 2e11] (seeded)."""
    p = M.plate(nx, ny, 3, name=f"soft_{nx}x{ny}", traction=1e6)
    p.elem_E = np.exp(np.random.default_rng(seed).uniform(np.log(1e9), np.log(2e11), p.n_elems))
    return p


def scalar_K(rp, cols, vals, n):
    nb = len(cols)
    rows = np.repeat(np.arange(n), np.diff(rp))
    R_ = np.repeat(2 * rows, 4) + np.tile([0, 0, 1, 1], nb)
    C_ = np.repeat(2 * cols, 4) + np.tile([0, 1, 0, 1], nb)
    return sp.csr_matrix((vals.reshape(-1), (R_, C_)), shape=(2 * n, 2 * n))


def diag_blocks(rp, cols, vals, n):
    rows = np.repeat(np.arange(n), np.diff(rp))
    d = rows == cols
    out = np.zeros((n, 2, 2))
    out[rows[d]] = vals[d]
    return out


def random_theta(net, seed, head=0.3):
    """The network's initial weights with a random non-zero head (so c varies)."""
    th = net.weights().astype(np.float64)
    rng = np.random.default_rng(seed)
    o = R.N_PARAMS - (3 * R.H + 3)
    th[o:] = rng.normal(0.0, head, 3 * R.H + 3) / np.sqrt(R.H)
    th[o + 3 * R.H:] = rng.normal(0.0, 0.2, 3)
    th[:o] += rng.normal(0.0, 0.01, o)   # non-zero biases too
    return th.astype(np.float32)


@pytest.fixture(scope="module")
def setup(libbfm):
    p = soft_plate()
    prob = LN.DeviceProblem(p)
    rp, cols, vals, b = prob.download()
    net = LN.Network(seed=3)
    yield p, prob, net, (rp, cols, vals, b)
    net.close()
    prob.close()


def test_features_match_oracle(setup):
    p, prob, net, (rp, cols, vals, b) = setup
    f_gpu, _, _ = net.forward(prob)
    f_ref = R.features(p, rp, cols, vals, b)
    # BF16 inputs: half a BF16 ulp of the reference value (plus double-rounding ties)
    tol = 2.0 ** -8 * np.abs(f_ref) + 1e-6
    bad = np.abs(f_gpu - f_ref) > tol
    assert not bad.any(), (np.argwhere(bad)[:5], f_gpu[bad][:5], f_ref[bad][:5])
    assert np.count_nonzero(f_gpu[:, 11:]) == 0


def test_untrained_network_is_block_jacobi(setup):
    p, prob, net, (rp, cols, vals, b) = setup
    _, c, B = net.forward(prob)
    assert np.all(c == 0.0)
    Kd = diag_blocks(rp, cols, vals, p.n_nodes)
    np.testing.assert_allclose(B, np.linalg.inv(Kd), rtol=1e-13, atol=0)


def test_forward_matches_oracle(setup):
    p, prob, net, (rp, cols, vals, b) = setup
    th = random_theta(net, 1)
    init = net.weights()
    net.set_weights(th)
    try:
        f_gpu, c_gpu, B_gpu = net.forward(prob)
        c_ref, _ = R.forward(th.astype(np.float64), f_gpu.astype(np.float64), rp, cols, emulate=True)
        assert np.abs(c_ref).max() > 0.05
        # FP32 accumulation order differs from float64: 1e-3 of the output scale
        assert np.abs(c_gpu - c_ref).max() <= 1e-3 * R.C_SCALE
        B_ref = R.blocks(c_ref, diag_blocks(rp, cols, vals, p.n_nodes))
        assert np.linalg.norm(B_gpu - B_ref) <= 5e-3 * np.linalg.norm(B_ref)
        # every block SPD: 1 + c0 > 0 and det(I + C) > 0 for |c| < 0.45
        det = B_gpu[:, 0, 0] * B_gpu[:, 1, 1] - B_gpu[:, 0, 1] ** 2
        assert (B_gpu[:, 0, 0] > 0).all() and (det > 0).all()
    finally:
        net.set_weights(init)


def test_tcgen05_and_mma_layers_agree(setup):
    """The forward dense layers on the tcgen05 tensor cores (the default) and
    on the warp-level mma.sync path (BFM_GPU_MPNN_GEMM=mma) give the same
    network output up to FP32 accumulation order (1e-3 of the output scale,
    as against the oracle), on a mesh whose node count is not a multiple of
    the 128-node tile."""
    import os
    p, prob, net, _ = setup
    assert p.n_nodes % 128 != 0
    th = random_theta(net, 2)
    init = net.weights()
    net.set_weights(th)
    old = os.environ.get("BFM_GPU_MPNN_GEMM")
    try:
        os.environ.pop("BFM_GPU_MPNN_GEMM", None)
        _, c_tc, B_tc = net.forward(prob)
        os.environ["BFM_GPU_MPNN_GEMM"] = "mma"
        _, c_mma, B_mma = net.forward(prob)
    finally:
        if old is None:
            os.environ.pop("BFM_GPU_MPNN_GEMM", None)
        else:
            os.environ["BFM_GPU_MPNN_GEMM"] = old
        net.set_weights(init)
    assert np.abs(c_mma).max() > 0.05
    assert np.abs(c_tc - c_mma).max() <= 1e-3 * R.C_SCALE
    assert np.linalg.norm(B_tc - B_mma) <= 5e-3 * np.linalg.norm(B_mma)


@pytest.fixture(scope="module")
def pair(setup):
    """(r, e, v): a solver pair and a power vector of B K (60 steps, untrained network)."""
    p, prob, net, _ = setup
    prs = LN.pairs(prob, stops=(256,))
    assert prs
    r, e = prs[0]
    gen = torch.Generator(device="cuda").manual_seed(0)
    v = torch.rand(2 * p.n_nodes, dtype=torch.float64, device="cuda", generator=gen) - 0.5
    torch.cuda.synchronize()
    net.gradient(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 60)
    return r, e, v


def test_gradient_matches_oracle(setup, pair):
    p, prob, net, (rp, cols, vals, b) = setup
    r, e, v = pair
    th = random_theta(net, 2)
    init = net.weights()
    net.set_weights(th)
    try:
        f_gpu, _, _ = net.forward(prob)
        loss_gpu, g_gpu = net.gradient(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 0)
        K = scalar_K(rp, cols, vals, p.n_nodes)
        args = (th.astype(np.float64), f_gpu.astype(np.float64), rp, cols, K, diag_blocks(rp, cols, vals, p.n_nodes),
                r.cpu().numpy(), e.cpu().numpy(), v.cpu().numpy())
        loss_ref, g_ref, _ = R.loss_and_grad(*args, emulate=True)
        assert loss_gpu > 0.0          # log of a condition-number estimate
        assert abs(loss_gpu - loss_ref) <= 1e-4 * max(1.0, abs(loss_ref))
        # every parameter block, relative to its own norm: BF16 storage emulated, FP32 sums
        k = 0
        for shape in R.SHAPES:
            n = int(np.prod(shape))
            gg, gr = g_gpu[k:k + n], g_ref[k:k + n]
            assert np.linalg.norm(gg - gr) <= 2e-2 * np.linalg.norm(gr) + 1e-12, (shape, k)
            k += n
        # and the float64 network without any BF16 rounding: same direction
        _, g64, _ = R.loss_and_grad(*args, emulate=False)
        cos = g_gpu @ g64 / (np.linalg.norm(g_gpu) * np.linalg.norm(g64))
        assert cos > 0.98
    finally:
        net.set_weights(init)


def test_training_lowers_the_loss(setup, pair):
    p, prob, _, _ = setup
    r, e, v = pair
    net = LN.Network(seed=4)
    try:
        # fixed power vector: the condition-number estimate falls by at least 5%
        losses = [net.train_step(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 1e-3, 0) for _ in range(60)]
        assert np.isfinite(losses).all()
        assert np.mean(losses[-10:]) < np.mean(losses[:10]) - np.log(1.05)
    finally:
        net.close()


def test_save_load_roundtrip(setup, tmp_path):
    _, _, net, _ = setup
    th = random_theta(net, 5)
    other = LN.Network(seed=9)
    try:
        other.set_weights(th)
        other.save(tmp_path / "w.bin")
        third = LN.Network(seed=10, path=tmp_path / "w.bin")
        np.testing.assert_array_equal(third.weights(), th)
        third.close()
        (tmp_path / "bad.bin").write_bytes(b"not a network")
        lib = bfm_gb300.lib()
        assert lib.bfm_gpu_mpnn_load(other.h, str(tmp_path / "bad.bin").encode()) == -1
        assert "network file" in bfm_gb300.last_error()
    finally:
        other.close()


@pytest.mark.parametrize("precision", [bfm_gb300.FP64, bfm_gb300.MIXED_EXACT, bfm_gb300.FP64_DF])
def test_untrained_learned_solve_equals_block_jacobi(libbfm, precision):
    p = soft_plate(64, 16, seed=12)
    prob = LN.DeviceProblem(p, precision=precision)
    net = LN.Network(seed=0)
    try:
        net.use()
        sj = prob.solve(precond=bfm_gb300.PC_BLOCK_JACOBI, rtol=1e-8)
        xj = prob.solution()
        sl = prob.solve(precond=bfm_gb300.PC_LEARNED, rtol=1e-8)
        xl = prob.solution()
        assert sj.status == 0 and sl.status == 0 and sl.fallback == 0
        assert sl.iterations == sj.iterations
        np.testing.assert_array_equal(xl, xj)
    finally:
        net.close()
        prob.close()


def test_learned_without_network_is_an_error(libbfm):
    prob = LN.DeviceProblem(soft_plate(16, 4))
    try:
        libbfm.bfm_gpu_mpnn_use(None)
        o = bfm_gb300.default_opts(precond=bfm_gb300.PC_LEARNED)
        import ctypes as C
        assert libbfm.bfm_gpu_problem_solve(prob.P, C.byref(o)) == -1
        assert "network" in bfm_gb300.last_error()
    finally:
        prob.close()


def test_nan_network_falls_back_to_jacobi(libbfm):
    """Fault injection on the host: non-finite network output -> breakdown of
    the learned solve -> Jacobi takes over and converges."""
    p = soft_plate(64, 16, seed=13)
    prob = LN.DeviceProblem(p)
    net = LN.Network(seed=0)
    try:
        th = net.weights()
        th[-1] = np.nan
        net.set_weights(th)
        net.use()
        sj = prob.solve(precond=bfm_gb300.PC_JACOBI, rtol=1e-8)
        xj = prob.solution()
        s = prob.solve(precond=bfm_gb300.PC_LEARNED, rtol=1e-8)
        assert s.fallback == 1 and s.status == 0
        assert s.iterations == sj.iterations
        np.testing.assert_allclose(prob.solution(), xj, rtol=0, atol=1e-12 * np.abs(xj).max())
    finally:
        net.close()
        prob.close()


def test_trained_network_beats_jacobi(libbfm):
    """The gain test: a network trained here on solver-generated pairs from
    small uneven plates and perforated plates cuts the PCG iterations of a
    held-out perforated plate below Jacobi's, at the same accuracy."""
    train_meshes = LN.training_meshes(21, n_plates=1, n_batch=1, batch_parts=6)
    train_meshes[0] = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=22)
    probs = [LN.DeviceProblem(q) for q in train_meshes]
    held = LN.DeviceProblem(M.cfg_perforated(nx=384, ny=96, n_holes=200, seed=3))
    net = LN.Network(seed=5)
    try:
        hist, n = LN.train(net, probs, 1500, lr=1e-3, epochs=1, seed=1)
        ev = LN.evaluate(net, held, rtol=1e-8)
        print("gain test:", hist, ev)
        assert ev["learned"]["status"] == 0 and ev["learned"]["fallback"] == 0
        assert ev["learned"]["rel_residual"] <= 1e-8
        assert ev["learned"]["iterations"] < ev["jacobi"]["iterations"]
        # training moves it from its block-Jacobi start without losing ground
        assert ev["learned"]["iterations"] <= ev["block_jacobi"]["iterations"]
    finally:
        net.close()
        for q in probs:
            q.close()
        held.close()


@pytest.fixture(scope="module")
def ssor_setup(libbfm):
    """A soft plate in the SSOR preconditioner's colour order, with one SSOR
    training pair and a power vector of M^-1 K (40 steps, untrained network)."""
    p = soft_plate(seed=14)
    prob = LN.DeviceProblem(p)
    net = LN.Network(seed=3)
    r, e = LN.pairs(prob, stops=(64,), ssor=True)[0]
    gen = torch.Generator(device="cuda").manual_seed(0)
    v = torch.rand(2 * p.n_nodes, dtype=torch.float64, device="cuda", generator=gen) - 0.5
    torch.cuda.synchronize()
    net.gradient(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 40)
    yield p, prob, net, (r, e, v)
    net.close()
    prob.close()


def test_ssor_gradient_matches_oracle(ssor_setup):
    """SSOR context (relaxation blocks): the loss x.M x terms and their
    gradients on the GPU against oracle/mpnn_ref.py with ssor=True, the
    matrix in the problem's colour-major working order."""
    p, prob, net, (r, e, v) = ssor_setup
    th = random_theta(net, 6)
    init = net.weights()
    net.set_weights(th)
    try:
        f_gpu, _, _ = net.forward(prob)
        loss_gpu, g_gpu = net.gradient(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 0)
        rp, cols, vals, b = prob.download()
        K = scalar_K(rp, cols, vals, p.n_nodes)
        args = (th.astype(np.float64), f_gpu.astype(np.float64), rp, cols, K, diag_blocks(rp, cols, vals, p.n_nodes),
                r.cpu().numpy(), e.cpu().numpy(), v.cpu().numpy())
        loss_ref, g_ref, _ = R.loss_and_grad(*args, emulate=True, ssor=True)
        assert abs(loss_gpu - loss_ref) <= 1e-4 * max(1.0, abs(loss_ref))
        assert np.linalg.norm(g_gpu - g_ref) <= 2e-2 * np.linalg.norm(g_ref)
        # a different objective from the block-Jacobi one
        loss_j, _, _ = R.loss_and_grad(*args, emulate=True)
        assert abs(loss_j - loss_ref) > 1e-3
    finally:
        net.set_weights(init)


def test_ssor_power_vector_is_bounded_by_one(ssor_setup):
    """With the untrained network (block SSOR, symmetric Gauss-Seidel) the
    spectrum of M^-1 K lies in (0, 1] (M - K = L D^-1 U is semidefinite): the
    power vector's Rayleigh quotient x.Kx / x.Mx is at most 1, and near the
    top of the spectrum."""
    p, prob, net, (r, e, v) = ssor_setup
    loss, _ = net.gradient(prob, r.data_ptr(), e.data_ptr(), v.data_ptr(), 20)
    rp, cols, vals, b = prob.download()
    K = scalar_K(rp, cols, vals, p.n_nodes)
    vv = v.cpu().numpy()
    Lo, Up = R.lu_split(K, p.n_nodes)
    Kd = diag_blocks(rp, cols, vals, p.n_nodes)
    D = sp.block_diag(list(Kd), format="csr")
    Mv = (D + Lo) @ sp.linalg.spsolve(D.tocsc(), (D + Up) @ vv)
    ratio = (vv @ (K @ vv)) / (vv @ Mv)
    assert 0.3 < ratio <= 1.0 + 1e-9
