"""Multicolour block SSOR on the GPU: the colour-major renumbering (a valid
colouring, K and b permuted bit for bit, the solution back in the caller's
order), the solve against the FP64 direct oracle in FP64 and double-float,
the iteration count against the float64 restatement (oracle/ssor_ref.py), the
learned relaxation blocks, and switching preconditioners on one problem."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import bfm_gb300
from bfm_gb300 import api, learned as LN, meshgen as M
from common import load, rel
from oracle import oracle as O, ssor_ref as S

pytestmark = pytest.mark.gpu


def plate(nx=96, ny=24, seed=3):
    return M.cfg_perforated(nx=nx, ny=ny, n_holes=40, seed=seed)


def ordering(prob):
    L = prob.lib
    n = prob.n_nodes
    perm = np.zeros(n, np.int32)
    off = np.zeros(65, np.int32)
    nc = C.c_int()
    assert L.bfm_gpu_problem_ordering(prob.P, perm.ctypes.data, off.ctypes.data, C.byref(nc)) == 0
    return perm, off[:nc.value + 1], nc.value


def scalar(rp, cols, vals, n):
    rows = np.repeat(np.arange(n), np.diff(rp))
    R_ = np.repeat(2 * rows, 4) + np.tile([0, 0, 1, 1], len(cols))
    C_ = np.repeat(2 * cols, 4) + np.tile([0, 1, 0, 1], len(cols))
    return sp.csr_matrix((vals.reshape(-1), (R_, C_)), shape=(2 * n, 2 * n))


@pytest.fixture(scope="module")
def problem(libbfm):
    p = plate()
    prob = LN.DeviceProblem(p)
    yield p, prob
    prob.close()


def test_colour_order_and_permuted_system(problem):
    p, prob = problem
    prob.solve(precond=bfm_gb300.PC_JACOBI, rtol=1e-8)
    rp0, c0, v0, b0 = prob.download()
    perm0, _, nc0 = ordering(prob)
    assert nc0 == 0 and np.array_equal(perm0, np.arange(p.n_nodes))
    s = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
    assert s.status == 0
    perm, off, nc = ordering(prob)
    assert 2 <= nc <= 8 and off[0] == 0 and off[-1] == p.n_nodes
    assert np.array_equal(np.sort(perm), np.arange(p.n_nodes))
    K0 = scalar(rp0, c0, v0, p.n_nodes)
    assert S.is_colouring(S.node_graph(K0, p.n_nodes), perm, off)
    # inside every colour the nodes go by coarse cell (each cell one contiguous
    # run), then by ascending caller index
    cell = S.cell_grid(np.asarray(p.coords, dtype=np.float64))[0]
    assert len(np.unique(cell)) >= 2
    for c in range(nc):
        seg = perm[off[c]:off[c + 1]]
        cs = cell[seg]
        starts = np.flatnonzero(np.r_[True, cs[1:] != cs[:-1]])
        assert len(starts) == len(np.unique(cs))
        for a, b in zip(starts, np.r_[starts[1:], len(seg)]):
            assert np.all(np.diff(seg[a:b]) > 0)
    # the working system is P K P^T and P b, bit for bit
    rp, cols, vals, b = prob.download()
    dperm = np.stack([2 * perm, 2 * perm + 1], 1).ravel()
    K = scalar(rp, cols, vals, p.n_nodes)
    assert (K != K0[dperm][:, dperm]).nnz == 0
    assert np.array_equal(b, b0[dperm])
    # every row: lower-colour blocks, the diagonal, higher-colour blocks
    rows = np.repeat(np.arange(p.n_nodes), np.diff(rp))
    assert np.all(np.diff(cols)[np.diff(rows) == 0] > 0)


@pytest.mark.parametrize("precision,tol", [(bfm_gb300.FP64, 1e-10), (bfm_gb300.FP64_DF, 1e-8)])
def test_ssor_solve_matches_direct_oracle(libbfm, precision, tol):
    p = plate(seed=5)
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        sj = prob.solve(precond=bfm_gb300.PC_JACOBI, rtol=1e-10)
        s = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-10)
        assert s.status == 0 and s.rel_residual <= 1e-10
        x, _, _ = O.solve_direct(p)
        assert rel(prob.solution(), x) < tol
        # the point of it: well under half of Jacobi's iterations
        assert s.iterations < 0.5 * sj.iterations, (s.iterations, sj.iterations)
    finally:
        prob.close()


@pytest.mark.parametrize("precision", [bfm_gb300.FP64, bfm_gb300.FP64_DF])
def test_iterations_match_the_restatement(libbfm, precision):
    """CG with the GPU's sweeps vs float64 CG with the float64 restatement of
    the same preconditioner (same colouring): the counts agree within a few
    per cent."""
    p = plate(seed=4)
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        s = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        assert s.status == 0
        perm, off, _ = ordering(prob)
        K, b = O.assemble_csr(p)
        pc = S.BlockSSOR(K, perm, off)
        x, it = S.pcg(sp.csr_matrix(K), b, pc.apply, rtol=1e-8)
        assert abs(s.iterations - it) <= max(3, 0.1 * it), (s.iterations, it)
        assert rel(prob.solution(), x) < 1e-6
    finally:
        prob.close()


def test_untrained_learned_ssor_is_block_ssor(libbfm):
    p = plate(seed=7)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    net = LN.Network(seed=0)
    try:
        net.use()
        s0 = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        x0 = prob.solution()
        s1 = prob.solve(precond=bfm_gb300.PC_LEARNED_SSOR, rtol=1e-8)
        assert s1.status == 0 and s1.fallback == 0 and s1.iterations == s0.iterations
        np.testing.assert_array_equal(prob.solution(), x0)
    finally:
        net.close()
        prob.close()


def test_nan_network_falls_back_to_block_ssor(libbfm):
    p = plate(seed=8)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    net = LN.Network(seed=0)
    try:
        th = net.weights()
        th[-1] = np.nan
        net.set_weights(th)
        net.use()
        s0 = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        s1 = prob.solve(precond=bfm_gb300.PC_LEARNED_SSOR, rtol=1e-8)
        assert s1.fallback == 1 and s1.status == 0 and s1.iterations == s0.iterations
    finally:
        net.close()
        prob.close()


def test_switching_back_restores_the_caller_order(problem):
    p, prob = problem
    s1 = prob.solve(precond=bfm_gb300.PC_JACOBI, rtol=1e-8)
    x1 = prob.solution()
    prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
    s2 = prob.solve(precond=bfm_gb300.PC_JACOBI, rtol=1e-8)
    assert ordering(prob)[2] == 0
    assert s2.iterations == s1.iterations
    np.testing.assert_array_equal(prob.solution(), x1)


@pytest.mark.parametrize("precision,tol", [(bfm_gb300.MIXED_EXACT, 1e-6), (bfm_gb300.MIXED, 1e-4)])
@pytest.mark.parametrize("precond", [bfm_gb300.PC_SSOR, bfm_gb300.PC_SSOR2])
def test_mixed_ssor_matches_direct_oracle(libbfm, precision, tol, precond):
    """The mixed precisions with the SSOR preconditioners: FP32 operator,
    vectors and sweeps' input and output, FP64 dots; every FP64 residual
    replacement is an iterative-refinement step (the inner PCG keeps its
    direction by default).  MIXED_EXACT solves the FP64 system (error bound of
    the refinement), MIXED its FP32-integrated one (error bound of the FP32
    element integration).  The iteration count stays within 30% of the FP64
    solve's with the two-level preconditioner; with plain SSOR, whose solve
    takes several times more iterations, the FP32 vectors cost more (under 2x
    measured: 1,335 against 765)."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    ref = LN.DeviceProblem(p, precision=bfm_gb300.FP64)
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        s64 = ref.solve(precond=precond, rtol=1e-8)
        s = prob.solve(precond=precond, rtol=1e-8, replace_drop=0.01)
        assert s.status == 0 and s.rel_residual <= 1e-8, (s.status, s.rel_residual)
        assert s.replacements >= 2  # refinement steps
        x, _, _ = O.solve_direct(p)
        assert rel(prob.solution(), x) < tol
        bound = 1.3 if precond == bfm_gb300.PC_SSOR2 else 2.0
        assert s.iterations <= bound * s64.iterations, (s.iterations, s64.iterations)
    finally:
        prob.close()
        ref.close()


def test_mixed_refinement_keeps_or_restarts(libbfm):
    """refine_restart: 0 keeps the inner PCG's direction across refinement
    steps, 1 restarts it; both reach the solution of the FP64 system."""
    p = M.cfg_perforated(nx=192, ny=48, n_holes=100, seed=6)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.MIXED_EXACT)
    try:
        x, _, _ = O.solve_direct(p)
        for restart in (0, 1):
            s = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-8, replace_drop=0.01, refine_restart=restart)
            print(f"refine_restart {restart}: {s.iterations} iterations, {s.replacements} refinement steps")
            assert s.status == 0 and s.replacements >= 2
            assert rel(prob.solution(), x) < 1e-6
    finally:
        prob.close()


@pytest.mark.parametrize("name", ["p1_16x8_nt", "q1_24x8_jitter", "axi_p1_12x8", "lepl8", "gear12"])
def test_sim_run_with_ssor(libbfm, name, monkeypatch):
    """Through bfm_sim_run with the SSOR preconditioner: all condition kinds,
    Q1, the axisymmetric element and the reference's own unstructured meshes,
    against the FP64 direct oracle."""
    monkeypatch.setenv("BFM_GPU_AXISYM_REFERENCE", "0")
    p, _ = load(name)
    if p.stress == 3:
        p.stress = 2
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-12, precond=bfm_gb300.PC_SSOR)))
    try:
        h = api.SimHandle.from_problem(libbfm, p)
        assert h.run() == 0, h.error()
        x, _, _ = O.solve_direct(p)
        assert rel(h.effects(), x) < 1e-9
    finally:
        libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


def test_colouring_is_reused_for_the_same_mesh(libbfm):
    """Three colours on a triangle plate (DSATUR); uploading the same element
    array again keeps the colouring, a different one makes a new one."""
    p = plate(seed=9)
    prob = LN.DeviceProblem(p)
    try:
        prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        perm1, off1, nc1 = ordering(prob)
        assert nc1 == 3
        el = np.ascontiguousarray(p.elems, dtype=np.int32)
        xy = np.ascontiguousarray(p.coords, dtype=np.float64)
        assert libbfm.bfm_gpu_problem_set_geometry(prob.P, xy.ctypes.data, el.ctypes.data, 0) == 0
        prob.assemble(bfm_gb300.FP64)
        s = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        perm2, off2, _ = ordering(prob)
        assert s.status == 0 and np.array_equal(perm1, perm2) and np.array_equal(off1, off2)
        # flip the diagonal of one grid square: another graph, another colouring
        el2 = el.copy()
        el2[0], el2[1] = [el[0][0], el[0][1], el[1][2]], [el[0][1], el[0][2], el[1][2]]
        assert libbfm.bfm_gpu_problem_set_geometry(prob.P, xy.ctypes.data, el2.ctypes.data, 0) == 0
        prob.assemble(bfm_gb300.FP64)
        s = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-8)
        perm3, off3, _ = ordering(prob)
        assert s.status == 0
        p2 = M.Problem(p.name, 3, p.coords, el2, E=p.E, nu=p.nu, rho=p.rho, stress=p.stress, forces=p.forces,
                       conds=p.conds, edges=p.edges, elem_E=p.elem_E)
        K2, _ = O.assemble_csr(p2)
        assert S.is_colouring(S.node_graph(sp.csr_matrix(K2), p.n_nodes), perm3, off3)
    finally:
        prob.close()


@pytest.mark.parametrize("precision", [bfm_gb300.FP64, bfm_gb300.FP64_DF])
def test_per_colour_kernels_match_the_persistent_kernel(libbfm, precision, monkeypatch):
    """The per-colour launches (used where a graph cannot hold a cooperative
    node) compute the same sweeps as the persistent kernel: same solution to
    rounding, same iteration count to a couple of iterations (only the order
    of the partial sums of (r, z) differs)."""
    p = plate(seed=11)
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        s1 = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-10)
        x1 = prob.solution()
    finally:
        prob.close()
    monkeypatch.setenv("BFM_GPU_SSOR_PER_COLOUR", "1")
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        s2 = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-10)
        persistent = C.c_int(-1)
        t = C.c_double()
        assert libbfm.bfm_gpu_problem_time_precond(prob.P, 2, C.byref(t), None, C.byref(persistent)) == 0
        assert persistent.value == 0
        x2 = prob.solution()
    finally:
        prob.close()
    assert s1.status == 0 and s2.status == 0
    assert abs(s1.iterations - s2.iterations) <= 2
    assert rel(x2, x1) < 1e-9


@pytest.mark.parametrize("precision,tol", [(bfm_gb300.FP64, 1e-10), (bfm_gb300.FP64_DF, 1e-8)])
def test_two_level_matches_direct_oracle_and_restatement(libbfm, precision, tol):
    """Two-level SSOR (additive rigid-body coarse correction on a cell grid)
    on a 256x64 plate (8 x 2 cells): the solution against the direct oracle, the
    iteration count against the float64 restatement with the GPU's own
    colouring, and fewer iterations than plain SSOR."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    prob = LN.DeviceProblem(p, precision=precision)
    try:
        s1 = prob.solve(precond=bfm_gb300.PC_SSOR, rtol=1e-10)
        s2 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
        assert s2.status == 0 and s2.rel_residual <= 1e-10
        x, _, _ = O.solve_direct(p)
        assert rel(prob.solution(), x) < tol
        # 16 cells only at this size; the 2048x512 plate's 1,024 cells cut 6,172 iterations to about 330
        assert s2.iterations < 0.6 * s1.iterations, (s2.iterations, s1.iterations)
        perm, off, _ = ordering(prob)
        K, b = O.assemble_csr(p)
        K = sp.csr_matrix(K)
        tl = S.TwoLevel(K, p.coords, S.free_dofs(K), S.BlockSSOR(K, perm, off))
        _, it = S.pcg(K, b, tl.apply, rtol=1e-10)
        assert abs(s2.iterations - it) <= max(3, 0.1 * it), (s2.iterations, it)
    finally:
        prob.close()


def test_two_level_one_launch_matches_separate_kernels(libbfm, monkeypatch):
    """The coarse correction as one cooperative launch (with the persistent
    sweeps) and as separate kernels (with the per-colour sweeps): the same
    arithmetic, so the same iterations and solution up to the order of the
    sweeps' dot products."""
    p = M.cfg_perforated(nx=192, ny=48, n_holes=60, seed=8)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    try:
        s1 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
        x1 = prob.solution()
    finally:
        prob.close()
    monkeypatch.setenv("BFM_GPU_SSOR_PER_COLOUR", "1")
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    try:
        s2 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
        x2 = prob.solution()
    finally:
        prob.close()
    assert s1.status == 0 and s2.status == 0
    assert abs(s1.iterations - s2.iterations) <= 2, (s1.iterations, s2.iterations)
    assert rel(x2, x1) < 1e-9


def test_two_level_denser_grid(libbfm, monkeypatch):
    """BFM_GPU_COARSE_NODES=300 on a 256x64 plate (15 x 4 cells instead of 8 x 2):
    still the direct oracle's solution, and fewer iterations than the default
    grid."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    try:
        s1 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
    finally:
        prob.close()
    monkeypatch.setenv("BFM_GPU_COARSE_NODES", "300")
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    try:
        s2 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
        assert s2.status == 0 and s2.rel_residual <= 1e-10
        x, _, _ = O.solve_direct(p)
        assert rel(prob.solution(), x) < 1e-8
        assert s2.iterations < s1.iterations, (s2.iterations, s1.iterations)
    finally:
        prob.close()


def test_untrained_learned_two_level_is_two_level(libbfm):
    p = M.cfg_perforated(nx=128, ny=32, n_holes=40, seed=6)
    prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
    net = LN.Network(seed=0)
    try:
        net.use()
        s0 = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-8)
        x0 = prob.solution()
        s1 = prob.solve(precond=bfm_gb300.PC_LEARNED_SSOR2, rtol=1e-8)
        assert s1.status == 0 and s1.fallback == 0 and s1.iterations == s0.iterations
        np.testing.assert_array_equal(prob.solution(), x0)
    finally:
        net.close()
        prob.close()


@pytest.mark.parametrize("name", ["p1_16x8_nt", "q1_24x8_jitter", "axi_p1_12x8", "lepl8", "gear12"])
def test_sim_run_with_two_level(libbfm, name, monkeypatch):
    """bfm_sim_run with the two-level SSOR on every fixture (a single cell on
    the small meshes: the coarse space is the three rigid-body modes of the
    whole body; three on gear12, some of them nearly empty), against the FP64
    direct oracle."""
    monkeypatch.setenv("BFM_GPU_AXISYM_REFERENCE", "0")
    p, _ = load(name)
    if p.stress == 3:
        p.stress = 2
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-12, precond=bfm_gb300.PC_SSOR2)))
    try:
        h = api.SimHandle.from_problem(libbfm, p)
        assert h.run() == 0, h.error()
        x, _, _ = O.solve_direct(p)
        assert rel(h.effects(), x) < 1e-9
    finally:
        libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


def test_blocked_coarse_inverse_matches_columnwise(libbfm, monkeypatch):
    """X = L^-1 of the coarse factor by block rows (the default: the block-row
    recurrence in FP32, X being stored in FP32) and column by column in
    double-float (BFM_GPU_COARSE_LINV_COLUMNS=1): the same matrix to about
    FP32 rounding, so the same iterations (within 2) and solution."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    out = []
    for cols in ("0", "1"):
        monkeypatch.setenv("BFM_GPU_COARSE_LINV_COLUMNS", cols)
        prob = LN.DeviceProblem(p, precision=bfm_gb300.FP64_DF)
        try:
            s = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=1e-10)
            assert s.status == 0
            out.append((s.iterations, prob.solution()))
        finally:
            prob.close()
    assert abs(out[0][0] - out[1][0]) <= 2, (out[0][0], out[1][0])
    assert rel(out[0][1], out[1][1]) < 1e-9


@pytest.mark.parametrize("precision,rtol,tol", [(bfm_gb300.FP64_DF, 1e-10, 1e-9), (bfm_gb300.MIXED, 1e-8, 1e-7)])
def test_sweep_kernel_stage_tables_match_fallbacks(libbfm, monkeypatch, precision, rtol, tol):
    """The TMA sweep kernel's coarse stages with their shared-memory tables
    (the host-built work list of the triangular products, the restriction's
    chunk table: the default) and with the fallbacks a grid or coarse space
    too large for the tables takes (one warp per row of X, the restriction's
    global arrays; BFM_GPU_SSOR_STAGE_TABLES=0): the same operators summed
    in other orders, so the same iterations (within 2) and solution."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    out = []
    for tables in ("1", "0"):
        monkeypatch.setenv("BFM_GPU_SSOR_STAGE_TABLES", tables)
        prob = LN.DeviceProblem(p, precision=precision)
        try:
            s = prob.solve(precond=bfm_gb300.PC_SSOR2, rtol=rtol, replace_drop=0.1)
            assert s.status == 0 and s.rel_residual <= rtol, (s.status, s.rel_residual)
            out.append((s.iterations, prob.solution()))
        finally:
            prob.close()
    assert abs(out[0][0] - out[1][0]) <= 2, (out[0][0], out[1][0])
    assert rel(out[0][1], out[1][1]) < tol
