"""Batched uneven solves: one persistent kernel, one CG per mesh, checked
mesh by mesh against the FP64 direct oracle (displacement error <= 1e-6,
the mixed-precision bound), with the Jacobi and the two-level block Jacobi
preconditioners; the two-level form's iteration counts against its float64
restatement (oracle/ssor_ref.py, TwoLevelJacobi)."""
import os

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import batch as BA, meshgen as M
from oracle import oracle as O
from oracle import ssor_ref as S

pytestmark = pytest.mark.gpu

PCS = [bfm_gb300.PC_JACOBI, bfm_gb300.PC_TWO_LEVEL_JACOBI]
KERNELS = ["block", "tiled"]  # one block per part (default) / the tiled persistent kernel


def make_batch(lib, ps, kernel="block"):
    """A Batch on the given kernel (chosen when the parts are set)."""
    old = os.environ.get("BFM_GPU_BATCH_KERNEL")
    os.environ["BFM_GPU_BATCH_KERNEL"] = kernel
    try:
        return BA.Batch(lib, ps)
    finally:
        if old is None:
            del os.environ["BFM_GPU_BATCH_KERNEL"]
        else:
            os.environ["BFM_GPU_BATCH_KERNEL"] = old


def small_batch(n=12, seed=9):
    rng = np.random.default_rng(seed)
    ps = M.batch_uneven(n, seed=seed)
    # keep the oracle quick: shrink the meshes but keep them uneven
    out = []
    for k, p in enumerate(ps):
        nx, ny = int(rng.integers(8, 40)), int(rng.integers(4, 16))
        coords, elems = M.grid(nx, ny, 3)
        conds = []
        for kind, v, _ in p.conds:
            side = ["left", "right", "bottom", "top"][k % 4] if kind != M.NEUMANN_Y else \
                ["right", "top", "left", "bottom"][k % 4]
            conds.append((kind, v, M.side_mask(coords, side)))
        # tractions before the clamp: a corner node shared by both sides stays clamped
        # (per-edge loads never act on a constrained DOF)
        conds.sort(key=lambda c: c[0] != M.NEUMANN_Y)
        eE = np.exp(rng.uniform(np.log(1e9), np.log(2e11), len(elems)))
        out.append(M.Problem(f"b{k}", 3, coords, elems, nu=p.nu, elem_E=eE, forces=[], conds=conds,
                             edges=M.boundary_edges(nx, ny)))
    return out


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("pc", PCS)
def test_batch_matches_direct_oracle(libbfm, pc, kernel):
    ps = small_batch()
    B = make_batch(libbfm, ps, kernel)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-10, precond=pc))
        st = B.stats()
        xs = B.solutions()
    finally:
        B.close()
    assert np.all(st["status"] == 0), st
    assert np.all(st["rel_residual"] <= 1e-10)
    assert st["rows_per_tile"] in (128, 256, 512, 1024) and st["lanes_per_row"] in (1, 2, 4)
    for p, x in zip(ps, xs):
        ref, _, _ = O.solve_direct(p)
        err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
        assert err <= 1e-6, (p.name, err)
    assert len(set(st["iterations"].tolist())) > 1  # uneven meshes converge at their own pace


@pytest.mark.parametrize("pc", PCS)
def test_batch_rerun_is_bit_identical(libbfm, pc):
    ps = small_batch(6, seed=3)
    B = BA.Batch(libbfm, ps)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=pc))
        x1 = np.concatenate(B.solutions())
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=pc))
        x2 = np.concatenate(B.solutions())
    finally:
        B.close()
    assert np.array_equal(x1, x2)


@pytest.mark.parametrize("pc", PCS)
def test_step_graph_matches_separate_calls(libbfm, pc):
    """bfm_gpu_problem_step_parts (assembly + batched solve captured as one
    graph) gives the solutions of the separate assemble + solve calls, bit for
    bit, on every replay, and captures again when an input changes."""
    ps = small_batch(8, seed=5)
    B = BA.Batch(libbfm, ps)
    try:
        o = bfm_gb300.default_opts(rtol=1e-8, autotune=0, precond=pc)
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(o)
        x0 = np.concatenate(B.solutions())
        for _ in range(3):
            B.step(bfm_gb300.MIXED_EXACT, o)
            st = B.stats()
            assert np.all(st["status"] == 0)
            assert np.array_equal(np.concatenate(B.solutions()), x0)
        # twice the loads: twice the displacements (linear elasticity)
        lo = B.keep[7] * 2.0
        le = B.keep[6]
        assert libbfm.bfm_gpu_problem_set_edge_loads(B.P, len(le), le.ctypes.data, lo.ctypes.data, 0) == 0
        B.keep.append(lo)
        B.step(bfm_gb300.MIXED_EXACT, o)
        x2 = np.concatenate(B.solutions())
        assert np.linalg.norm(x2 - 2 * x0) <= 1e-7 * np.linalg.norm(2 * x0)
    finally:
        B.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_two_level_operator_matches_restatement(libbfm, kernel):
    """The two-level block Jacobi operator itself: after exactly one iteration
    each mesh's solution is alpha M b, so its direction must be that of the
    float64 restatement's M b (oracle/ssor_ref.py, TwoLevelJacobi).  The GPU
    forms A_c from the FP32 operator and A_c^-1 in FP32: agreement to 2e-3."""
    ps = small_batch(10, seed=11)
    B = make_batch(libbfm, ps, kernel)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8, max_iters=1, precond=bfm_gb300.PC_TWO_LEVEL_JACOBI))
        st = B.stats()
        xs = B.solutions()
    finally:
        B.close()
    assert np.all(st["iterations"] == 1)
    worst = 0.0
    for p, x in zip(ps, xs):
        K, b = O.assemble_csr(p)
        z = S.TwoLevelJacobi(K, p.coords, S.free_dofs(K)).apply(b)
        u, v = x / np.linalg.norm(x), z / np.linalg.norm(z)
        worst = max(worst, float(np.linalg.norm(u - v)))
    print(f"two-level operator: worst direction difference {worst:.2e}")
    assert worst <= 2e-3


def test_two_level_iterations_near_restatement(libbfm):
    """Per mesh, the solve's iteration count stays within the FP32 iteration's
    cost over the float64 restatement (at most 1.8x; an emulation of the FP32
    vectors on the CPU shows 1.0-1.7x on these meshes)."""
    ps = small_batch(10, seed=11)
    B = BA.Batch(libbfm, ps)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=bfm_gb300.PC_TWO_LEVEL_JACOBI))
        st = B.stats()
    finally:
        B.close()
    assert np.all(st["status"] == 0)
    for p, it in zip(ps, st["iterations"]):
        K, b = O.assemble_csr(p)
        _, it_ref = S.pcg(K, b, S.TwoLevelJacobi(K, p.coords, S.free_dofs(K)).apply, rtol=1e-8)
        assert 0.8 * it_ref - 3 <= int(it) <= 1.8 * it_ref + 3, (p.name, int(it), it_ref)


def test_two_level_cuts_the_tail(libbfm):
    """On full-size uneven plates (the batched workload's generator) the
    coarse space takes the slowest mesh from several times the median
    iteration count to within twice it, and every mesh still converges."""
    ps = M.batch_uneven(24, seed=4)
    B = BA.Batch(libbfm, ps)
    its = {}
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        for pc in PCS:
            B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=pc))
            st = B.stats()
            assert np.all(st["status"] == 0) and np.all(st["rel_residual"] <= 1e-8), (pc, st)
            its[pc] = st["iterations"]
    finally:
        B.close()
    jac, two = its[bfm_gb300.PC_JACOBI], its[bfm_gb300.PC_TWO_LEVEL_JACOBI]
    print(f"jacobi {int(np.median(jac))}/{int(jac.max())}, two-level {int(np.median(two))}/{int(two.max())} (median/max)")
    assert two.max() * 3 <= jac.max()
    assert two.max() <= 2 * np.median(two)


@pytest.mark.parametrize("pc", PCS)
def test_block_and_tiled_kernels_agree(libbfm, pc):
    """The block-per-part kernel and the tiled persistent kernel run the same
    iteration: every mesh converges in both, with solutions within the
    mixed-precision bound of each other and about the same iteration counts."""
    ps = small_batch(12, seed=21)
    out = {}
    for kernel in KERNELS:
        B = make_batch(libbfm, ps, kernel)
        try:
            B.assemble(bfm_gb300.MIXED_EXACT)
            B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=pc))
            out[kernel] = (B.stats(), np.concatenate(B.solutions()))
        finally:
            B.close()
    (sb, xb), (st, xt) = out["block"], out["tiled"]
    assert np.all(sb["status"] == 0) and np.all(st["status"] == 0)
    assert np.linalg.norm(xb - xt) <= 1e-6 * np.linalg.norm(xt)
    assert np.all(np.abs(sb["iterations"] - st["iterations"]) <= 0.1 * st["iterations"] + 5)
