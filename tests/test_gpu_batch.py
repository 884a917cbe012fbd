"""Batched uneven solves: one persistent kernel, one CG per mesh, checked
mesh by mesh against the FP64 direct oracle (displacement error <= 1e-6,
the mixed-precision bound)."""
import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import batch as BA, meshgen as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


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


def test_batch_matches_direct_oracle(libbfm):
    ps = small_batch()
    B = BA.Batch(libbfm, ps)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-10))
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


def test_batch_rerun_is_bit_identical(libbfm):
    ps = small_batch(6, seed=3)
    B = BA.Batch(libbfm, ps)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8))
        x1 = np.concatenate(B.solutions())
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8))
        x2 = np.concatenate(B.solutions())
    finally:
        B.close()
    assert np.array_equal(x1, x2)


def test_step_graph_matches_separate_calls(libbfm):
    """bfm_gpu_problem_step_parts (assembly + batched solve captured as one
    graph) gives the solutions of the separate assemble + solve calls, bit for
    bit, on every replay, and captures again when an input changes."""
    ps = small_batch(8, seed=5)
    B = BA.Batch(libbfm, ps)
    try:
        o = bfm_gb300.default_opts(rtol=1e-8, autotune=0)
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
