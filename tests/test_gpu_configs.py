"""The benchmark configurations at their stated sizes, against the FP64
direct oracle (the C restatement of the reference assembly, system.c:109-227
with the rules of rule.c:90-111, solved by SuperLU).

- 1024x256 Q1 plate, interior nodes jittered by +-0.2h (seed 2), 526,850 DOF:
  K bit-identical to the oracle's, b to 1e-14; FP64 Jacobi-PCG to relative
  residual 1e-10 (or the FP64 floor just above it: the exact solution rounded
  to FP64 has a relative residual of about 1.4e-10) agrees with the direct
  solve to DIRECT_Q1.
- 2048x512 P1 perforated plate (200 soft inclusions, seed 3), 2,102,274 DOF:
  K bit-identical, b to 1e-14; every fast method reaches relative residual 1e-8 and
  a displacement error at most 1e-6 against the direct solve.
- 256 uneven P1 plates (seed 4) in one batched solve: every mesh within 1e-6
  of its own direct solve.

The direct solves take about a minute and 10 GB of host memory at the
largest size (SuperLU with a minimum-degree order on A + A^T)."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api, batch as BA, meshgen as M
from bfm_gb300.methods import METHODS as MT
from oracle import oracle as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

DIRECT_Q1 = 1e-10  # FP64 Jacobi-PCG at rtol 1e-10 vs the direct solve, 526,850 DOF (measured 1.3e-13)
DIRECT_MIXED = 1e-6  # the displacement bound of the fast methods at rtol 1e-8


def direct(K, b):
    """The FP64 direct solve, refined once with a residual in extended
    precision (numpy's long double), and the relative residual of that
    solution rounded to FP64: the floor no FP64 solution can go much below
    (on the Q1 plate it is above 1e-10)."""
    import scipy.sparse.linalg as spla
    lu = spla.splu(K.tocsc(), permc_spec="MMD_AT_PLUS_A", options=dict(SymmetricMode=True))
    x = lu.solve(b)
    KL, bL = K.astype(np.longdouble), b.astype(np.longdouble)
    r = bL - KL @ x.astype(np.longdouble)
    x = (x.astype(np.longdouble) + lu.solve(r.astype(np.float64))).astype(np.float64)
    floor = float(np.linalg.norm((bL - KL @ x.astype(np.longdouble)).astype(np.float64)) / np.linalg.norm(b))
    return x, floor


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check_system(D, Ko, bo):
    """The GPU's FP64 K and b (caller order) against the oracle's, bit for bit."""
    rp, cols, vals, b, perm = D.system()
    Kg = api.scalar_csr(rp, cols, vals, D.p.n_nodes, perm)
    bg = np.empty_like(b)
    bg[np.stack([2 * perm, 2 * perm + 1], 1).ravel()] = b
    assert Kg.shape == Ko.shape
    assert (Kg - Ko).count_nonzero() == 0
    assert rel(bg, bo) <= 1e-14


@pytest.fixture(scope="module")
def q1_large():
    p = M.cfg_q1_large()
    Ko, bo = O.assemble_csr(p)
    return (p, Ko, bo) + direct(Ko, bo)


@pytest.fixture(scope="module")
def perforated():
    p = M.cfg_perforated()
    Ko, bo = O.assemble_csr(p)
    return (p, Ko, bo) + direct(Ko, bo)


def test_q1_large_fp64_jacobi_vs_direct(libbfm, q1_large):
    p, Ko, bo, x, floor = q1_large
    assert p.n_dof == 526_850
    D = api.DeviceProblem(libbfm, p)
    try:
        D.assemble(bfm_gb300.FP64)
        check_system(D, Ko, bo)
        D.solve(bfm_gb300.default_opts(rtol=1e-10))
        s = D.stats()
        # 1e-10 or, where the FP64-rounded exact solution itself sits above it,
        # that floor: the solver then stops with BFM_GPU_STAGNATED (5)
        assert s.status in (0, 5) and s.rel_residual <= max(1e-10, 1.05 * floor), (s.status, s.rel_residual, floor)
        err = rel(D.solution(), x)
        print(f"q1 1024x256: {s.iterations} iterations, relative residual {s.rel_residual:.3e} "
              f"(FP64 floor {floor:.3e}), error vs direct {err:.3e}")
        assert err <= DIRECT_Q1
    finally:
        D.close()


METHODS = ["ssor2_df", "ssor2_fp64", "ssor2_mixed", "ssor2_mixed_exact", "mixed_exact"]


def test_perforated_system_is_the_oracles(libbfm, perforated):
    p, Ko, bo, _, _ = perforated
    assert p.n_dof == 2_102_274
    D = api.DeviceProblem(libbfm, p)
    try:
        D.assemble(bfm_gb300.FP64)
        check_system(D, Ko, bo)
    finally:
        D.close()


@pytest.mark.parametrize("name", METHODS)
def test_perforated_methods_vs_direct(libbfm, perforated, name):
    """Every method to relative residual 1e-8 of its own operator, within 1e-6
    of the direct solve.  The MIXED precision integrates in FP32, so its
    operator differs from the FP64 one at the 1e-7 level and so does its
    solution (measured 8e-8 on this plate)."""
    p, _, _, x, floor = perforated
    precision, precond, drop = MT[name]
    D = api.DeviceProblem(libbfm, p)
    try:
        o = bfm_gb300.default_opts(rtol=1e-8, precision=precision, precond=precond, replace_drop=drop)
        D.assemble(precision)
        D.solve(o)
        s = D.stats()
        assert s.status == 0 and s.rel_residual <= 1e-8, (s.status, s.rel_residual)
        err = rel(D.solution(), x)
        print(f"{name}: {s.iterations} iterations, relative residual {s.rel_residual:.3e} "
              f"(FP64 floor {floor:.3e}), error vs direct {err:.3e}")
        assert err <= DIRECT_MIXED
    finally:
        D.close()


@pytest.mark.parametrize("pc", [bfm_gb300.PC_JACOBI, bfm_gb300.PC_TWO_LEVEL_JACOBI])
def test_batch_256_uneven_vs_direct(libbfm, pc):
    ps = M.batch_uneven(256, seed=4)
    B = BA.Batch(libbfm, ps)
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        B.solve(bfm_gb300.default_opts(rtol=1e-8, precond=pc))
        st = B.stats()
        xs = B.solutions()
    finally:
        B.close()
    assert np.all(st["status"] == 0) and np.all(st["rel_residual"] <= 1e-8)
    worst = 0.0
    for p, xg in zip(ps, xs):
        ref, _, _ = O.solve_direct(p)
        worst = max(worst, rel(xg, ref))
    print(f"batch of 256: worst error vs direct {worst:.3e}, iterations {int(st['iterations'].min())}.."
          f"{int(st['iterations'].max())}")
    assert worst <= DIRECT_MIXED
