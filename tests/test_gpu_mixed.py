"""Mixed precision: FP32 matrix and Krylov vectors, FP64 inner products,
FP64 solution and FP64 residual replacement.  Checked against the FP64
direct oracle; the error bound each mode must meet is written here."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api, meshgen as M
from common import load, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run(lib, p, precision, rtol=1e-8, precond=0):
    lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=rtol, precision=precision, precond=precond)))
    try:
        h = api.SimHandle.from_problem(lib, p)
        rc = h.run()
        s = bfm_gb300.bfm_gpu_stats_t()
        lib.bfm_gpu_last_stats(C.byref(s))
        return rc, h, s
    finally:
        lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


@pytest.fixture(scope="module")
def perforated():
    p = M.cfg_perforated(nx=256, ny=64, n_holes=25, seed=3)
    x, _, _ = O.solve_direct(p)
    return p, x


def test_mixed_exact_reaches_fp64_accuracy(libbfm, perforated):
    p, x = perforated
    rc, h, s = run(libbfm, p, bfm_gb300.MIXED_EXACT, rtol=1e-8)
    assert rc == 0, h.error()
    assert s.rel_residual <= 1e-8          # FP64 true residual of the FP64 system
    assert s.replacements >= 1
    assert rel(h.effects(), x) <= 1e-6     # displacement error vs the FP64 oracle


def test_mixed_fp32_integration_error_is_bounded(libbfm, perforated):
    p, x = perforated
    rc, h, s = run(libbfm, p, bfm_gb300.MIXED, rtol=1e-8)
    assert rc == 0, h.error()
    assert s.rel_residual <= 1e-8          # of the FP32-integrated system (its own operator)
    assert rel(h.effects(), x) <= 1e-4     # FP32 element integration: error of the discrete operator


@pytest.mark.parametrize("name", ["p1_64x16", "q1_24x8_jitter", "gear12"])
def test_mixed_exact_vs_reference_fixtures(libbfm, name):
    p, d = load(name)
    rc, h, s = run(libbfm, p, bfm_gb300.MIXED_EXACT, rtol=1e-10)
    assert rc == 0, h.error()
    assert rel(h.effects(), d["effects"]) <= 1e-8


def test_block_jacobi_fp64(libbfm):
    p, d = load("gear12")
    rc, h, s = run(libbfm, p, bfm_gb300.FP64, rtol=1e-12, precond=bfm_gb300.PC_BLOCK_JACOBI)
    assert rc == 0, h.error()
    assert rel(h.effects(), d["effects"]) <= 1e-10
