"""Axisymmetric element on the GPU (reference libbfm/src/system.c:229-356,
539-622): with the reference's own formulas (BFM_GPU_AXISYM_REFERENCE=1) K is
bit-identical to the reference's and b agrees to 1e-14; by default (the
plane-strain constant, the radius on every stiffness term, consistent edge
loads) K is bit-identical to the oracle's and the CG solve agrees with the
oracle's direct solve, in every precision."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api
from common import AXI_CASES, dense_K, load, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def fp64_opts(libbfm):
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-12)))
    yield
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


def corrected(name):
    p, d = load(name)
    p.stress = 2
    return p, d


@pytest.mark.parametrize("name", AXI_CASES)
def test_reference_formulas_bit_exact(libbfm, name, monkeypatch):
    monkeypatch.setenv("BFM_GPU_AXISYM_REFERENCE", "1")
    p, d = load(name)
    assert p.stress == 3
    h = api.SimHandle.from_problem(libbfm, p)
    K, b, perm = h.system(renumber=True)
    assert np.array_equal(K, dense_K(d, p.n_dof))
    assert rel(b, d["b"]) < 1e-14
    assert np.array_equal(perm, d["perm"])


@pytest.mark.parametrize("name", AXI_CASES)
def test_corrected_formulas_match_oracle(libbfm, name, monkeypatch):
    monkeypatch.delenv("BFM_GPU_AXISYM_REFERENCE", raising=False)
    p, _ = corrected(name)
    h = api.SimHandle.from_problem(libbfm, p)
    K, b, _ = h.system()
    Ko, bo = O.assemble_dense(p)
    assert np.array_equal(K, Ko)
    assert rel(b, bo) < 1e-14
    assert h.run() == 0, h.error()
    x, _, _ = O.solve_direct(p)
    assert rel(h.effects(), x) < 1e-10


@pytest.mark.parametrize("precision,tol", [(bfm_gb300.FP64_DF, 1e-9), (bfm_gb300.MIXED_EXACT, 1e-6),
                                           (bfm_gb300.MIXED, 1e-6)])
def test_corrected_formulas_other_precisions(libbfm, precision, tol, monkeypatch):
    monkeypatch.delenv("BFM_GPU_AXISYM_REFERENCE", raising=False)
    p, _ = corrected("axi_p1_12x8")
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-10, precision=precision)))
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0, h.error()
    x, _, _ = O.solve_direct(p)
    assert rel(h.effects(), x) < tol


def test_formulation_code_is_checked(libbfm):
    P = C.c_void_p()
    assert libbfm.bfm_gpu_problem_create(C.byref(P), 3, 3, 1, 0, 0, None) == 0
    try:
        assert libbfm.bfm_gpu_problem_set_material(P, 1.0, 0.3, 1.0, 4, None, None, 0) == -1
        assert "formulation" in bfm_gb300.last_error()
        assert libbfm.bfm_gpu_problem_set_material(P, 1.0, 0.3, 1.0, 2, None, None, 0) == 0
    finally:
        libbfm.bfm_gpu_problem_destroy(P)
