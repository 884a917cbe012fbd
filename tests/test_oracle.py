"""The oracle (CPU restatement) against the reference's golden outputs."""
import numpy as np
import pytest

from common import AXI_CASES, CASES, dense_K, load, rel
from oracle import oracle as O


def test_lepl8_matches_shipped_golden_files():
    # data/U.txt and data/V.txt are printed with %14.7e: 8 significant digits
    p, d = load("lepl8")
    eff, _, _ = O.solve_reference(p)
    u, v = eff[0::2], eff[1::2]
    tol = 5e-8 * np.abs(d["U_txt"]).max()
    assert np.abs(u - d["U_txt"]).max() <= tol
    assert np.abs(v - d["V_txt"]).max() <= 5e-8 * np.abs(d["V_txt"]).max()


@pytest.mark.parametrize("name", CASES + AXI_CASES)
def test_restatement_is_bit_exact(name):
    p, d = load(name)
    eff, perm, _ = O.solve_reference(p)
    assert np.array_equal(perm, d["perm"]), "RCM permutation differs"
    assert np.array_equal(eff, d["effects"]), f"effects differ, rel {rel(eff, d['effects']):.3e}"


@pytest.mark.parametrize("name", CASES + AXI_CASES)
def test_dense_assembly_bit_exact(name):
    p, d = load(name)
    K, b = O.assemble_dense(p)
    assert np.array_equal(K, dense_K(d, p.n_dof))
    assert np.array_equal(b, d["b"])


@pytest.mark.parametrize("name", CASES + AXI_CASES)
def test_csr_restatement_matches_dense(name):
    p, d = load(name)
    Kc, bc = O.assemble_csr(p)
    Kd = dense_K(d, p.n_dof)
    assert np.array_equal(Kc.toarray(), Kd)
    assert rel(bc, d["b"]) < 1e-14
    perm, _ = O.rcm_csr(Kc)
    assert np.array_equal(perm, d["perm"])


@pytest.mark.parametrize("name", ["p1_64x16", "q1_24x8_jitter", "p1_20x10_shuffled", "gear12"])
def test_direct_oracle_agrees_with_reference(name):
    p, d = load(name)
    x, _, _ = O.solve_direct(p)
    # band LU without pivoting vs SuperLU on a system with cond ~1e12
    assert rel(x, d["effects"]) < 1e-9


def test_empty_problem():
    from bfm_gb300 import meshgen as M
    p = M.Problem("empty", 3, np.zeros((0, 2)), np.zeros((0, 3), np.int64))
    eff, perm, _ = O.solve_reference(p)
    assert eff.size == 0 and perm.size == 0


def axi_problem(name, stress):
    p, _ = load(name)
    p.stress = stress
    return p


@pytest.mark.parametrize("name", AXI_CASES)
def test_axisymmetric_modes(name):
    """The reference's axisymmetric formulas give an indefinite K; mode 2 (the
    plane-strain constant, the radius on every term, consistent edge loads)
    gives an SPD one whose loads sum to the exact edge integrals."""
    K3, _ = O.assemble_dense(axi_problem(name, 3))
    K2, b2 = O.assemble_dense(axi_problem(name, 2))
    assert np.linalg.eigvalsh(0.5 * (K3 + K3.T)).min() < 0
    assert np.linalg.eigvalsh(0.5 * (K2 + K2.T)).min() > 0
    # total Neumann X load with no body force and no constraints: value x
    # integral of r dz over the left edge (r = 1) and the right edge (r = 4)
    p = axi_problem(name, 2)
    p.forces = []
    p.conds = [c for c in p.conds if c[0] == 2]
    _, b = O.assemble_dense(p)
    assert b[0::2].sum() == pytest.approx(2e5 * 1.0 * 2.0 - 5e4 * 4.0 * 2.0, rel=1e-13)
