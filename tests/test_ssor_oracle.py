"""The float64 restatement of the multicolour block SSOR preconditioner
(oracle/ssor_ref.py) on its own: the colouring check, M^-1 against the
explicit M = (D + L) D^-1 (D + U), and PCG iterations against Jacobi's."""
import numpy as np
import scipy.sparse as sp

from bfm_gb300 import meshgen as M
from oracle import oracle as O, ssor_ref as S


def greedy_order(G):
    n = G.shape[0]
    col = -np.ones(n, int)
    for v in range(n):
        used = set(col[G.indices[G.indptr[v]:G.indptr[v + 1]]])
        c = 0
        while c in used:
            c += 1
        col[v] = c
    perm = np.argsort(col, kind="stable")
    off = np.concatenate([[0], np.cumsum(np.bincount(col))])
    return perm, off


def test_restatement():
    p = M.cfg_perforated(nx=48, ny=12, n_holes=20, seed=3)
    K, b = O.assemble_csr(p)
    K = sp.csr_matrix(K)
    G = S.node_graph(K, p.n_nodes)
    perm, off = greedy_order(G)
    assert S.is_colouring(G, perm, off)
    assert not S.is_colouring(G, perm, np.array([0, p.n_nodes]))
    pc = S.BlockSSOR(K, perm, off)
    # explicit M in the working order
    dperm = np.stack([2 * perm, 2 * perm + 1], 1).ravel()
    A = K[dperm][:, dperm].toarray()
    n = p.n_nodes
    blk = np.kron(np.eye(n), np.ones((2, 2))) > 0
    D = np.where(blk, A, 0.0)
    Lm = np.where(~blk, np.tril(A), 0.0)
    Um = np.where(~blk, np.triu(A), 0.0)
    Mw = (D + Lm) @ np.linalg.inv(D) @ (D + Um)
    r = np.random.default_rng(0).normal(size=2 * n)
    z = pc.apply(r)
    np.testing.assert_allclose(Mw @ z[dperm], r[dperm], rtol=1e-9, atol=1e-9 * np.abs(r).max())
    _, it_ssor = S.pcg(K, b, pc.apply)
    d = K.diagonal()
    _, it_jac = S.pcg(K, b, lambda v: v / d)
    assert it_ssor < 0.5 * it_jac


def test_coarse_grid_rule():
    """The cell grid the GPU builds (fem_gpu.cu coarse_grid), restated: about
    one cell per 1,000 nodes as square as the box allows, at most 1,024 cells,
    fewer while the band factorisation's cost 1.5 cells bw^2 passes 8e6 (bw =
    3 (shorter side + 1) + 2 <= 101)."""
    assert S.coarse_grid(2049 * 513, 4.0, 1.0) == (64, 16)          # the 2.1M-DOF plate: 1,024 cells
    assert S.coarse_grid(2049 * 513, 4.0, 1.0, per_cell=1250) == (58, 14)
    assert S.coarse_grid(257 * 65, 4.0, 1.0) == (8, 2)
    assert S.coarse_grid(500, 4.0, 1.0) == (1, 1)                   # fewer nodes than one cell
    assert S.coarse_grid(10 ** 6, 0.0, 1.0) == (1, 1000)            # a line of nodes
    # w/h = 2.16: 47 x 22 (1,034) after rounding both counts; capped to 47 x 21
    assert S.coarse_grid(1024 * 1000, 2.16, 1.0) == (47, 21)
    for n, w in ((1024 * 1000, 2.16), (1024 * 1000, 3.3), (700 * 1000, 1.7), (900 * 1000, 5.5)):
        gx, gy = S.coarse_grid(n, w, 1.0)
        assert gx * gy <= min(n // 1000, 1024)
    gx, gy = S.coarse_grid(10 ** 6, 1.0, 1.0)                       # square box: the cost cap binds
    bw = 3 * (min(gx, gy) + 1) + 2
    assert gx * gy < 1000 and 1.5 * gx * gy * bw * bw <= 8e6 and bw <= 101


def test_two_level_restatement():
    """The additive two-level preconditioner (rigid-body modes of a cell grid)
    on a 256x64 plate: 8 x 2 cells, and well under half of SSOR's iterations."""
    p = M.cfg_perforated(nx=256, ny=64, n_holes=200, seed=3)
    K, b = O.assemble_csr(p)
    K = sp.csr_matrix(K)
    perm, off = greedy_order(S.node_graph(K, p.n_nodes))
    ssor = S.BlockSSOR(K, perm, off)
    tl = S.TwoLevel(K, p.coords, S.free_dofs(K), ssor)
    assert tl.n_cells == 16
    # symmetric positive definite preconditioner: z.r > 0 and M^-1 symmetric on random vectors
    rng = np.random.default_rng(1)
    u, v = rng.normal(size=2 * p.n_nodes), rng.normal(size=2 * p.n_nodes)
    assert abs(u @ tl.apply(v) - v @ tl.apply(u)) <= 1e-8 * abs(u @ tl.apply(v))
    assert u @ tl.apply(u) > 0
    _, it1 = S.pcg(K, b, ssor.apply)
    _, it2 = S.pcg(K, b, tl.apply)
    assert it2 < 0.5 * it1, (it2, it1)
