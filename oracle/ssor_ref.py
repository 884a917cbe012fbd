"""Test infrastructure: a float64 restatement of the multicolour block SSOR
preconditioner of the GPU path (bfm_gb300/csrc/cg_kernels.cuh, k_ssor_fwd /
k_ssor_bwd), and the PCG that uses it.

The preconditioner has no counterpart in the reference (libbfm solves with a
band LU, libbfm/src/matrix.c:253-404); this file restates the method from its
definition so the GPU sweeps can be checked against it:

    M = (D~ + L) D~^-1 (D~ + U),   A = L + D + U

in a colour-major node order (L: the 2x2 blocks of lower-colour neighbours,
U: higher-colour ones; a coupling inside a colour range, which a valid
colouring does not have, would belong to neither), D~ the relaxation blocks.
Only tests import it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def node_graph(K: sp.spmatrix, n_nodes: int) -> sp.csr_matrix:
    """The node adjacency (with self loops) of a 2-DOF-per-node matrix."""
    Kc = sp.coo_matrix(K)
    G = sp.csr_matrix((np.ones(Kc.nnz), (Kc.row // 2, Kc.col // 2)), shape=(n_nodes, n_nodes))
    G.sum_duplicates()
    return G


def conflicts(G: sp.csr_matrix, perm: np.ndarray, offsets: np.ndarray) -> int:
    """Number of nodes with a neighbour in their own colour range, G the
    caller's graph and perm the working order (perm[w] = caller node)."""
    n = G.shape[0]
    colour = np.empty(n, np.int64)
    for c in range(len(offsets) - 1):
        colour[perm[offsets[c]:offsets[c + 1]]] = c
    Gc = sp.coo_matrix(G)
    bad = (Gc.row != Gc.col) & (colour[Gc.row] == colour[Gc.col])
    return int(np.unique(Gc.row[bad]).size)


def is_colouring(G: sp.csr_matrix, perm: np.ndarray, offsets: np.ndarray) -> bool:
    """True when no two nodes of one colour range are adjacent in G."""
    return conflicts(G, perm, offsets) == 0


class BlockSSOR:
    """z = M^-1 r for A (scalar CSR, caller order) with the working order
    perm and colour offsets, relaxation block inverses Dinv (n_nodes, 2, 2,
    caller order; default: inverses of A's diagonal blocks)."""

    def __init__(self, A: sp.spmatrix, perm: np.ndarray, offsets: np.ndarray, Dinv: np.ndarray | None = None):
        A = sp.csr_matrix(A)
        n = A.shape[0] // 2
        self.n, self.offsets = n, np.asarray(offsets)
        self.dperm = np.stack([2 * perm, 2 * perm + 1], 1).ravel()
        Ap = sp.coo_matrix(A[self.dperm][:, self.dperm])
        rn, cn = Ap.row // 2, Ap.col // 2
        cls = np.searchsorted(self.offsets, np.arange(n), side="right") - 1

        def part(mask):
            return sp.csr_matrix((Ap.data[mask], (Ap.row[mask], Ap.col[mask])), shape=Ap.shape)
        other = cls[rn] != cls[cn]
        self.L, self.U = part((cn < rn) & other), part((cn > rn) & other)
        if Dinv is None:
            D = np.zeros((n, 2, 2))
            d = rn == cn
            np.add.at(D, (rn[d], Ap.row[d] % 2, Ap.col[d] % 2), Ap.data[d])
            self.Dinv = np.linalg.inv(D)
        else:
            self.Dinv = np.asarray(Dinv)[perm]

    def _blk(self, s, e, v):
        return np.einsum("nij,nj->ni", self.Dinv[s:e], v.reshape(-1, 2)).ravel()

    def apply(self, r: np.ndarray) -> np.ndarray:
        o = self.offsets
        nc = len(o) - 1
        rp = r[self.dperm]
        y = np.zeros_like(rp)
        for c in range(nc):                      # (D~ + L) y = r
            s, e = 2 * o[c], 2 * o[c + 1]
            y[s:e] = self._blk(o[c], o[c + 1], rp[s:e] - self.L[s:e] @ y)
        z = y.copy()
        for c in range(nc - 2, -1, -1):          # (D~ + U) z = D~ y
            s, e = 2 * o[c], 2 * o[c + 1]
            z[s:e] = y[s:e] - self._blk(o[c], o[c + 1], self.U[s:e] @ z)
        out = np.empty_like(z)
        out[self.dperm] = z
        return out


def pcg(A: sp.spmatrix, b: np.ndarray, apply, rtol: float = 1e-8, max_iters: int = 100000):
    """PCG (Fletcher-Reeves beta) to ||r|| <= rtol ||b||; returns (x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply(r)
    p = z.copy()
    g = r @ z
    nb = np.linalg.norm(b)
    for it in range(1, max_iters + 1):
        q = A @ p
        a = g / (p @ q)
        x += a * p
        r -= a * q
        if np.linalg.norm(r) <= rtol * nb:
            return x, it
        z = apply(r)
        g2 = r @ z
        p = z + (g2 / g) * p
        g = g2
    return x, max_iters
