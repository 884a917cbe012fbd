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


def coarse_grid(n: int, w: float, h: float, per_cell: int = 1000):
    """Cell counts (gx, gy) of the coarse grid for n nodes in a w x h box
    (bfm_gb300/csrc/fem_gpu.cu, coarse_grid): about one cell per `per_cell`
    nodes, at most 1024 (gy rounded, then capped so gx gy stays within the
    target), as square as the box allows, and fewer while the band
    factorisation's cost 1.5 cells bw^2 (bw = 3 (shorter side + 1) + 2, the
    half-bandwidth of A_c for cells numbered along the shorter side first)
    exceeds 8e6 or bw exceeds 101."""
    target = min(max(n // per_cell, 1), 1024)
    while True:
        gx = gy = 1
        if w > 0 and h > 0:
            gx = min(max(int(np.floor(np.sqrt(target * w / h) + 0.5)), 1), target)
            gy = max(min(int(np.floor(target / gx + 0.5)), target // gx), 1)
        elif w > 0:
            gx = target
        elif h > 0:
            gy = target
        bw = 3 * (min(gx, gy) + 1) + 2
        if (bw <= 101 and 1.5 * gx * gy * bw * bw <= 8e6) or target == 1:
            return gx, gy
        target = target * 9 // 10


def cell_grid(coords: np.ndarray):
    """The aggregation of the two-level preconditioner (bfm_gb300/csrc/
    fem_gpu.cu, build_aggregates): the coarse_grid cells over the bounding box.
    Returns (cell of each node, gx, gy, x0, y0, cw, ch); cells are numbered
    cx + gx cy here (the GPU numbers them along the shorter side first, which
    only reorders the coarse DOFs)."""
    n = len(coords)
    x0, y0 = coords.min(0)
    x1, y1 = coords.max(0)
    w, h = x1 - x0, y1 - y0
    gx, gy = coarse_grid(n, w, h)
    cw = w * (1 + 1e-12) / gx if w > 0 else 1.0
    ch = h * (1 + 1e-12) / gy if h > 0 else 1.0
    cx = np.clip(((coords[:, 0] - x0) / cw).astype(np.int64), 0, gx - 1)
    cy = np.clip(((coords[:, 1] - y0) / ch).astype(np.int64), 0, gy - 1)
    return cx + gx * cy, gx, gy, x0, y0, cw, ch


class TwoLevel:
    """z = M_SSOR^-1 r + P A_c^-1 P^T r (additive), P the rigid-body modes of
    each cell -- per node [[1, 0, -dy], [0, 1, dx]] with (dx, dy) its offset
    from the cell centre over H = max(cell width, height), rounded to FP32 as
    the GPU stores them, rows of constrained DOFs zero -- and A_c = P^T A P on
    the coarse DOFs that A sees (the others dropped, as the GPU's pivot test
    does).  A and coords in the caller's order; `free` per DOF."""

    def __init__(self, A: sp.spmatrix, coords: np.ndarray, free: np.ndarray, ssor: BlockSSOR):
        A = sp.csr_matrix(A)
        n = len(coords)
        cell, gx, gy, x0, y0, cw, ch = cell_grid(coords)
        H = max(cw, ch)
        xc = x0 + (cell % gx + 0.5) * cw
        yc = y0 + (cell // gx + 0.5) * ch
        dx = ((coords[:, 0] - xc) / H).astype(np.float32).astype(np.float64)
        dy = ((coords[:, 1] - yc) / H).astype(np.float32).astype(np.float64)
        f0, f1 = free[0::2].astype(float), free[1::2].astype(float)
        nc = 3 * gx * gy
        rows = np.concatenate([2 * np.arange(n), 2 * np.arange(n), 2 * np.arange(n) + 1, 2 * np.arange(n) + 1])
        cols = np.concatenate([3 * cell, 3 * cell + 2, 3 * cell + 1, 3 * cell + 2])
        vals = np.concatenate([f0, -dy * f0, f1, dx * f1])
        P = sp.csr_matrix((vals, (rows, cols)), shape=(2 * n, nc))
        Ac = (P.T @ A @ P).toarray()
        Ac = 0.5 * (Ac + Ac.T)
        keep = np.diag(Ac) > 0
        self.P = P[:, keep].tocsr()
        self.Ainv = np.linalg.inv(Ac[np.ix_(keep, keep)])
        self.ssor = ssor
        self.n_cells = gx * gy

    def apply(self, r: np.ndarray) -> np.ndarray:
        return self.ssor.apply(r) + self.P @ (self.Ainv @ (self.P.T @ r))


def free_dofs(A: sp.spmatrix) -> np.ndarray:
    """DOFs whose row is not an eliminated Dirichlet row (a lone 1 on the
    diagonal).  Explicitly stored zeros do not count: the oracle's assembly
    keeps the structural pattern, zeros of eliminated rows included."""
    A = sp.csr_matrix(A, copy=True)
    A.eliminate_zeros()
    nnz = np.diff(A.indptr)
    return ~((nnz == 1) & (A.diagonal() == 1.0))


# ---------------------------------------------------------------- batched two-level block Jacobi

def part_grid(n: int, w: float, h: float, per_cell: int = 48, max_cells: int = 64):
    """Cell counts (gx, gy) of one part's coarse grid in the batched solver's
    two-level block Jacobi (bfm_gb300/csrc/batch.cu, part_grid): about one
    cell per `per_cell` nodes, at most `max_cells`, as square as the part's
    bounding box allows (gy rounded, then capped so gx gy stays within the
    target)."""
    target = min(max(n // per_cell, 1), max_cells)
    gx = gy = 1
    if w > 0 and h > 0:
        gx = min(max(int(np.floor(np.sqrt(target * w / h) + 0.5)), 1), target)
        gy = max(min(int(np.floor(target / gx + 0.5)), target // gx), 1)
    elif w > 0:
        gx = target
    elif h > 0:
        gy = target
    return gx, gy


class BlockJacobi:
    """z = D^-1 r, D the nodes' 2x2 diagonal blocks of A (scalar CSR)."""

    def __init__(self, A: sp.spmatrix):
        A = sp.csr_matrix(A)
        n = A.shape[0] // 2
        D = np.zeros((n, 2, 2))
        idx = np.arange(n)
        for a in range(2):
            for b in range(2):
                D[:, a, b] = np.asarray(A[2 * idx + a, 2 * idx + b]).ravel()
        self.Dinv = np.linalg.inv(D)

    def apply(self, r: np.ndarray) -> np.ndarray:
        return np.einsum("nij,nj->ni", self.Dinv, r.reshape(-1, 2)).ravel()


class TwoLevelJacobi:
    """One part of the batched solver's two-level block Jacobi: z = D^-1 r +
    P A_c^-1 P^T r, with the part_grid cells over the part's bounding box, P
    per node [[f0, 0, -f0 dy], [0, f1, f1 dx]] ((dx, dy) the offset from the
    cell's centre over H = max(cell width, height), rounded to FP32 as the GPU
    stores it; f = 0 on an eliminated DOF) and A_c = P^T A P on the coarse DOFs
    A sees (the GPU drops a coarse DOF whose pivot in the Cholesky of the
    diagonally scaled A_c falls below 1e-5; here the ones with a zero
    diagonal).  A and coords of the part alone; `free` per DOF."""

    def __init__(self, A: sp.spmatrix, coords: np.ndarray, free: np.ndarray, per_cell: int = 48, max_cells: int = 64):
        A = sp.csr_matrix(A)
        n = len(coords)
        x0, y0 = coords.min(0)
        w, h = coords.max(0) - coords.min(0)
        gx, gy = part_grid(n, w, h, per_cell, max_cells)
        cw = w * (1 + 1e-12) / gx if w > 0 else 1.0
        ch = h * (1 + 1e-12) / gy if h > 0 else 1.0
        H = max(cw, ch)
        cx = np.clip(((coords[:, 0] - x0) / cw).astype(np.int64), 0, gx - 1)
        cy = np.clip(((coords[:, 1] - y0) / ch).astype(np.int64), 0, gy - 1)
        cell = cx + gx * cy
        dx = ((coords[:, 0] - (x0 + (cx + 0.5) * cw)) / H).astype(np.float32).astype(np.float64)
        dy = ((coords[:, 1] - (y0 + (cy + 0.5) * ch)) / H).astype(np.float32).astype(np.float64)
        f0, f1 = free[0::2].astype(float), free[1::2].astype(float)
        idx = np.arange(n)
        rows = np.concatenate([2 * idx, 2 * idx, 2 * idx + 1, 2 * idx + 1])
        cols = np.concatenate([3 * cell, 3 * cell + 2, 3 * cell + 1, 3 * cell + 2])
        vals = np.concatenate([f0, -dy * f0, f1, dx * f1])
        P = sp.csr_matrix((vals, (rows, cols)), shape=(2 * n, 3 * gx * gy))
        Ac = (P.T @ A @ P).toarray()
        Ac = 0.5 * (Ac + Ac.T)
        keep = np.diag(Ac) > 0
        self.P = P[:, keep].tocsr()
        self.Ainv = np.linalg.inv(Ac[np.ix_(keep, keep)])
        self.smoother = BlockJacobi(A)
        self.n_cells = gx * gy

    def apply(self, r: np.ndarray) -> np.ndarray:
        return self.smoother.apply(r) + self.P @ (self.Ainv @ (self.P.T @ r))
