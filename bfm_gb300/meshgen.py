"""Synthetic plane-elasticity problems on a rectangular plate.

The workloads are the plate problems of the benchmark definitions: a 4 m x
1 m plate meshed by an nx x ny grid (P1: each cell split into two triangles,
Q1: quads with the reference's local node order (+,+), (-,+), (-,-), (+,-)),
left edge clamped, gravity, optionally a downward traction on the right
edge, jittered interior nodes, circular soft inclusions, per-element
materials.  Every random choice comes from numpy.random.default_rng(seed).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

DIRICHLET_X, DIRICHLET_Y, NEUMANN_X, NEUMANN_Y = 0, 1, 2, 3

STEEL = dict(E=211e9, nu=0.3, rho=7850.0)
GRAVITY = 9.81


@dataclass
class Problem:
    name: str
    kind: int                      # 3 (P1) or 4 (Q1)
    coords: np.ndarray             # (N, 2) float64
    elems: np.ndarray              # (E, kind) int64
    E: float = STEEL["E"]
    nu: float = STEEL["nu"]
    rho: float = STEEL["rho"]
    stress: int = 1  # 0 plane strain, 1 plane stress, 2 axisymmetric (x = radius), 3 axisymmetric with the reference's formulas
    elem_E: np.ndarray | None = None
    elem_nu: np.ndarray | None = None
    forces: list = field(default_factory=list)      # [(fx, fy)] body accelerations
    conds: list = field(default_factory=list)       # [(kind, value, mask[N] bool)]
    edges: np.ndarray | None = None                 # (M, 2) int64 edges (boundary edges unless edge_boundary says)
    edge_boundary: np.ndarray | None = None         # (M,) bool: the edge has one adjacent element (None: all)
    edge_loads: tuple | None = None                 # (edges (M, 2), tractions (M, 2)): per-edge Neumann loads

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.elems.shape[0])

    @property
    def n_dof(self) -> int:
        return 2 * self.n_nodes


def grid(nx: int, ny: int, kind: int, lx: float = 4.0, ly: float = 1.0):
    """Nodes (i, j) -> j*(nx+1)+i; returns coords (N,2), elems (E,kind)."""
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys)
    coords = np.stack([X.ravel(), Y.ravel()], axis=1)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny))
    i, j = i.ravel(), j.ravel()
    n00 = j * (nx + 1) + i
    n10 = n00 + 1
    n01 = n00 + (nx + 1)
    n11 = n01 + 1
    if kind == 4:
        elems = np.stack([n11, n01, n00, n10], axis=1)
    elif kind == 3:
        t1 = np.stack([n00, n10, n11], axis=1)
        t2 = np.stack([n00, n11, n01], axis=1)
        elems = np.stack([t1, t2], axis=1).reshape(-1, 3)
    else:
        raise ValueError("kind must be 3 or 4")
    return coords, elems.astype(np.int64)


def boundary_edges(nx: int, ny: int) -> np.ndarray:
    """All border edges of the grid as node pairs (counter-clockwise)."""
    w = nx + 1
    bottom = [(i, i + 1) for i in range(nx)]
    right = [(j * w + nx, (j + 1) * w + nx) for j in range(ny)]
    top = [(ny * w + i + 1, ny * w + i) for i in range(nx)]
    left = [((j + 1) * w, j * w) for j in range(ny)]
    return np.array(bottom + right + top + left, dtype=np.int64)


def side_mask(coords: np.ndarray, side: str, lx: float = 4.0, ly: float = 1.0) -> np.ndarray:
    x, y = coords[:, 0], coords[:, 1]
    tol = 1e-9
    return {"left": x < tol, "right": x > lx - tol, "bottom": y < tol, "top": y > ly - tol}[side]


def jitter(coords: np.ndarray, nx: int, ny: int, frac: float, rng, lx=4.0, ly=1.0) -> np.ndarray:
    """Move interior nodes by U(-frac h, frac h) per component."""
    hx, hy = lx / nx, ly / ny
    c = coords.copy()
    x, y = c[:, 0], c[:, 1]
    interior = (x > 1e-9) & (x < lx - 1e-9) & (y > 1e-9) & (y < ly - 1e-9)
    k = int(interior.sum())
    c[interior, 0] += rng.uniform(-frac * hx, frac * hx, k)
    c[interior, 1] += rng.uniform(-frac * hy, frac * hy, k)
    return c


def plate(nx: int, ny: int, kind: int, *, name: str = "plate", stress: bool = True, jitter_frac: float = 0.0,
          seed: int | None = None, traction: float | None = None, gravity: bool = True, **mat) -> Problem:
    coords, elems = grid(nx, ny, kind)
    if jitter_frac:
        coords = jitter(coords, nx, ny, jitter_frac, np.random.default_rng(seed))
    left = side_mask(coords, "left")
    conds = [(DIRICHLET_X, 0.0, left), (DIRICHLET_Y, 0.0, left)]
    edges = None
    if traction is not None:
        conds.append((NEUMANN_Y, -float(traction), side_mask(coords, "right")))
        edges = boundary_edges(nx, ny)
    p = Problem(name=name, kind=kind, coords=coords, elems=elems, stress=stress,
                forces=[(0.0, -GRAVITY)] if gravity else [], conds=conds, edges=edges)
    for k, v in {**STEEL, **mat}.items():
        setattr(p, k, v)
    return p


def cfg_small() -> Problem:
    """64x16 P1 plate, 1,105 nodes, 2,210 DOF, plane stress, gravity, left clamped."""
    return plate(64, 16, 3, name="p1_64x16")


def cfg_q1_large(nx: int = 1024, ny: int = 256) -> Problem:
    """1024x256 Q1 plate, interior nodes jittered by +-0.2h (seed 2), 1e6 Pa downward traction on the right edge."""
    return plate(nx, ny, 4, name=f"q1_{nx}x{ny}_jitter", jitter_frac=0.2, seed=2, traction=1e6)


def holes(coords: np.ndarray, elems: np.ndarray, n_holes: int, rng, lx=4.0, ly=1.0,
          rmin=0.005, rmax=0.02) -> np.ndarray:
    """Mask of elements whose centroid lies inside one of n_holes random circles."""
    cx = rng.uniform(0.0, lx, n_holes)
    cy = rng.uniform(0.0, ly, n_holes)
    r = rng.uniform(rmin, rmax, n_holes)
    cent = coords[elems].mean(axis=1)
    inside = np.zeros(len(elems), dtype=bool)
    # bucket the holes by a coarse grid to keep this O(E)
    for k in range(n_holes):
        d2 = (cent[:, 0] - cx[k]) ** 2 + (cent[:, 1] - cy[k]) ** 2
        inside |= d2 < r[k] ** 2
    return inside


def cfg_perforated(nx: int = 2048, ny: int = 512, n_holes: int = 200, seed: int = 3) -> Problem:
    """2048x512 P1 plate (1,051,137 nodes, 2,102,274 DOF) with 200 soft circular
    inclusions (E x 1e-3), radii U(0.005, 0.02) m, centres uniform (seed 3);
    left edge clamped, gravity, 1e6 Pa downward traction on the right edge."""
    p = plate(nx, ny, 3, name=f"p1_{nx}x{ny}_perforated", traction=1e6)
    inside = holes(p.coords, p.elems, n_holes, np.random.default_rng(seed))
    p.elem_E = np.where(inside, p.E * 1e-3, p.E).astype(np.float64)
    return p


def batch_uneven(n: int = 256, seed: int = 4) -> list[Problem]:
    """n independent plane-stress P1 plates: nx ~ U{32..256}, ny ~ U{8..64},
    per-element E log-uniform in [1e9, 2e11], nu ~ U(0.2, 0.35) per problem,
    one clamped side, a traction U(1e5, 1e7) Pa on another side."""
    rng = np.random.default_rng(seed)
    out = []
    sides = ["left", "right", "bottom", "top"]
    for k in range(n):
        nx = int(rng.integers(32, 257))
        ny = int(rng.integers(8, 65))
        coords, elems = grid(nx, ny, 3)
        clamp = sides[int(rng.integers(0, 4))]
        load = [s for s in sides if s != clamp][int(rng.integers(0, 3))]
        tr = float(rng.uniform(1e5, 1e7))
        nu = float(rng.uniform(0.2, 0.35))
        eE = np.exp(rng.uniform(np.log(1e9), np.log(2e11), len(elems)))
        cm = side_mask(coords, clamp)
        lm = side_mask(coords, load)
        # the traction is listed first, so a corner shared with the clamped side stays clamped
        conds = [(NEUMANN_Y, -tr, lm), (DIRICHLET_X, 0.0, cm), (DIRICHLET_Y, 0.0, cm)]
        out.append(Problem(name=f"batch{k}_{nx}x{ny}", kind=3, coords=coords, elems=elems, nu=nu, elem_E=eE,
                           forces=[], conds=conds, edges=boundary_edges(nx, ny)))
    return out


def neumann_edge_loads(p: Problem, node_offset: int = 0):
    """The Neumann X/Y conditions of p as per-edge tractions: every boundary
    edge with both end nodes flagged gets the condition's value in its
    component (edges shifted by node_offset).  Returns (edges (M, 2) int32,
    loads (M, 2) float64)."""
    ed, ld = [], []
    for kind, value, mask in p.conds:
        if kind not in (NEUMANN_X, NEUMANN_Y) or p.edges is None:
            continue
        sel = mask[p.edges[:, 0]] & mask[p.edges[:, 1]]
        e = p.edges[sel] + node_offset
        l = np.zeros((len(e), 2))
        l[:, 0 if kind == NEUMANN_X else 1] = value
        ed.append(e)
        ld.append(l)
    if not ed:
        return np.zeros((0, 2), np.int32), np.zeros((0, 2))
    return np.concatenate(ed).astype(np.int32), np.concatenate(ld)


def gauss_tables(kind: int):
    """Weights and shape tables of the reference's Gauss rules (rule.c:90-111,
    shape.c:3-85), as arrays (w[nq], phi[nq,kind], dxi[nq,kind], deta[nq,kind])."""
    if kind == 3:
        a, b = 1.0 / 6, 1 - 1.0 / 3
        pts = [(a, a), (b, a), (a, b)]
        w = np.full(3, 1.0 / 6)
        phi = np.array([[1 - x - e, x, e] for x, e in pts])
        dxi = np.tile([-1.0, 1.0, 0.0], (3, 1))
        deta = np.tile([-1.0, 0.0, 1.0], (3, 1))
    else:
        s = 0.577350269189626
        pts = [(-s, s), (-s, -s), (s, -s), (s, s)]
        w = np.ones(4)
        phi = np.array([[(1 + x) * (1 + e) / 4, (1 - x) * (1 + e) / 4, (1 - x) * (1 - e) / 4, (1 + x) * (1 - e) / 4]
                        for x, e in pts])
        dxi = np.array([[(1 + e) / 4, (-1 - e) / 4, (-1 + e) / 4, (1 - e) / 4] for x, e in pts])
        deta = np.array([[(1 + x) / 4, (1 - x) / 4, (-1 + x) / 4, (-1 - x) / 4] for x, e in pts])
    return w, phi, dxi, deta
