"""Generate tests/golden/*.npz from the reference libbfm itself.

Run in a tree where the reference sources exist (it compiles them into
oracle/_ref/ with oracle/Makefile):

    python tests/golden/make_golden.py [--reference /path/to/bfm]

Every fixture holds the problem's input arrays and what the reference library
returned for it through its own public API (bfm_sim_run for displacements;
bfm_system_create_planar_* + bfm_system_renumber for the assembled matrix, the
right-hand side and the RCM permutation).  The 8.lepl1110 case also holds the
values of the reference's shipped golden files data/U.txt and data/V.txt; the
obj_*.npz files hold what its Wavefront reader made of two of its meshes.
The GPU machine never needs the reference tree: tests read only these files.
"""
from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent


def parse_lepl1110(path: Path):
    """Nodes, edges, elements and domains of a LEPL1110 mesh file."""
    lines = path.read_text().splitlines()
    i = 0
    coords, edges, elems, domains = [], [], [], {}
    kind = None
    while i < len(lines):
        t = lines[i].strip()
        if t.startswith("Number of nodes"):
            n = int(t.split()[-1])
            coords = [tuple(map(float, lines[i + 1 + k].split(":")[1].split())) for k in range(n)]
            i += n
        elif t.startswith("Number of edges"):
            n = int(t.split()[-1])
            edges = [tuple(map(int, lines[i + 1 + k].split(":")[1].split())) for k in range(n)]
            i += n
        elif t.startswith("Number of triangles") or t.startswith("Number of quads"):
            kind = 3 if "triangles" in t else 4
            n = int(t.split()[-1])
            elems = [tuple(map(int, lines[i + 1 + k].split(":")[1].split())) for k in range(n)]
            i += n
        elif t.startswith("Domain"):
            name = lines[i + 1].split(":", 1)[1].strip()
            cnt = int(lines[i + 2].split(":")[1])
            vals = []
            j = i + 3
            while len(vals) < cnt:
                vals += [int(v) for v in lines[j].split()]
                j += 1
            domains[name] = vals
            i = j - 1
        i += 1
    return (np.array(coords, np.float64), np.array(edges, np.int64), np.array(elems, np.int64), kind, domains)


def read_golden_values(path: Path) -> np.ndarray:
    txt = path.read_text().splitlines()[1:]
    vals = []
    for line in txt:
        for k in range(0, len(line), 14):
            chunk = line[k:k + 14].strip()
            if chunk:
                vals.append(float(chunk))
    return np.array(vals)


def save(name: str, p, h, extra: dict | None = None, system: bool = True):
    from bfm_gb300 import meshgen as M
    eff = h.effects()
    d = dict(kind=p.kind, stress=int(p.stress), coords=p.coords, elems=p.elems, E=p.E, nu=p.nu, rho=p.rho,
             forces=np.array(p.forces, np.float64).reshape(-1, 2),
             cond_kind=np.array([c[0] for c in p.conds], np.int32),
             cond_value=np.array([c[1] for c in p.conds], np.float64),
             cond_nodes=np.packbits(np.stack([np.asarray(c[2], bool) for c in p.conds]), axis=1),
             edges=p.edges if p.edges is not None else np.zeros((0, 2), np.int64),
             effects=eff)
    if p.edge_boundary is not None:
        d["edge_boundary"] = np.asarray(p.edge_boundary, np.uint8)
    if system:
        K, b, perm = h.system(renumber=True)
        nz = np.nonzero(K)
        d.update(K_rows=nz[0].astype(np.int32), K_cols=nz[1].astype(np.int32), K_vals=K[nz], b=b, perm=perm)
    d.update(extra or {})
    np.savez_compressed(OUT / f"{name}.npz", **d)
    print(f"{name}: N={p.n_nodes} E={p.n_elems} |u|max={np.abs(eff).max():.3e}", file=sys.stderr)


def main():
    from oracle import oracle as O
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("BFM_REFERENCE", str(O.REF_TREE)))
    ap.add_argument("--only", default=None, help="regenerate one fixture")
    args = ap.parse_args()
    os.environ["BFM_REFERENCE"] = args.reference
    O.REF_TREE = Path(args.reference)
    from bfm_gb300 import api, meshgen as M
    R = O.ref_lib()
    assert R is not None, "reference sources not found"
    ref = Path(args.reference)

    if args.only in (None, "p1_16x8_nt"):
        normal_tangent_case(R, api, M)
    if args.only in (None, "axi"):
        axisymmetric_cases(R, api, M)
    if args.only in (None, "obj"):
        wavefront_cases(R, ref)
    if args.only is not None:
        return

    # 1. the reference's own fixture: Q1 mesh, planar strain, gravity, two Dirichlet domains
    coords, edges, elems, kind, domains = parse_lepl1110(ref / "meshes" / "8.lepl1110")
    N = len(coords)

    def dom_mask(name):
        m = np.zeros(N, bool)
        for e in domains[name]:
            m[edges[e]] = True
        return m

    p = M.Problem("lepl8", kind, coords, elems, E=2.11e11, nu=0.3, rho=7850.0, stress=False,
                  forces=[(0.0, -9.81)], conds=[(M.DIRICHLET_X, 0.0, dom_mask("Symmetry")),
                                                (M.DIRICHLET_Y, 0.0, dom_mask("Bottom"))], edges=edges)
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    U = read_golden_values(ref / "data" / "U.txt")
    V = read_golden_values(ref / "data" / "V.txt")
    names = np.array(list(domains.keys()))
    dom_edges = [np.array(domains[k], np.int64) for k in domains]
    save("lepl8", p, h, dict(U_txt=U, V_txt=V, domain_names=names,
                             domain_ptr=np.cumsum([0] + [len(v) for v in dom_edges]),
                             domain_edges=np.concatenate(dom_edges)))

    # 2. 64x16 P1 plate, plane stress, gravity, left edge clamped
    p = M.cfg_small()
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("p1_64x16", p, h)

    # 3. jittered Q1 plate with a right-edge traction
    p = M.plate(24, 8, 4, name="q1_24x8_jitter", jitter_frac=0.2, seed=7, traction=1e6)
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("q1_24x8_jitter", p, h)

    # 4. condition-order semantics: non-zero and repeated Dirichlet values,
    #    Neumann before and after Dirichlet on shared nodes, plane strain
    coords, el = M.grid(12, 6, 3)
    left, right = M.side_mask(coords, "left"), M.side_mask(coords, "right")
    bottom, top = M.side_mask(coords, "bottom"), M.side_mask(coords, "top")
    conds = [(M.NEUMANN_X, 2e5, right), (M.DIRICHLET_X, 1e-4, left), (M.DIRICHLET_Y, 0.0, left),
             (M.DIRICHLET_X, -2e-4, left & (coords[:, 1] > 0.5)), (M.NEUMANN_Y, -3e5, top),
             (M.DIRICHLET_Y, 5e-5, bottom & (coords[:, 0] > 3.0)), (M.NEUMANN_Y, 1e5, bottom)]
    p = M.Problem("p1_12x6_conds", 3, coords, el, stress=False, forces=[(0.0, -9.81), (1.5, 0.0)], conds=conds,
                  edges=M.boundary_edges(12, 6))
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("p1_12x6_conds", p, h)

    # 5. jittered P1 plate with shuffled node numbering (an unbanded matrix for RCM)
    rng = np.random.default_rng(11)
    base = M.plate(20, 10, 3, jitter_frac=0.25, seed=5)
    order = rng.permutation(base.n_nodes)      # new id of old node
    inv = np.argsort(order)
    p = M.Problem("p1_20x10_shuffled", 3, base.coords[inv], order[base.elems], forces=base.forces,
                  conds=[(k, v, m[inv]) for k, v, m in base.conds])
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("p1_20x10_shuffled", p, h)

    # 6. an unstructured P1 mesh from the reference's meshes (no edge section:
    #    the reference reader cannot load it, so it goes in through the C API)
    coords, _, elems, kind, _ = parse_lepl1110(ref / "meshes" / "gear12.lepl1110")
    hub = np.hypot(coords[:, 0], coords[:, 1]) < 10.0
    p = M.Problem("gear12", 3, coords, elems, stress=True, forces=[(0.0, -9.81)],
                  conds=[(M.DIRICHLET_X, 0.0, hub), (M.DIRICHLET_Y, 0.0, hub)])
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("gear12", p, h)


def normal_tangent_case(R, api, M):
    """Normal and tangent conditions (system.c:388-425, 500-522) mixed with
    X/Y ones, in an order that exercises the first/last-value and
    load-survival rules; the edge list holds interior edges too, which the
    normal/tangent Dirichlet sums must skip (one adjacent element only)."""
    nx, ny = 16, 8
    coords, el = M.grid(nx, ny, 3)
    w = nx + 1
    bnd = M.boundary_edges(nx, ny)
    inner = np.array([(4 * w + i, 4 * w + i + 1) for i in range(nx)], np.int64)
    edges = np.concatenate([bnd, inner])
    eb = np.concatenate([np.ones(len(bnd), bool), np.zeros(len(inner), bool)])
    x, y = coords[:, 0], coords[:, 1]
    left, right = M.side_mask(coords, "left"), M.side_mask(coords, "right")
    bottom, top = M.side_mask(coords, "bottom"), M.side_mask(coords, "top")
    DN, DT, NN, NT = 6, 7, 4, 5
    conds = [(DN, 3e-5, x < 0.6), (M.DIRICHLET_X, 0.0, left), (M.DIRICHLET_Y, 0.0, left),
             (NT, 2e5, top), (NN, -3e5, right), (DT, 5e-5, bottom & (x > 3.0)), (NN, 1e5, bottom),
             (DN, 2e-5, right & (y > 0.8))]
    p = M.Problem("p1_16x8_nt", 3, coords, el, stress=True, forces=[(0.0, -9.81)], conds=conds, edges=edges,
                  edge_boundary=eb)
    h = api.SimHandle.from_problem(R, p, elem_material=False)
    assert h.run() == 0
    save("p1_16x8_nt", p, h)


def axisymmetric_cases(R, api, M):
    """Axisymmetric systems (system.c:229-356, 539-622) with x the radius:
    an annular section r in [1, 4], z in [0, 2], P1 and Q1, body force,
    Neumann X/Y loads, a normal load (which that system skips) and Dirichlet
    conditions in interleaved order.  stress=3 marks the reference's own
    formulas; its band solve of the resulting (indefinite) K is kept too."""
    for name, kind, nx, ny in (("axi_p1_12x8", 3, 12, 8), ("axi_q1_10x6", 4, 10, 6)):
        grid, el = M.grid(nx, ny, kind)   # [0, 4] x [0, 1]
        left, right = M.side_mask(grid, "left"), M.side_mask(grid, "right")
        bottom, top = M.side_mask(grid, "bottom"), M.side_mask(grid, "top")
        coords = np.stack([1.0 + grid[:, 0] * 0.75, grid[:, 1] * 2.0], axis=1)
        y = coords[:, 1]
        NN = 4  # Neumann normal
        conds = [(M.NEUMANN_X, 2e5, left), (M.DIRICHLET_Y, 0.0, bottom), (M.NEUMANN_Y, -1e5, top),
                 (NN, 1e5, right), (M.DIRICHLET_X, 1e-5, right & (y < 0.5)), (M.NEUMANN_X, -5e4, right)]
        p = M.Problem(name, kind, coords, el, stress=3, forces=[(0.0, -9.81)], conds=conds,
                      edges=M.boundary_edges(nx, ny))
        h = api.SimHandle.from_problem(R, p, elem_material=False)
        assert h.run() == 0
        save(name, p, h)


def parse_obj(path: Path):
    """Vertices (x, y) and triangles (0-based) of a Wavefront file."""
    xy, tri = [], []
    for line in path.read_text().splitlines():
        t = line.split()
        if t and t[0] == "v":
            xy.append((float(t[1]), float(t[2])))
        elif t and t[0] == "f":
            tri.append(tuple(int(v.split("/")[0]) - 1 for v in t[1:4]))
    return np.array(xy, np.float64), np.array(tri, np.int64)


def wavefront_cases(R, ref: Path):
    """The reference's Wavefront reader (mesh.c:203-279) with its edge
    extraction (compute_edges, mesh.c:52-102) on two of its own meshes: the
    vertices and faces it read, and its edge list in order -- end nodes in the
    order kept, the two adjacent elements (-1: none).  The test writes the
    vertices and faces back as a Wavefront file for the reader under test."""
    import ctypes as C
    import tempfile
    from bfm_gb300 import abi
    # a unit square of two triangles: its last sorted half-edge is unpaired
    tmp = Path(tempfile.mkdtemp()) / "square.obj"
    tmp.write_text("o sq\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3\nf 1 3 4\n")
    for name, path in (("test", ref / "meshes" / "test.obj"), ("bridge", ref / "meshes" / "bridge.obj"),
                       ("square", tmp)):
        st = abi.bfm_state_t()
        assert R.bfm_state_create(C.byref(st)) == 0
        mesh = abi.bfm_mesh_t()
        assert R.bfm_mesh_read_wavefront(C.byref(mesh), C.byref(st), str(path).encode(), False) == 0
        n, m, ne = mesh.n_nodes, mesh.n_elems, mesh.n_edges
        coords = np.ctypeslib.as_array(mesh.coords, shape=(n * 2,)).reshape(n, 2).copy()
        elems = np.ctypeslib.as_array(mesh.elems, shape=(m * 3,)).reshape(m, 3).astype(np.int64)
        ed = np.array([(mesh.edges[i].nodes[0], mesh.edges[i].nodes[1], mesh.edges[i].elems[0], mesh.edges[i].elems[1])
                       for i in range(ne)], np.int64)
        xy, tri = parse_obj(path)
        assert np.array_equal(xy, coords) and np.array_equal(tri, elems)
        np.savez_compressed(OUT / f"obj_{name}.npz", coords=coords, elems=elems, edge_nodes=ed[:, :2],
                            edge_elems=ed[:, 2:])
        print(f"obj_{name}: N={n} E={m} edges={ne}", file=sys.stderr)


if __name__ == "__main__":
    main()
