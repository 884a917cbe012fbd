"""Host-side logic of the library that runs without a GPU: sparse RCM,
dense/band matrices and permutations, mesh and problem-file readers, the
U/V writer, and the no-fallback rule."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from bfm_gb300 import abi
from common import CASES, GOLDEN, dense_K, gpu_available, load


def rcm_lib(lib, K):
    K = sp.csr_matrix(K)
    K.sort_indices()
    n = K.shape[0]
    rp = np.ascontiguousarray(K.indptr, np.int64)
    ci = np.ascontiguousarray(K.indices, np.int64)
    v = np.ascontiguousarray(K.data, np.float64)
    perm, inv = np.zeros(n, np.int64), np.zeros(n, np.int64)
    assert lib.bfm_gpu_rcm_csr(n, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, perm.ctypes.data, inv.ctypes.data) == 0
    return perm, inv


@pytest.mark.parametrize("name", CASES)
def test_sparse_rcm_bit_exact(libbfm, name):
    p, d = load(name)
    K = dense_K(d, p.n_dof)
    perm, inv = rcm_lib(libbfm, K)
    assert np.array_equal(perm, d["perm"])
    assert np.array_equal(inv[perm], np.arange(p.n_dof))


def test_sparse_rcm_ignores_stored_zeros(libbfm):
    _, d = load("p1_64x16")
    n = 2 * 1105
    K = sp.coo_matrix((d["K_vals"], (d["K_rows"], d["K_cols"])), shape=(n, n)).tocsr()
    # add explicit zeros where the mesh has structure but the value vanished
    Z = K.copy().tolil()
    rng = np.random.default_rng(0)
    for i in rng.integers(0, n, 200):
        j = min(n - 1, i + 1)
        if Z[i, j] == 0:
            Z[i, j] = 0.0
    perm, _ = rcm_lib(libbfm, Z.tocsr())
    assert np.array_equal(perm, d["perm"])


def make_full(lib, st, A):
    m = abi.bfm_matrix_t()
    n = A.shape[0]
    assert lib.bfm_matrix_full_create(C.byref(m), C.byref(st), abi.MAJOR_ROW, n) == 0
    for i in range(n):
        for j in range(n):
            lib.bfm_matrix_set(C.byref(m), i, j, float(A[i, j]))
    return m


def test_dense_and_band_lu(libbfm):
    lib = libbfm
    st = abi.bfm_state_t()
    lib.bfm_state_create(C.byref(st))
    rng = np.random.default_rng(1)
    n, k = 12, 2
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - k), min(n, i + k + 1)):
            A[i, j] = rng.uniform(-1, 1)
        A[i, i] = 10.0
    y = rng.uniform(-1, 1, n)
    m = make_full(lib, st, A)
    assert lib.bfm_matrix_bandwidth(C.byref(m)) == k
    band = abi.bfm_matrix_t()
    assert lib.bfm_matrix_band_create(C.byref(band), C.byref(st), abi.MAJOR_ROW, n, k) == 0
    assert lib.bfm_matrix_copy(C.byref(band), C.byref(m)) == 0
    # band storage index j + i*2k (row-major), as the reference lays it out
    assert band.band.data[3 + 2 * 2 * k] == A[2, 3]
    assert np.isnan(lib.bfm_matrix_get(C.byref(band), n, 0))
    assert lib.bfm_matrix_get(C.byref(band), 0, n - 1) == 0.0
    assert lib.bfm_matrix_set(C.byref(band), 0, n - 1, 1.0) == -1
    for mat in (m, band):
        v = abi.bfm_vec_t()
        lib.bfm_vec_create(C.byref(v), C.byref(st), n)
        for i in range(n):
            v.data[i] = y[i]
        assert lib.bfm_matrix_solve(C.byref(mat), C.byref(v)) == 0
        x = np.array([v.data[i] for i in range(n)])
        assert np.allclose(A @ x, y, rtol=1e-12, atol=1e-12)
    # zero pivot fails like the reference (|pivot| < 1e-20)
    Z = make_full(lib, st, np.zeros((3, 3)))
    assert lib.bfm_matrix_lu(C.byref(Z)) == -1


def test_perm_rcm_on_dense_matrix(libbfm):
    p, d = load("p1_20x10_shuffled")
    st = abi.bfm_state_t()
    libbfm.bfm_state_create(C.byref(st))
    n = p.n_dof
    m = abi.bfm_matrix_t()
    libbfm.bfm_matrix_full_create(C.byref(m), C.byref(st), abi.MAJOR_ROW, n)
    K = dense_K(d, n)
    C.memmove(m.full.data, K.ctypes.data, K.nbytes)
    perm = abi.bfm_perm_t()
    libbfm.bfm_perm_create(C.byref(perm), C.byref(st), n)
    assert libbfm.bfm_perm_rcm(C.byref(perm), C.byref(m)) == 0
    got = np.array([perm.perm[i] for i in range(n)])
    assert np.array_equal(got, d["perm"])
    # permute the matrix and a vector, then undo the vector permutation
    assert libbfm.bfm_perm_perm_matrix(C.byref(perm), C.byref(m), False) == 0
    Kp = np.ctypeslib.as_array(m.full.data, shape=(n * n,)).reshape(n, n)
    assert np.array_equal(Kp[np.ix_(got, got)], K)
    v = abi.bfm_vec_t()
    libbfm.bfm_vec_create(C.byref(v), C.byref(st), n)
    x = np.arange(n, dtype=float)
    C.memmove(v.data, x.ctypes.data, x.nbytes)
    libbfm.bfm_perm_perm_vec(C.byref(perm), C.byref(v), False)
    libbfm.bfm_perm_perm_vec(C.byref(perm), C.byref(v), True)
    assert np.array_equal(np.ctypeslib.as_array(v.data, shape=(n,)), x)


def write_lepl1110(path, d, with_edges=True):
    coords, elems, edges = d["coords"], d["elems"], d["edges"]
    lines = [f"Number of nodes {len(coords)} "]
    lines += [f"{i:6d} : {x:14.7e} {y:14.7e} " for i, (x, y) in enumerate(coords)]
    if with_edges:
        lines.append(f"Number of edges {len(edges)} ")
        lines += [f"{i:6d} : {a:6d} {b:6d} " for i, (a, b) in enumerate(edges)]
    word = "triangles" if elems.shape[1] == 3 else "quads"
    lines.append(f"Number of {word} {len(elems)} ")
    lines += [f"{i:6d} : " + " ".join(f"{v:6d}" for v in e) for i, e in enumerate(elems)]
    if with_edges and "domain_names" in d:
        names, ptr, de = d["domain_names"], d["domain_ptr"], d["domain_edges"]
        lines.append(f"Number of domains {len(names)}")
        for k, nm in enumerate(names):
            lines += [f"  Domain : {k:6d} ", f"  Name : {nm}", f"  Number of elements : {ptr[k + 1] - ptr[k]:6d}"]
            vals = de[ptr[k]:ptr[k + 1]]
            for s in range(0, len(vals), 10):
                lines.append("".join(f"{v:6d}" for v in vals[s:s + 10]))
    path.write_text("\n".join(lines) + "\n")


PROBLEM = """Type of problem    :  Planar strains
Young modulus      :  2.1100000e+11
Poisson ratio      :  3.0000000e-01
Mass density       :  7.8500000e+03
Gravity            :  9.8100000e+00
Boundary condition :  Dirichlet-X        =  0.0000000e+00 : Symmetry
Boundary condition :  Dirichlet-Y        =  0.0000000e+00 : Bottom
"""


def test_lepl1110_reader_and_problem_parser(libbfm, tmp_path):
    p, d = load("lepl8")
    # coordinates go through %14.7e text, as in the reference's mesh files
    write_lepl1110(tmp_path / "m.lepl1110", d)
    (tmp_path / "problem.txt").write_text(PROBLEM)
    st = abi.bfm_state_t()
    libbfm.bfm_state_create(C.byref(st))
    mesh = abi.bfm_mesh_t()
    assert libbfm.bfm_mesh_read_lepl1110(C.byref(mesh), C.byref(st), str(tmp_path / "m.lepl1110").encode()) == 0
    assert (mesh.n_nodes, mesh.n_elems, mesh.n_edges, mesh.kind, mesh.dim) == (335, 280, 108, 4, 2)
    elems = np.ctypeslib.as_array(mesh.elems, shape=(280 * 4,)).reshape(-1, 4)
    assert np.array_equal(elems, d["elems"])
    coords = np.ctypeslib.as_array(mesh.coords, shape=(335 * 2,)).reshape(-1, 2)
    assert np.allclose(coords, d["coords"], rtol=1e-7, atol=0)
    assert mesh.domains[0].name.decode().strip() == "Symmetry"
    ez = abi.bfm_ez_lepl1110_t()
    assert libbfm.bfm_ez_lepl1110_create(C.byref(ez), C.byref(st), C.byref(mesh),
                                         str(tmp_path / "problem.txt").encode()) == 0
    assert ez.sim.kind == abi.SIM_PLANAR_STRAIN
    assert (ez.material.E, ez.material.nu, ez.material.rho) == (2.11e11, 0.3, 7850.0)
    assert ez.sim.n_forces == 1 and ez.gravity.linear.force.data[1] == -9.81
    assert ez.instance.n_conditions == 2
    for c in range(2):
        cond = ez.instance.conditions[c].contents
        mask = np.array([cond.nodes[i] for i in range(335)])
        assert cond.kind == p.conds[c][0]
        assert np.array_equal(mask, p.conds[c][2])
    # writer: %14.7e, three per line, byte-compatible with the reference's rule
    eff = d["effects"]
    C.memmove(ez.instance.effects, eff.ctypes.data, eff.nbytes)
    assert libbfm.bfm_ez_lepl1110_write(C.byref(ez), 0, str(tmp_path / "U.txt").encode()) == 0
    expect = "Number of nodes 335\n"
    for i in range(335):
        expect += "%14.7e" % eff[2 * i]
        if i + 1 != 670 and (i + 1) % 3 == 0:
            expect += "\n"
    expect += "\n"
    assert (tmp_path / "U.txt").read_text() == expect
    # the reference's shipped golden file carries the same numbers
    got = np.array([float(expect.splitlines()[1 + i // 3][14 * (i % 3):14 * (i % 3) + 14]) for i in range(335)])
    assert np.allclose(got, d["U_txt"], rtol=0, atol=1e-20)
    libbfm.bfm_ez_lepl1110_destroy(C.byref(ez))


def test_lepl1110_reader_without_edge_section(libbfm, tmp_path):
    _, d = load("gear12")
    write_lepl1110(tmp_path / "g.lepl1110", d, with_edges=False)
    st = abi.bfm_state_t()
    libbfm.bfm_state_create(C.byref(st))
    mesh = abi.bfm_mesh_t()
    assert libbfm.bfm_mesh_read_lepl1110(C.byref(mesh), C.byref(st), str(tmp_path / "g.lepl1110").encode()) == 0
    assert (mesh.n_nodes, mesh.n_elems, mesh.n_edges, mesh.kind) == (4418, 8186, 0, 3)


@pytest.mark.parametrize("name", ["test", "bridge", "square"])
def test_wavefront_reader_matches_reference(libbfm, tmp_path, name):
    """bfm_mesh_read_wavefront (mesh.c:203-279) and its edge list (compute_edges,
    mesh.c:52-102) against the reference library's output on two of its own
    meshes and a two-triangle square (tests/golden/obj_*.npz): vertices, faces,
    and every edge in order -- end nodes, both adjacent elements -- bit for bit,
    including the reference's dropping of an unpaired last half-edge."""
    d = np.load(GOLDEN / f"obj_{name}.npz")
    path = tmp_path / f"{name}.obj"
    with open(path, "w") as f:
        f.write("# vertices and faces as the reference read them\no shape\n")
        for x, y in d["coords"]:
            f.write(f"v {float(x)!r} {float(y)!r} 0.000000\n")
        f.write("s 0\n")
        for a, b, c in d["elems"] + 1:
            f.write(f"f {a} {b} {c}\n")
    st = abi.bfm_state_t()
    libbfm.bfm_state_create(C.byref(st))
    mesh = abi.bfm_mesh_t()
    assert libbfm.bfm_mesh_read_wavefront(C.byref(mesh), C.byref(st), str(path).encode(), False) == 0
    n, m, ne = mesh.n_nodes, mesh.n_elems, mesh.n_edges
    assert (n, m, ne) == (len(d["coords"]), len(d["elems"]), len(d["edge_nodes"]))
    assert np.array_equal(np.ctypeslib.as_array(mesh.coords, shape=(2 * n,)).reshape(n, 2), d["coords"])
    assert np.array_equal(np.ctypeslib.as_array(mesh.elems, shape=(3 * m,)).reshape(m, 3), d["elems"])
    ed = np.array([(mesh.edges[i].nodes[0], mesh.edges[i].nodes[1], mesh.edges[i].elems[0], mesh.edges[i].elems[1])
                   for i in range(ne)], np.int64)
    assert np.array_equal(ed[:, :2], d["edge_nodes"])
    assert np.array_equal(ed[:, 2:], d["edge_elems"])
    libbfm.bfm_mesh_destroy(C.byref(mesh))


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU behaviour")
def test_no_cpu_fallback(libbfm):
    from bfm_gb300 import api
    p, _ = load("p1_12x6_conds")
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == -1
    assert "no CUDA device" in h.error()
