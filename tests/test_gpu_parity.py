"""GPU path vs the reference (golden fixtures) and the FP64 direct oracle.

Tolerances: displacements 1e-10 relative (2-norm) to the reference for the
FP64 path; stiffness matrix, RCM permutation, pattern and Dirichlet masks
bit-exact."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api, meshgen as M
from common import CASES, dense_K, load, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PARITY_RTOL = 1e-10


@pytest.fixture(autouse=True)
def fp64_opts(libbfm):
    o = bfm_gb300.default_opts(rtol=1e-12)
    libbfm.bfm_gpu_set_opts(C.byref(o))
    yield
    libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


def stats(lib):
    s = bfm_gb300.bfm_gpu_stats_t()
    lib.bfm_gpu_last_stats(C.byref(s))
    return s


@pytest.mark.parametrize("name", CASES)
def test_sim_run_matches_reference(libbfm, name):
    p, d = load(name)
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0, h.error()
    s = stats(libbfm)
    # the FP64 true residual floors near eps*||K||*||u||/||b|| (K ~ 1e11, cond ~ 1e12 unscaled):
    # at rtol 1e-12 the solver may stop there (BFM_GPU_STAGNATED, 5) instead of at rtol
    assert s.status in (0, 5) and s.rel_residual < 1e-8
    assert rel(h.effects(), d["effects"]) < PARITY_RTOL


def test_lepl8_shipped_golden_files(libbfm):
    p, d = load("lepl8")
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0, h.error()
    e = h.effects()
    assert np.abs(e[0::2] - d["U_txt"]).max() <= 5e-8 * np.abs(d["U_txt"]).max()
    assert np.abs(e[1::2] - d["V_txt"]).max() <= 5e-8 * np.abs(d["V_txt"]).max()


@pytest.mark.parametrize("name", CASES)
def test_stiffness_rhs_and_rcm(libbfm, name):
    """K assembled on the GPU is bit-identical to the reference's; the RCM of
    its exact zeros is the reference's permutation."""
    p, d = load(name)
    h = api.SimHandle.from_problem(libbfm, p)
    K, b, perm = h.system(renumber=True)
    assert np.array_equal(K, dense_K(d, p.n_dof))
    assert rel(b, d["b"]) < 1e-14
    assert np.array_equal(perm, d["perm"])


def device_problem(lib, p, precision=0):
    P = C.c_void_p()
    n_edges = 0 if p.edges is None else len(p.edges)
    assert lib.bfm_gpu_problem_create(C.byref(P), p.kind, p.n_nodes, p.n_elems, n_edges, len(p.conds), None) == 0, \
        bfm_gb300.last_error()
    keep = []

    def a(x, dt):
        x = np.ascontiguousarray(x, dtype=dt)
        keep.append(x)
        return x.ctypes.data

    assert lib.bfm_gpu_problem_set_geometry(P, a(p.coords, np.float64), a(p.elems, np.int32), 0) == 0
    assert lib.bfm_gpu_problem_set_material(P, p.E, p.nu, p.rho, int(p.stress),
                                            None if p.elem_E is None else a(p.elem_E, np.float64),
                                            None if p.elem_nu is None else a(p.elem_nu, np.float64), 0) == 0
    w, ph, dx, de = M.gauss_tables(p.kind)
    assert lib.bfm_gpu_problem_set_rule(P, len(w), a(w, np.float64), a(ph, np.float64), a(dx, np.float64),
                                        a(de, np.float64)) == 0
    f = np.array(p.forces, np.float64).reshape(-1)
    assert lib.bfm_gpu_problem_set_forces(P, len(p.forces), a(f, np.float64) if len(f) else None, None, 0) == 0
    if p.conds:
        kinds = a([c[0] for c in p.conds], np.int32)
        vals = a([c[1] for c in p.conds], np.float64)
        masks = a(np.stack([c[2] for c in p.conds]).astype(np.uint8), np.uint8)
        edges = a(p.edges, np.int32) if p.edges is not None else None
        assert lib.bfm_gpu_problem_set_conditions(P, len(p.conds), kinds, vals, masks, n_edges, edges, 0) == 0
    assert lib.bfm_gpu_problem_assemble(P, precision) == 0, bfm_gb300.last_error()
    return P, keep


def download(lib, P, n_nodes):
    nb = C.c_int64()
    assert lib.bfm_gpu_problem_n_blocks(P, C.byref(nb)) == 0
    rp = np.zeros(n_nodes + 1, np.int32)
    cols = np.zeros(nb.value, np.int32)
    vals = np.zeros(4 * nb.value)
    b = np.zeros(2 * n_nodes)
    assert lib.bfm_gpu_problem_download(P, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data, b.ctypes.data) == 0
    return rp, cols, vals, b


@pytest.mark.parametrize("name", CASES)
def test_pattern_is_the_node_graph(libbfm, name):
    """Block pattern = pairs of nodes sharing an element (structural), columns ascending."""
    p, _ = load(name)
    P, _k = device_problem(libbfm, p)
    rp, cols, _, _ = download(libbfm, P, p.n_nodes)
    Kc, _ = O.assemble_csr(p)  # the oracle's structural scalar CSR, 2x2 blocks expanded
    node_pat = set()
    Kc = Kc.tocoo()
    for r, c in zip(Kc.row // 2, Kc.col // 2):
        node_pat.add((int(r), int(c)))
    got = {(r, int(c)) for r in range(p.n_nodes) for c in cols[rp[r]:rp[r + 1]]}
    assert got == node_pat
    for r in range(p.n_nodes):
        assert np.all(np.diff(cols[rp[r]:rp[r + 1]]) > 0)
    libbfm.bfm_gpu_problem_destroy(P)


@pytest.mark.parametrize("name", CASES)
def test_dirichlet_dof_masks(libbfm, name):
    """Constrained DOFs (rows reduced to the identity, b = value) match the reference."""
    p, d = load(name)
    P, _k = device_problem(libbfm, p)
    rp, cols, vals, b = download(libbfm, P, p.n_nodes)
    n = p.n_dof
    K = np.zeros((n, n))
    for r in range(p.n_nodes):
        for k in range(rp[r], rp[r + 1]):
            c = cols[k]
            K[2 * r:2 * r + 2, 2 * c:2 * c + 2] = vals[4 * k:4 * k + 4].reshape(2, 2)
    Kref = dense_K(d, n)
    eye_rows = lambda A: np.array([A[i, i] == 1.0 and np.count_nonzero(A[i]) == 1 and np.count_nonzero(A[:, i]) == 1
                                   for i in range(n)])
    assert np.array_equal(eye_rows(K), eye_rows(Kref))
    assert np.array_equal(K, Kref)
    libbfm.bfm_gpu_problem_destroy(P)


def test_repeat_runs_are_bit_identical(libbfm):
    p, _ = load("gear12")
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0
    e1 = h.effects()
    assert h.run() == 0
    assert np.array_equal(e1, h.effects())


@pytest.mark.parametrize("kind,nx,ny", [(4, 96, 24), (3, 128, 32)])
def test_medium_plates_vs_direct_oracle(libbfm, kind, nx, ny):
    p = M.plate(nx, ny, kind, jitter_frac=0.2, seed=3, traction=1e6)
    x, _, _ = O.solve_direct(p)
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0, h.error()
    assert rel(h.effects(), x) < 1e-9


def test_per_element_material(libbfm):
    p = M.cfg_perforated(nx=128, ny=32, n_holes=12, seed=3)
    x, _, _ = O.solve_direct(p)
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0, h.error()
    assert rel(h.effects(), x) < 1e-8


def test_valence_cap_reports_error_and_recovers(libbfm):
    # a fan of 40 triangles around node 0: more incident elements than the kernel cap
    n = 40
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    coords = np.vstack([[0.0, 0.0], np.stack([np.cos(ang), np.sin(ang)], 1)])
    elems = np.array([[0, 1 + i, 1 + (i + 1) % n] for i in range(n)], np.int64)
    ring = np.ones(n + 1, bool)
    ring[0] = False
    p = M.Problem("fan", 3, coords, elems, conds=[(M.DIRICHLET_X, 0.0, ring), (M.DIRICHLET_Y, 0.0, ring)],
                  forces=[(0.0, -9.81)])
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == -1
    assert "caps" in h.error()
    q, d = load("p1_12x6_conds")
    h2 = api.SimHandle.from_problem(libbfm, q)
    assert h2.run() == 0
    assert rel(h2.effects(), d["effects"]) < PARITY_RTOL


def test_bad_element_index_reports_error_and_recovers(libbfm):
    """An element referring to a node beyond the mesh is reported (the 64-bit
    ids are narrowed and checked on the device), and the same handle runs
    again once the element array is repaired."""
    p = M.plate(8, 4, 3)
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == 0
    good = h.effects().copy()
    elems = h.keep[1]  # the mesh's size_t element array (uint64, flat)
    old = int(elems[7])
    elems[7] = p.n_nodes + 5
    assert h.run() == -1
    assert "refers to node" in h.error() and f"element {7 // 3}" in h.error()
    elems[7] = old
    assert h.run() == 0
    assert np.array_equal(h.effects(), good)


def test_no_constraints_is_reported(libbfm):
    p = M.plate(8, 4, 3)
    p.conds = []
    h = api.SimHandle.from_problem(libbfm, p)
    assert h.run() == -1
    assert "positive definite" in h.error() or "not reach" in h.error()
