"""The allocation-free solve, bfm_gpu_pcg_solve_noalloc.

It exists for callers that cannot allocate device memory: its Krylov vectors
and solver state live in a fixed array inside the library.  Here it gets a
matrix assembled by the regular problem API, in device buffers the test owns,
and must return the solution of the regular entry point (bfm_gpu_problem_solve,
same FP64 Jacobi-PCG) within the tolerance of the parity tests, on two calls in
a row (the second call finds the first call's leftovers in the array), and the
FP64 direct solve of the oracle within the same tolerance."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import meshgen as M

pytestmark = pytest.mark.gpu

RTOL = 1e-12      # solver tolerance of both entry points
MATCH = 1e-10     # relative 2-norm agreement required (the FP64 parity tolerance)


def regular_solve(lib, p):
    """Assemble and solve with the regular entry points; return the system and x."""
    P = C.c_void_p()
    keep = []

    def a(x, dt):
        x = np.ascontiguousarray(x, dtype=dt)
        keep.append(x)
        return x.ctypes.data

    n_edges = 0 if p.edges is None else len(p.edges)
    assert lib.bfm_gpu_problem_create(C.byref(P), p.kind, p.n_nodes, p.n_elems, n_edges, len(p.conds), None) == 0
    assert lib.bfm_gpu_problem_set_geometry(P, a(p.coords, np.float64), a(p.elems, np.int32), 0) == 0
    assert lib.bfm_gpu_problem_set_material(P, p.E, p.nu, p.rho, int(p.stress), None, None, 0) == 0
    w, ph, dx, de = M.gauss_tables(p.kind)
    assert lib.bfm_gpu_problem_set_rule(P, len(w), a(w, np.float64), a(ph, np.float64), a(dx, np.float64),
                                        a(de, np.float64)) == 0
    f = np.array(p.forces, np.float64).reshape(-1)
    assert lib.bfm_gpu_problem_set_forces(P, len(p.forces), a(f, np.float64), None, 0) == 0
    masks = np.stack([c[2] for c in p.conds]).astype(np.uint8)
    assert lib.bfm_gpu_problem_set_conditions(P, len(p.conds), a([c[0] for c in p.conds], np.int32),
                                              a([c[1] for c in p.conds], np.float64), a(masks, np.uint8),
                                              n_edges, a(p.edges, np.int32) if n_edges else None, 0) == 0
    assert lib.bfm_gpu_problem_assemble(P, bfm_gb300.FP64) == 0
    o = bfm_gb300.default_opts(rtol=RTOL, autotune=0)
    assert lib.bfm_gpu_problem_solve(P, C.byref(o)) == 0
    s = bfm_gb300.bfm_gpu_stats_t()
    # 0: converged; 5: stopped at the FP64 roundoff floor above RTOL (as accurate as it gets)
    assert lib.bfm_gpu_problem_stats(P, C.byref(s)) == 0 and s.status in (0, 5)
    x = np.zeros(p.n_dof)
    assert lib.bfm_gpu_problem_solution(P, x.ctypes.data, 0) == 0
    nb = C.c_int64()
    assert lib.bfm_gpu_problem_n_blocks(P, C.byref(nb)) == 0
    rp = np.zeros(p.n_nodes + 1, np.int32)
    cols = np.zeros(nb.value, np.int32)
    vals = np.zeros(4 * nb.value)
    b = np.zeros(p.n_dof)
    assert lib.bfm_gpu_problem_download(P, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data, b.ctypes.data) == 0
    lib.bfm_gpu_problem_destroy(P)
    return rp, cols, vals, b, x


def test_noalloc_matches_regular_solve_twice(libbfm):
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    p = M.plate(96, 24, 3, traction=1e6)
    rp, cols, vals, b, x_ref = regular_solve(libbfm, p)
    x_dir, _, _ = O.solve_direct(p)
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(rp).to(dev)
    d_cols = torch.from_numpy(cols).to(dev)
    d_vals = torch.from_numpy(vals).to(dev)
    d_b = torch.from_numpy(b).to(dev)
    torch.cuda.synchronize()
    for call in range(2):
        d_x = torch.full((p.n_dof,), float("nan"), dtype=torch.float64, device=dev)
        it, res = C.c_int(), C.c_double()
        rc = libbfm.bfm_gpu_pcg_solve_noalloc(p.n_nodes, d_rp.data_ptr(), d_cols.data_ptr(), d_vals.data_ptr(),
                                              d_b.data_ptr(), d_x.data_ptr(), RTOL, 200000, C.byref(it),
                                              C.byref(res), None)
        assert rc == 0, bfm_gb300.last_error()
        x = d_x.cpu().numpy()
        err = np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)
        assert err < MATCH, f"call {call}: relative difference {err:.3e}"
        err_dir = np.linalg.norm(x - x_dir) / np.linalg.norm(x_dir)
        assert err_dir < MATCH, f"call {call}: relative error {err_dir:.3e} vs the direct oracle"
        assert it.value > 0 and res.value < 1e-8


def test_noalloc_rejects_oversized_problems(libbfm):
    it, res = C.c_int(), C.c_double()
    rc = libbfm.bfm_gpu_pcg_solve_noalloc(65537, None, None, None, None, None, 1e-8, 10, C.byref(it), C.byref(res), None)
    assert rc == -1
    assert "65536 nodes" in bfm_gb300.last_error()
