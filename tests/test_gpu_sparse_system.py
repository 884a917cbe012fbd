"""The lower-level system API (bfm_system_create_planar_*, bfm_system_renumber,
bfm_matrix_solve, bfm_perm_perm_vec; reference system.c:44-81, 531-538,
matrix.c:531-541, sim.c:103-135) with sparse storage.

The reference stores the system matrix dense: 8.9 GB at the 33,410 DOF of a
256x64 plate, and O(n^2) work to renumber it.  With BFM_MATRIX_KIND_SPARSE the
same call sequence runs in O(nnz) memory -- checked through the state's own
allocator hooks, which every host buffer of the library goes through: no
request comes near n^2 doubles -- and gives the reference's RCM permutation
bit for bit and the direct oracle's displacements to 1e-10."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import abi, api, meshgen as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_sparse_system_sequence_matches_oracle(libbfm):
    p = M.plate(256, 64, 3, jitter_frac=0.2, seed=7, traction=1e6)
    n = p.n_dof
    Ko, bo = O.assemble_csr(p)
    x_ref = O.solve_direct(p)[0]
    perm_ref, _ = O.rcm_csr(Ko)
    lib = libbfm
    h = api.SimHandle.from_problem(lib, p)
    # record the largest host allocation the library asks the state for
    largest = [0]
    libc = C.CDLL(None)
    libc.malloc.restype = C.c_void_p
    libc.malloc.argtypes = [C.c_size_t]
    libc.realloc.restype = C.c_void_p
    libc.realloc.argtypes = [C.c_void_p, C.c_size_t]

    @C.CFUNCTYPE(C.c_void_p, C.c_size_t)
    def alloc(size):
        largest[0] = max(largest[0], size)
        return libc.malloc(size)

    @C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_size_t)
    def realloc(ptr, size):
        largest[0] = max(largest[0], size)
        return libc.realloc(ptr, size)

    st = h.state
    old_hooks = (st.alloc, st.realloc)
    st.alloc = C.cast(alloc, C.c_void_p).value
    st.realloc = C.cast(realloc, C.c_void_p).value
    assert lib.bfm_gpu_set_system_storage(abi.MATRIX_SPARSE) == 0
    lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-12)))
    s = abi.bfm_system_t()
    try:
        rc = lib.bfm_system_create_planar_stress(C.byref(s), C.byref(h.instances[0]), h.sim.n_forces, h.sim.forces)
        assert rc == 0, h.error()
        assert s.A.kind == abi.MATRIX_SPARSE and s.A.m == n
        assert s.A.u.sparse.nnz % 4 == 0 and s.A.u.sparse.nnz >= Ko.nnz  # 4 per 2x2 block
        # entries and right-hand side as the oracle's (the FP64 assembly is bit-exact)
        b = np.ctypeslib.as_array(s.b.data, shape=(n,)).copy()
        assert np.abs(b - bo).max() <= 1e-14 * np.abs(bo).max()
        Kc = Ko.tocoo()
        pick = np.random.default_rng(0).choice(Kc.nnz, 200, replace=False)
        for k in pick:
            assert lib.bfm_matrix_get(C.byref(s.A), int(Kc.row[k]), int(Kc.col[k])) == Kc.data[k]
        # the reference's sequence: renumber (RCM), solve, inverse permutation
        assert lib.bfm_system_renumber(C.byref(s)) == 0
        assert s.A.kind == abi.MATRIX_SPARSE
        perm = np.ctypeslib.as_array(s.perm.perm, shape=(n,)).astype(np.int64)
        assert np.array_equal(perm, perm_ref)
        assert lib.bfm_matrix_solve(C.byref(s.A), C.byref(s.b)) == 0, bfm_gb300.last_error()
        assert lib.bfm_perm_perm_vec(C.byref(s.perm), C.byref(s.b), True) == 0
        x = np.ctypeslib.as_array(s.b.data, shape=(n,)).copy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-10
        # no dense storage: every request is far below n^2 doubles
        assert largest[0] < n * n * 8 // 1000, largest[0]
        # read-only storage
        assert lib.bfm_matrix_set(C.byref(s.A), 0, 0, 1.0) == -1
    finally:
        lib.bfm_system_destroy(C.byref(s))
        st.alloc, st.realloc = old_hooks
        lib.bfm_gpu_set_system_storage(abi.MATRIX_FULL)
        lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))
