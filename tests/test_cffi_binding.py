"""The drop-in boundary as the reference binds it.

pybfm builds its Python module with cffi in API mode
(pybfm/bfm/gen_libbfm.py:11-48): the fifteen public headers, each with its
#include and #define lines stripped, go to ffi.cdef; the generated C source
includes the same headers and links -lbfm.  Here the same recipe runs over
this repository's include/bfm/*.h and links bfm_gb300/lib/libbfm.so, and the
resulting module drives the library the way pybfm does (ffi.new structs,
fields read directly, `assert not lib.<call>`): the LEPL1110 mesh reader and
problem parser on the reference's 8.lepl1110 case, the U/V writer, the dense
API's RCM and band solve, and bfm_sim_run (which, without a GPU, must fail
cleanly with its error record filled; with one, it must reproduce the
reference's golden displacements)."""
import importlib.util
import re
from pathlib import Path

import numpy as np
import pytest

from common import gpu_available, load
from test_host import PROBLEM, write_lepl1110

ROOT = Path(__file__).resolve().parents[1]
HEADERS = ["bfm/bfm.h", "bfm/math.h", "bfm/force.h", "bfm/material.h", "bfm/matrix.h", "bfm/mesh.h",
           "bfm/condition.h", "bfm/shape.h", "bfm/rule.h", "bfm/obj.h", "bfm/instance.h", "bfm/sim.h", "bfm/ez.h",
           "bfm/perm.h", "bfm/system.h"]


@pytest.fixture(scope="module")
def ffi_lib(libbfm_path, tmp_path_factory):
    cffi = pytest.importorskip("cffi")
    out = tmp_path_factory.mktemp("cffi")
    ffi = cffi.FFI()
    includes = ""
    for h in HEADERS:
        includes += f"#include <{h}>\n"
        src = (ROOT / "include" / h).read_text()
        src = re.sub("#include.*", "", src)
        src = re.sub("#define.*", "", src)
        ffi.cdef(src)
    libdir = str(Path(libbfm_path).parent)
    ffi.set_source("bfm_cffi_binding", includes, include_dirs=[str(ROOT / "include")], library_dirs=[libdir],
                   libraries=["bfm"], extra_link_args=[f"-Wl,-rpath,{libdir}"])
    so = ffi.compile(tmpdir=str(out))
    spec = importlib.util.spec_from_file_location("bfm_cffi_binding", so)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.ffi, mod.lib


def test_module_binds_every_reference_prototype(ffi_lib):
    ffi, lib = ffi_lib
    for name in ("bfm_state_create", "bfm_mesh_read_lepl1110", "bfm_mesh_read_wavefront", "bfm_ez_lepl1110_create",
                 "bfm_ez_lepl1110_write", "bfm_sim_run", "bfm_system_create_planar_stress", "bfm_system_renumber",
                 "bfm_matrix_solve", "bfm_perm_rcm", "bfm_instance_create", "bfm_condition_create"):
        assert callable(getattr(lib, name))
    # struct layouts the Python side touches directly (pybfm's condition.py:29,
    # instance.py:89-90, ez.py:22)
    assert ffi.sizeof("bfm_state_t") > 0 and ffi.offsetof("bfm_mesh_t", "coords") > 0


def test_lepl1110_case_through_the_binding(ffi_lib, tmp_path):
    ffi, lib = ffi_lib
    p, d = load("lepl8")
    write_lepl1110(tmp_path / "8.lepl1110", d)
    (tmp_path / "problem.txt").write_text(PROBLEM)
    state = ffi.new("bfm_state_t*")
    assert not lib.bfm_state_create(state)
    mesh = ffi.new("bfm_mesh_t*")
    assert not lib.bfm_mesh_read_lepl1110(mesh, state, str(tmp_path / "8.lepl1110").encode())
    assert (mesh.n_nodes, mesh.n_elems, mesh.kind) == (335, 280, 4)
    ez = ffi.new("bfm_ez_lepl1110_t*")
    assert not lib.bfm_ez_lepl1110_create(ez, state, mesh, str(tmp_path / "problem.txt").encode())
    assert ez.sim.kind == lib.BFM_SIM_KIND_PLANAR_STRAIN
    assert ez.instance.n_conditions == 2
    rc = lib.bfm_sim_run(ffi.addressof(ez.sim))
    if gpu_available():
        assert rc == 0
        eff = np.frombuffer(ffi.buffer(ez.instance.effects, 8 * 670), np.float64)
        assert np.abs(eff[0::2] - d["U_txt"]).max() <= 5e-8 * np.abs(d["U_txt"]).max()
        assert np.abs(eff[1::2] - d["V_txt"]).max() <= 5e-8 * np.abs(d["V_txt"]).max()
    else:
        # no CPU fallback: -1 and a filled error record, nothing written
        assert rc == -1
        assert state.err.has and b"no CUDA device" in ffi.string(state.err.msg)
        eff = d["effects"]
        ffi.memmove(ez.instance.effects, eff.tobytes(), eff.nbytes)
    assert not lib.bfm_ez_lepl1110_write(ez, 0, str(tmp_path / "U.txt").encode())
    got = np.array([float(v) for line in (tmp_path / "U.txt").read_text().splitlines()[1:]
                    for v in (line[k:k + 14] for k in range(0, len(line), 14)) if v.strip()])
    assert np.abs(got - d["U_txt"]).max() <= 5e-8 * np.abs(d["U_txt"]).max()
    assert not lib.bfm_ez_lepl1110_destroy(ez)


def test_dense_api_through_the_binding(ffi_lib):
    """bfm_perm_rcm and bfm_matrix_solve (band LU) on a small SPD matrix,
    against the oracle's restatement of the reference algorithms."""
    from oracle import oracle as O
    ffi, lib = ffi_lib
    n = 12
    rng = np.random.default_rng(5)
    A = np.zeros((n, n))
    for i in range(n):
        for j in (i + 3, i + 7):
            if j < n:
                A[i, j] = A[j, i] = -rng.uniform(0.5, 1.0)
    A += np.diag(np.abs(A).sum(1) + 1.0)
    b = rng.standard_normal(n)
    state = ffi.new("bfm_state_t*")
    assert not lib.bfm_state_create(state)
    M = ffi.new("bfm_matrix_t*")
    assert not lib.bfm_matrix_full_create(M, state, lib.BFM_MATRIX_MAJOR_ROW, n)
    ffi.memmove(M.full.data, A.tobytes(), A.nbytes)
    perm = ffi.new("bfm_perm_t*")
    assert not lib.bfm_perm_create(perm, state, n)
    assert not lib.bfm_perm_rcm(perm, M)
    got = np.frombuffer(ffi.buffer(perm.perm, 8 * n), np.uint64).astype(np.int64)
    ref, _ = O.rcm_dense(A)
    assert np.array_equal(got, ref)
    x = ffi.new("bfm_vec_t*")
    assert not lib.bfm_vec_create(x, state, n)
    ffi.memmove(x.data, b.tobytes(), b.nbytes)
    assert not lib.bfm_matrix_solve(M, x)
    sol = np.frombuffer(ffi.buffer(x.data, 8 * n), np.float64)
    assert np.allclose(sol, np.linalg.solve(A, b), rtol=1e-12, atol=0)
