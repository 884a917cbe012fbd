"""ctypes driver for the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the shipped library never does.

  liborc.so            CPU restatement of the reference path (bfm_oracle.c):
                       dense assembly + conditions, RCM, band LU; CSR assembly
  _ref/libbfm_ref.so   the reference libbfm compiled from its sources (only
                       where the reference tree exists; never on the GPU machine)

Parity pin: bfm_oracle.c reproduces the reference's golden U/V files and the
live reference's effects, stiffness matrix and RCM permutation, checked by
tests/test_oracle.py against tests/golden/*.npz (made by
tests/golden/make_golden.py from the reference build).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORC = HERE / "liborc.so"
REF = HERE / "_ref" / "libbfm_ref.so"
# the reference source tree: BFM_REFERENCE, else a "reference" folder beside the repository
REF_TREE = Path(os.environ.get("BFM_REFERENCE", HERE.parent.parent / "reference"))

_dp = C.POINTER(C.c_double)
_lp = C.POINTER(C.c_int64)


class orc_problem_t(C.Structure):
    _fields_ = [("kind", C.c_int), ("stress", C.c_int), ("n_nodes", C.c_int64), ("n_elems", C.c_int64),
                ("coords", _dp), ("elems", _lp), ("E", C.c_double), ("nu", C.c_double), ("rho", C.c_double),
                ("elem_E", _dp), ("elem_nu", _dp), ("n_points", C.c_int), ("weights", _dp), ("phi", _dp),
                ("dxi", _dp), ("deta", _dp), ("n_forces", C.c_int), ("forces", _dp), ("n_conds", C.c_int),
                ("cond_kind", C.POINTER(C.c_int)), ("cond_value", _dp), ("cond_nodes", C.POINTER(C.c_uint8)),
                ("n_edges", C.c_int64), ("edges", _lp), ("edge_boundary", C.POINTER(C.c_uint8))]


def build(ref: bool = False) -> None:
    """Compile liborc.so (and the reference, when its sources are present)."""
    import shutil
    targets = ["all"] + (["ref"] if ref and REF_TREE.exists() else [])
    if shutil.which("make"):
        subprocess.run(["make", "-s", "-C", str(HERE), f"REF={REF_TREE}", *targets], check=True)
        return
    # no make: the same recipe as oracle/Makefile's liborc.so target
    subprocess.run(["gcc", "-O2", "-fPIC", "-ffp-contract=off", "-std=gnu11", "-shared", "-o", str(ORC),
                    str(HERE / "bfm_oracle.c"), "-lm"], check=True)


_orc: C.CDLL | None = None


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        if not ORC.exists() or ORC.stat().st_mtime < (HERE / "bfm_oracle.c").stat().st_mtime:
            build()
        L = C.CDLL(str(ORC))
        L.orc_gauss_tables.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        L.orc_assemble_dense.argtypes = [C.POINTER(orc_problem_t), _dp, _dp]
        L.orc_rcm_dense.argtypes = [C.c_int64, _dp, _lp, _lp]
        L.orc_rcm_csr.argtypes = [C.c_int64, _lp, _lp, _dp, _lp, _lp]
        L.orc_solve_reference.argtypes = [C.POINTER(orc_problem_t), _dp, _lp, _lp]
        L.orc_assemble_csr.argtypes = [C.POINTER(orc_problem_t), _lp, _lp, _dp, _dp]
        L.orc_assemble_csr.restype = C.c_int64
        _orc = L
    return _orc


def ref_lib():
    """The reference library built from source, or None where it cannot be."""
    if not REF.exists():
        if not REF_TREE.exists():
            return None
        build(ref=True)
    from bfm_gb300 import abi
    return abi.bind(C.CDLL(str(REF)))


class _Prob:
    """orc_problem_t for a meshgen.Problem, with its arrays kept alive."""

    def __init__(self, p):
        self.keep = []
        s = orc_problem_t()
        s.kind, s.stress = p.kind, int(p.stress)
        s.n_nodes, s.n_elems = p.n_nodes, p.n_elems
        s.coords = self._a(p.coords, np.float64)
        s.elems = self._a(p.elems, np.int64)
        s.E, s.nu, s.rho = p.E, p.nu, p.rho
        s.elem_E = self._a(p.elem_E, np.float64) if p.elem_E is not None else None
        s.elem_nu = self._a(p.elem_nu, np.float64) if p.elem_nu is not None else None
        nq = p.kind
        w, ph, dx, de = (np.zeros(nq * k) for k in (1, p.kind, p.kind, p.kind))
        orc().orc_gauss_tables(p.kind, self._a(w), self._a(ph), self._a(dx), self._a(de))
        s.n_points = nq
        s.weights, s.phi, s.dxi, s.deta = (self._a(v) for v in (w, ph, dx, de))
        s.n_forces = len(p.forces)
        s.forces = self._a(np.array(p.forces, dtype=np.float64).reshape(-1)) if p.forces else None
        s.n_conds = len(p.conds)
        if p.conds:
            s.cond_kind = self._a(np.array([c[0] for c in p.conds], dtype=np.int32), np.int32, C.c_int)
            s.cond_value = self._a(np.array([c[1] for c in p.conds], dtype=np.float64))
            masks = np.stack([np.asarray(c[2], dtype=np.uint8) for c in p.conds])
            s.cond_nodes = self._a(masks, np.uint8, C.c_uint8)
        if p.edges is not None:
            s.n_edges = len(p.edges)
            s.edges = self._a(p.edges, np.int64)
            if getattr(p, "edge_boundary", None) is not None:
                s.edge_boundary = self._a(np.asarray(p.edge_boundary, np.uint8), np.uint8, C.c_uint8)
        self.s = s

    def _a(self, arr, dtype=np.float64, ctype=None):
        a = np.ascontiguousarray(arr, dtype=dtype)
        self.keep.append(a)
        ct = ctype or {np.float64: C.c_double, np.int64: C.c_int64}[np.dtype(dtype).type]
        return a.ctypes.data_as(C.POINTER(ct))


def assemble_dense(p):
    """Dense K (n x n) and b after conditions, exactly as the reference."""
    n = p.n_dof
    K = np.zeros((n, n))
    b = np.zeros(n)
    pr = _Prob(p)
    rc = orc().orc_assemble_dense(C.byref(pr.s), K.ctypes.data_as(_dp), b.ctypes.data_as(_dp))
    assert rc == 0
    return K, b


def rcm_dense(K: np.ndarray):
    n = K.shape[0]
    K = np.ascontiguousarray(K, dtype=np.float64)
    perm = np.zeros(n, np.int64)
    inv = np.zeros(n, np.int64)
    assert orc().orc_rcm_dense(n, K.ctypes.data_as(_dp), perm.ctypes.data_as(_lp), inv.ctypes.data_as(_lp)) == 0
    return perm, inv


def solve_reference(p):
    """The reference pipeline restated: effects (2N), RCM perm, bandwidth."""
    n = p.n_dof
    eff = np.zeros(n)
    perm = np.zeros(n, np.int64)
    bw = C.c_int64(0)
    pr = _Prob(p)
    assert orc().orc_solve_reference(C.byref(pr.s), eff.ctypes.data_as(_dp), perm.ctypes.data_as(_lp),
                                     C.byref(bw)) == 0
    return eff, perm, bw.value


def assemble_csr(p):
    """Scalar CSR K (scipy) and b, values bit-identical to the dense restatement."""
    import scipy.sparse as sp
    pr = _Prob(p)
    L = orc()
    nnz = L.orc_assemble_csr(C.byref(pr.s), None, None, None, None)
    n = p.n_dof
    rp = np.zeros(n + 1, np.int64)
    cols = np.zeros(nnz, np.int64)
    vals = np.zeros(nnz)
    b = np.zeros(n)
    got = L.orc_assemble_csr(C.byref(pr.s), rp.ctypes.data_as(_lp), cols.ctypes.data_as(_lp),
                             vals.ctypes.data_as(_dp), b.ctypes.data_as(_dp))
    assert got == nnz
    return sp.csr_matrix((vals, cols, rp), shape=(n, n)), b


def solve_direct(p):
    """FP64 direct solve (SuperLU) of the restated CSR system."""
    import scipy.sparse.linalg as spla
    K, b = assemble_csr(p)
    return spla.spsolve(K.tocsc(), b), K, b


def rcm_csr(K):
    """Bit-exact reference RCM on a scipy CSR matrix (sorted indices)."""
    K = K.tocsr()
    K.sort_indices()
    n = K.shape[0]
    rp = np.ascontiguousarray(K.indptr, dtype=np.int64)
    ci = np.ascontiguousarray(K.indices, dtype=np.int64)
    v = np.ascontiguousarray(K.data, dtype=np.float64)
    perm = np.zeros(n, np.int64)
    inv = np.zeros(n, np.int64)
    assert orc().orc_rcm_csr(n, rp.ctypes.data_as(_lp), ci.ctypes.data_as(_lp), v.ctypes.data_as(_dp),
                             perm.ctypes.data_as(_lp), inv.ctypes.data_as(_lp)) == 0
    return perm, inv
