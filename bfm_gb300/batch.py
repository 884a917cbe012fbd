"""Batches of independent meshes for the persistent batched solver.

`Batch(lib, problems)` concatenates meshgen.Problem instances into one
block-diagonal device problem: node and element ids are offset per mesh,
Young's modulus and Poisson's ratio become per-element arrays, clamped
sides become two Dirichlet conditions over all meshes, and every mesh's
Neumann traction becomes per-edge loads (each mesh may have its own
magnitude).  `solve()` runs bfm_gpu_problem_solve_parts: one persistent
cooperative kernel, one CG per mesh.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import MIXED_EXACT, bfm_gpu_opts_t, bfm_gpu_stats_t, default_opts, last_error
from . import meshgen as M


class Batch:
    def __init__(self, lib, problems, stream=None):
        self.lib = lib
        self.problems = problems
        kinds = {p.kind for p in problems}
        if len(kinds) != 1:
            raise ValueError("a batch holds meshes of one element kind")
        self.kind = kinds.pop()
        node_off = np.cumsum([0] + [p.n_nodes for p in problems]).astype(np.int32)
        self.node_off = node_off
        coords = np.concatenate([p.coords for p in problems])
        elems = np.concatenate([p.elems + node_off[k] for k, p in enumerate(problems)]).astype(np.int32)
        eE = np.concatenate([p.elem_E if p.elem_E is not None else np.full(p.n_elems, p.E) for p in problems])
        enu = np.concatenate([p.elem_nu if p.elem_nu is not None else np.full(p.n_elems, p.nu) for p in problems])
        dx = np.concatenate([self._mask(p, M.DIRICHLET_X) for p in problems]).astype(np.uint8)
        dy = np.concatenate([self._mask(p, M.DIRICHLET_Y) for p in problems]).astype(np.uint8)
        loads = [M.neumann_edge_loads(p, node_off[k]) for k, p in enumerate(problems)]
        ledges = np.concatenate([e for e, _ in loads]).astype(np.int32)
        lloads = np.concatenate([l for _, l in loads])
        self.n_nodes = int(node_off[-1])
        self.n_elems = len(elems)
        self.keep = [coords, elems, eE, enu, dx, dy, ledges, lloads, node_off]
        P = C.c_void_p()
        rc = lib.bfm_gpu_problem_create(C.byref(P), self.kind, self.n_nodes, self.n_elems, 0, 2, stream)
        assert rc == 0, last_error()
        self.P = P
        w, ph, dxi, deta = M.gauss_tables(self.kind)
        self.keep += [w, ph, dxi, deta]
        masks = np.concatenate([dx, dy])
        self.keep.append(masks)
        kinds = np.array([M.DIRICHLET_X, M.DIRICHLET_Y], np.int32)
        vals = np.zeros(2)
        self.keep += [kinds, vals]
        p0 = problems[0]
        ok = lib.bfm_gpu_problem_set_geometry(P, coords.ctypes.data, elems.ctypes.data, 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_material(P, p0.E, p0.nu, p0.rho, int(p0.stress), eE.ctypes.data,
                                                     enu.ctypes.data, 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_rule(P, len(w), w.ctypes.data, ph.ctypes.data, dxi.ctypes.data,
                                                 deta.ctypes.data) == 0
        ok = ok and lib.bfm_gpu_problem_set_forces(P, 0, None, None, 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_conditions(P, 2, kinds.ctypes.data, vals.ctypes.data, masks.ctypes.data,
                                                       0, None, 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_edge_loads(P, len(ledges), ledges.ctypes.data, lloads.ctypes.data, 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_parts(P, len(problems), node_off.ctypes.data) == 0
        assert ok, last_error()

    @staticmethod
    def _mask(p, kind):
        m = np.zeros(p.n_nodes, bool)
        for k, v, mask in p.conds:
            if k == kind:
                if v != 0.0:
                    raise ValueError("batched Dirichlet conditions must be homogeneous")
                m |= mask
        return m

    def assemble(self, precision=MIXED_EXACT):
        assert self.lib.bfm_gpu_problem_assemble(self.P, precision) == 0, last_error()

    def solve(self, opts: bfm_gpu_opts_t | None = None):
        o = opts or default_opts(rtol=1e-8)
        assert self.lib.bfm_gpu_problem_solve_parts(self.P, C.byref(o)) == 0, last_error()

    def step(self, precision=MIXED_EXACT, opts: bfm_gpu_opts_t | None = None):
        """Assembly + solve as one CUDA graph launch (bfm_gpu_problem_step_parts)."""
        o = opts or default_opts(rtol=1e-8)
        assert self.lib.bfm_gpu_problem_step_parts(self.P, precision, C.byref(o)) == 0, last_error()

    def stats(self):
        n = len(self.problems)
        it = np.zeros(n, np.int32)
        st = np.zeros(n, np.int32)
        rp = np.zeros(n, np.int32)
        res = np.zeros(n)
        rpt, lpr, ms = C.c_int(), C.c_int(), C.c_double()
        assert self.lib.bfm_gpu_problem_part_stats(self.P, it.ctypes.data, st.ctypes.data, rp.ctypes.data,
                                                   res.ctypes.data, C.byref(rpt), C.byref(lpr), C.byref(ms)) == 0, \
            last_error()
        return dict(iterations=it, status=st, replacements=rp, rel_residual=res, rows_per_tile=rpt.value,
                    lanes_per_row=lpr.value, ms_solve=ms.value)

    def coarse(self):
        """Per part, A_c^-1 of the two-level block Jacobi preconditioner (FP32)
        after a solve with it."""
        n = len(self.problems)
        nc = np.zeros(n, np.int32)
        off = np.zeros(n + 1, np.int64)
        assert self.lib.bfm_gpu_problem_parts_coarse(self.P, nc.ctypes.data, off.ctypes.data, None) == 0, last_error()
        a = np.zeros(max(int(off[-1]), 1), np.float32)
        assert self.lib.bfm_gpu_problem_parts_coarse(self.P, None, None, a.ctypes.data) == 0, last_error()
        return [a[off[k]:off[k] + nc[k] * nc[k]].reshape(nc[k], nc[k]) for k in range(n)]

    def assemble_stats(self):
        s = bfm_gpu_stats_t()
        assert self.lib.bfm_gpu_problem_stats(self.P, C.byref(s)) == 0
        return s

    def solutions(self):
        x = np.zeros(2 * self.n_nodes)
        assert self.lib.bfm_gpu_problem_solution(self.P, x.ctypes.data, 0) == 0
        return [x[2 * self.node_off[k]:2 * self.node_off[k + 1]] for k in range(len(self.problems))]

    def close(self):
        if self.P:
            self.lib.bfm_gpu_problem_destroy(self.P)
            self.P = None
