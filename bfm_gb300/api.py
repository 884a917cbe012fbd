"""Python front end over the libbfm C API, mirroring the reference's pybfm
classes (pybfm/bfm/{mesh,condition,force,material,rule,obj,instance,sim,ez}.py)
without their OpenGL parts, so it runs headless.

Two layers:
  * `SimHandle.from_problem(lib, problem)` builds the libbfm structures for a
    synthetic `meshgen.Problem` through the public API (the way a C caller
    does: bfm_mesh_create + fields, material, rule, obj, instance,
    conditions, forces, sim).  It works with any library exporting the
    libbfm ABI, which is how tests drive this library and the reference
    build side by side.
  * Mesh_lepl1110 / Ez_lepl1110 / Sim / ... with pybfm's names and call
    pattern; every C call is checked with `assert not ...`, as pybfm does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from . import lib as _gpu_lib


def _ptr(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class SimHandle:
    """libbfm structures for one Problem; keeps every buffer alive."""

    def __init__(self, lib: C.CDLL, kind_sim: int):
        self.lib = lib
        self.keep: list = []
        self.state = abi.bfm_state_t()
        assert not lib.bfm_state_create(C.byref(self.state))
        self.sim = abi.bfm_sim_t()
        assert not lib.bfm_sim_create(C.byref(self.sim), C.byref(self.state), kind_sim)
        self.instances: list[abi.bfm_instance_t] = []
        self.meshes: list[abi.bfm_mesh_t] = []

    @classmethod
    def from_problem(cls, lib: C.CDLL, problem, elem_material: bool = True) -> "SimHandle":
        st = int(problem.stress)
        h = cls(lib, abi.SIM_AXISYMMETRIC_STRAIN if st >= 2 else abi.SIM_PLANAR_STRESS if st else abi.SIM_PLANAR_STRAIN)
        h.add_problem(problem, elem_material=elem_material)
        return h

    def add_problem(self, p, elem_material: bool = True) -> abi.bfm_instance_t:
        lib, st = self.lib, C.byref(self.state)
        mesh = abi.bfm_mesh_t()
        assert not lib.bfm_mesh_create(C.byref(mesh), st, 2, p.kind)
        coords = np.ascontiguousarray(p.coords, dtype=np.float64).ravel()
        elems = np.ascontiguousarray(p.elems, dtype=np.uint64).ravel()
        mesh.n_nodes = p.n_nodes
        mesh.n_elems = p.n_elems
        mesh.coords = _ptr(coords, C.c_double)
        mesh.elems = _ptr(elems, C.c_size_t)
        self.keep += [coords, elems]
        if p.edges is not None:
            edges = (abi.bfm_edge_t * len(p.edges))()
            eb = getattr(p, "edge_boundary", None)
            for i, (a, b) in enumerate(p.edges):
                edges[i].nodes[0] = int(a)
                edges[i].nodes[1] = int(b)
                edges[i].elems[0] = -1
                # elems[1] == -1 marks a boundary edge (one adjacent element); interior
                # edges get a placeholder id, which only that test reads
                edges[i].elems[1] = -1 if eb is None or eb[i] else 0
            mesh.n_edges = len(p.edges)
            mesh.edges = C.cast(edges, C.POINTER(abi.bfm_edge_t))
            self.keep.append(edges)
        material = abi.bfm_material_t()
        assert not lib.bfm_material_create(C.byref(material), st, b"material", p.rho, p.E, p.nu)
        rule = abi.bfm_rule_t()
        assert not lib.bfm_rule_create_gauss_legendre(C.byref(rule), st, 2, p.kind)
        obj = abi.bfm_obj_t()
        assert not lib.bfm_obj_create(C.byref(obj), st, C.byref(mesh), C.byref(material), C.byref(rule))
        inst = abi.bfm_instance_t()
        assert not lib.bfm_instance_create(C.byref(inst), st, C.byref(obj))
        for kind, value, mask in p.conds:
            cond = abi.bfm_condition_t()
            assert not lib.bfm_condition_create(C.byref(cond), st, C.byref(mesh), kind)
            cond.value = float(value)
            m = np.ascontiguousarray(mask, dtype=np.bool_)
            C.memmove(cond.nodes, m.ctypes.data, m.nbytes)
            assert not lib.bfm_instance_add_condition(C.byref(inst), C.byref(cond))
            self.keep.append(cond)
        if not self.instances:  # forces are per simulation
            for fx, fy in p.forces:
                force = abi.bfm_force_t()
                vec = abi.bfm_vec_t()
                assert not lib.bfm_force_create(C.byref(force), st, 2)
                assert not lib.bfm_vec_create(C.byref(vec), st, 2)
                vec.data[0], vec.data[1] = fx, fy
                assert not lib.bfm_force_set_linear(C.byref(force), C.byref(vec))
                assert not lib.bfm_sim_add_force(C.byref(self.sim), C.byref(force))
                self.keep += [force, vec]
        if elem_material and (p.elem_E is not None or p.elem_nu is not None):
            eE = None if p.elem_E is None else np.ascontiguousarray(p.elem_E, dtype=np.float64)
            enu = None if p.elem_nu is None else np.ascontiguousarray(p.elem_nu, dtype=np.float64)
            self.keep += [eE, enu]
            assert not lib.bfm_gpu_instance_set_elem_material(
                C.byref(inst), None if eE is None else eE.ctypes.data, None if enu is None else enu.ctypes.data)
        assert not lib.bfm_sim_add_instance(C.byref(self.sim), C.byref(inst))
        self.keep += [mesh, material, rule, obj]
        self.meshes.append(mesh)
        self.instances.append(inst)
        return inst

    def run(self) -> int:
        return self.lib.bfm_sim_run(C.byref(self.sim))

    def effects(self, i: int = 0) -> np.ndarray:
        inst = self.instances[i]
        return np.ctypeslib.as_array(inst.effects, shape=(inst.n_effects,)).copy()

    def error(self) -> str:
        e = self.state.err
        return (e.msg or b"").decode() if e.has else ""

    def system(self, i: int = 0, renumber: bool = False):
        """Dense K, b from bfm_system_create_{planar_*,axisymmetric_strain} (and
        the RCM permutation)."""
        lib = self.lib
        s = abi.bfm_system_t()
        create = {abi.SIM_PLANAR_STRESS: lib.bfm_system_create_planar_stress,
                  abi.SIM_AXISYMMETRIC_STRAIN: lib.bfm_system_create_axisymmetric_strain}.get(
                      self.sim.kind, lib.bfm_system_create_planar_strain)
        rc = create(C.byref(s), C.byref(self.instances[i]), self.sim.n_forces, self.sim.forces)
        assert rc == 0, self.error()
        n = s.n
        K = np.ctypeslib.as_array(s.A.full.data, shape=(n * n,)).reshape(n, n).copy()
        b = np.ctypeslib.as_array(s.b.data, shape=(n,)).copy()
        perm = None
        if renumber:
            assert not lib.bfm_system_renumber(C.byref(s))
            perm = np.ctypeslib.as_array(s.perm.perm, shape=(n,)).astype(np.int64).copy()
        lib.bfm_system_destroy(C.byref(s))
        return K, b, perm


class DeviceProblem:
    """A meshgen.Problem uploaded once through the device-resident problem API
    (bfm_gpu_problem_*): assemble and solve repeatedly without re-uploading,
    and read back the solution and the assembled system."""

    def __init__(self, lib: C.CDLL, p, stream=None):
        from . import meshgen as M
        from . import last_error
        self.lib, self.p = lib, p
        self.keep: list = []
        P = C.c_void_p()
        n_edges = 0 if p.edges is None else len(p.edges)
        rc = lib.bfm_gpu_problem_create(C.byref(P), p.kind, p.n_nodes, p.n_elems, n_edges, len(p.conds), stream)
        assert rc == 0, last_error()
        self.P = P
        a = self._a
        ok = lib.bfm_gpu_problem_set_geometry(P, a(p.coords, np.float64), a(p.elems, np.int32), 0) == 0
        ok = ok and lib.bfm_gpu_problem_set_material(
            P, p.E, p.nu, p.rho, int(p.stress), None if p.elem_E is None else a(p.elem_E, np.float64),
            None if p.elem_nu is None else a(p.elem_nu, np.float64), 0) == 0
        w, ph, dx, de = M.gauss_tables(p.kind)
        ok = ok and lib.bfm_gpu_problem_set_rule(P, len(w), a(w, np.float64), a(ph, np.float64), a(dx, np.float64),
                                                 a(de, np.float64)) == 0
        f = np.array(p.forces, np.float64).reshape(-1)
        ok = ok and lib.bfm_gpu_problem_set_forces(P, len(p.forces), a(f, np.float64) if len(f) else None, None, 0) == 0
        if p.conds:
            kinds = a([c[0] for c in p.conds], np.int32)
            vals = a([c[1] for c in p.conds], np.float64)
            masks = a(np.stack([c[2] for c in p.conds]).astype(np.uint8), np.uint8)
            edges = a(p.edges, np.int32) if n_edges else None
            ok = ok and lib.bfm_gpu_problem_set_conditions(P, len(p.conds), kinds, vals, masks, n_edges, edges, 0) == 0
        assert ok, last_error()

    def _a(self, x, dt):
        x = np.ascontiguousarray(x, dtype=dt)
        self.keep.append(x)
        return x.ctypes.data

    def assemble(self, precision: int) -> None:
        from . import last_error
        assert self.lib.bfm_gpu_problem_assemble(self.P, precision) == 0, last_error()

    def solve(self, opts) -> None:
        from . import last_error
        assert self.lib.bfm_gpu_problem_solve(self.P, C.byref(opts)) == 0, last_error()

    def stats(self):
        from . import bfm_gpu_stats_t, last_error
        s = bfm_gpu_stats_t()
        assert self.lib.bfm_gpu_problem_stats(self.P, C.byref(s)) == 0, last_error()
        return s

    def solution(self) -> np.ndarray:
        x = np.zeros(self.p.n_dof)
        assert self.lib.bfm_gpu_problem_solution(self.P, x.ctypes.data, 0) == 0
        return x

    def system(self):
        """The assembled system in the working node order: (row_ptr, cols,
        vals (4 per block, FP64), b) and the order's perm (perm[w] = caller node)."""
        nb = C.c_int64()
        assert self.lib.bfm_gpu_problem_n_blocks(self.P, C.byref(nb)) == 0
        n = self.p.n_nodes
        rp = np.zeros(n + 1, np.int32)
        cols = np.zeros(nb.value, np.int32)
        vals = np.zeros(4 * nb.value)
        b = np.zeros(2 * n)
        assert self.lib.bfm_gpu_problem_download(self.P, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data,
                                                 b.ctypes.data) == 0
        perm = np.zeros(n, np.int32)
        assert self.lib.bfm_gpu_problem_ordering(self.P, perm.ctypes.data, None, None) == 0
        return rp, cols, vals, b, perm

    def close(self) -> None:
        if self.P:
            self.lib.bfm_gpu_problem_destroy(self.P)
            self.P = None


def scalar_csr(rp, cols, vals, n_nodes: int, perm=None):
    """A 2x2-block CSR system as a scipy scalar CSR matrix (the caller's node
    order when perm, perm[w] = caller node, is given)."""
    import scipy.sparse as sp
    nb = len(cols)
    brow = np.repeat(np.arange(n_nodes), np.diff(rp))
    if perm is not None:
        brow = perm[brow]
        bcol = perm[cols]
    else:
        bcol = cols
    r = (2 * brow)[:, None] + np.array([0, 0, 1, 1])[None, :]
    c = (2 * bcol)[:, None] + np.array([0, 1, 0, 1])[None, :]
    K = sp.csr_matrix((vals.reshape(nb, 4).ravel(), (r.ravel(), c.ravel())), shape=(2 * n_nodes, 2 * n_nodes))
    K.sort_indices()
    return K


# --------------------------------------------------------------------- pybfm-style classes

class _State:
    def __init__(self):
        self.lib = _gpu_lib()
        self.state = abi.bfm_state_t()
        assert not self.lib.bfm_state_create(C.byref(self.state))


_default: _State | None = None


def default_state() -> _State:
    global _default
    if _default is None:
        _default = _State()
    return _default


class Mesh:
    SIMPLEX = 3
    QUAD = 4

    def __init__(self, dim: int, kind: int):
        s = default_state()
        self.c_mesh = abi.bfm_mesh_t()
        assert not s.lib.bfm_mesh_create(C.byref(self.c_mesh), C.byref(s.state), dim, kind)
        self.dim, self.kind = dim, kind

    @property
    def coords(self):
        return [self.c_mesh.coords[i] for i in range(self.c_mesh.n_nodes * self.dim)]


class Mesh_lepl1110(Mesh):
    def __init__(self, name: str):
        s = default_state()
        self.c_mesh = abi.bfm_mesh_t()
        assert not s.lib.bfm_mesh_read_lepl1110(C.byref(self.c_mesh), C.byref(s.state), name.encode())
        self.dim, self.kind = self.c_mesh.dim, self.c_mesh.kind

    def __del__(self):
        try:
            default_state().lib.bfm_mesh_destroy(C.byref(self.c_mesh))
        except Exception:
            pass


class Mesh_wavefront(Mesh):
    def __init__(self, name: str, full: bool = False):
        s = default_state()
        self.c_mesh = abi.bfm_mesh_t()
        assert not s.lib.bfm_mesh_read_wavefront(C.byref(self.c_mesh), C.byref(s.state), name.encode(), full)
        self.dim, self.kind = self.c_mesh.dim, self.c_mesh.kind


class CSim:
    NONE, PLANAR_STRAIN, PLANAR_STRESS, AXISYMMETRIC_STRAIN = 0, 1, 2, 3

    def __init__(self, c_sim):
        self.c_sim = c_sim

    def run(self):
        s = default_state()
        rc = s.lib.bfm_sim_run(self.c_sim)
        assert not rc, (s.state.err.msg or b"").decode()


class Ez_lepl1110:
    """pybfm/bfm/ez.py: parse a LEPL1110 problem file for a mesh."""

    def __init__(self, mesh: Mesh, name: str):
        s = default_state()
        self.mesh = mesh
        self.c_ez = abi.bfm_ez_lepl1110_t()
        assert not s.lib.bfm_ez_lepl1110_create(C.byref(self.c_ez), C.byref(s.state), C.byref(mesh.c_mesh),
                                                name.encode())
        self.sim = CSim(C.pointer(self.c_ez.sim))

    def write(self, filename: str, shift: int):
        assert not default_state().lib.bfm_ez_lepl1110_write(C.byref(self.c_ez), shift, filename.encode())

    @property
    def effects(self) -> np.ndarray:
        inst = self.c_ez.instance
        return np.ctypeslib.as_array(inst.effects, shape=(inst.n_effects,)).copy()

    def __del__(self):
        try:
            default_state().lib.bfm_ez_lepl1110_destroy(C.byref(self.c_ez))
        except Exception:
            pass
