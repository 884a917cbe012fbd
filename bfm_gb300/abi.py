"""ctypes mirror of the libbfm C ABI.

The structures below have the field order and types of the public libbfm
headers (libbfm/src/bfm/*.h in the reference; include/bfm/*.h here), so one
set of definitions drives either shared object: this package's GPU-backed
``libbfm.so`` or, in tests, the reference library built from source.

cffi is the reference's own binding route (pybfm/bfm/gen_libbfm.py); ctypes is
used here because it needs no compiler at import time.
"""
from __future__ import annotations

import ctypes as C

c_size_t = C.c_size_t
c_ssize_t = C.c_ssize_t
c_double_p = C.POINTER(C.c_double)
c_size_p = C.POINTER(C.c_size_t)


class bfm_err_t(C.Structure):  # bfm.h:6-13
    _fields_ = [("has", C.c_bool), ("msg", C.c_char_p), ("file", C.c_char_p),
                ("func", C.c_char_p), ("line", c_size_t)]


class bfm_state_t(C.Structure):  # bfm.h:19-25
    _fields_ = [("err", bfm_err_t), ("alloc", C.c_void_p), ("realloc", C.c_void_p),
                ("free", C.c_void_p)]


P_state = C.POINTER(bfm_state_t)


class bfm_vec_t(C.Structure):  # math.h:14-19
    _fields_ = [("state", P_state), ("n", c_size_t), ("data", c_double_p)]


class bfm_edge_t(C.Structure):  # mesh.h:17-23
    _fields_ = [("nodes", c_size_t * 2), ("elems", c_ssize_t * 2)]


class bfm_domain_t(C.Structure):  # mesh.h:25-29
    _fields_ = [("name", C.c_char * 50), ("n_elements", c_size_t), ("elements", c_size_p)]


class bfm_mesh_t(C.Structure):  # mesh.h:31-48
    _fields_ = [("state", P_state), ("dim", c_size_t), ("kind", C.c_int),
                ("n_elems", c_size_t), ("n_nodes", c_size_t), ("n_edges", c_size_t),
                ("coords", c_double_p), ("elems", c_size_p), ("edges", C.POINTER(bfm_edge_t)),
                ("n_domains", c_size_t), ("domains", C.POINTER(bfm_domain_t))]


class bfm_colour_t(C.Structure):  # material.h:5-10
    _fields_ = [("r", C.c_double), ("g", C.c_double), ("b", C.c_double), ("a", C.c_double)]


class bfm_material_t(C.Structure):  # material.h:12-21
    _fields_ = [("state", P_state), ("name", C.c_char_p), ("colour", bfm_colour_t),
                ("rho", C.c_double), ("E", C.c_double), ("nu", C.c_double)]


class bfm_shape_t(C.Structure):  # shape.h:13-21
    _fields_ = [("state", P_state), ("dim", c_size_t), ("kind", C.c_int),
                ("phi", C.c_void_p), ("dphi", C.c_void_p)]


class bfm_rule_t(C.Structure):  # rule.h:6-17
    _fields_ = [("state", P_state), ("dim", c_size_t), ("kind", C.c_int), ("n_points", c_size_t),
                ("weights", c_double_p), ("points", C.POINTER(c_double_p)), ("shape", bfm_shape_t)]


class bfm_force_linear_t(C.Structure):  # force.h:12-14
    _fields_ = [("force", bfm_vec_t)]


class bfm_force_funky_t(C.Structure):  # force.h:20-23
    _fields_ = [("func", C.c_void_p), ("data", C.c_void_p)]


class _force_u(C.Union):
    _fields_ = [("linear", bfm_force_linear_t), ("funky", bfm_force_funky_t)]


class bfm_force_t(C.Structure):  # force.h:25-34
    _anonymous_ = ("u",)
    _fields_ = [("state", P_state), ("kind", C.c_int), ("dim", c_size_t), ("u", _force_u)]


class bfm_condition_t(C.Structure):  # condition.h:16-27
    _fields_ = [("state", P_state), ("mesh", C.POINTER(bfm_mesh_t)), ("kind", C.c_int),
                ("value", C.c_double), ("nodes", C.POINTER(C.c_bool))]


class bfm_obj_t(C.Structure):  # obj.h:8-14
    _fields_ = [("state", P_state), ("mesh", C.POINTER(bfm_mesh_t)),
                ("material", C.POINTER(bfm_material_t)), ("rule", C.POINTER(bfm_rule_t))]


class bfm_instance_t(C.Structure):  # instance.h:6-17
    _fields_ = [("state", P_state), ("obj", C.POINTER(bfm_obj_t)), ("n_effects", c_size_t),
                ("effects", c_double_p), ("n_conditions", c_size_t),
                ("conditions", C.POINTER(C.POINTER(bfm_condition_t)))]


class bfm_sim_t(C.Structure):  # sim.h:13-22
    _fields_ = [("state", P_state), ("kind", C.c_int), ("n_instances", c_size_t),
                ("instances", C.POINTER(C.POINTER(bfm_instance_t))), ("n_forces", c_size_t),
                ("forces", C.POINTER(C.POINTER(bfm_force_t)))]


class bfm_matrix_full_t(C.Structure):  # matrix.h:20-22
    _fields_ = [("data", c_double_p)]


class bfm_matrix_band_t(C.Structure):  # matrix.h:24-27
    _fields_ = [("k", c_size_t), ("data", c_double_p)]


class bfm_matrix_sparse_t(C.Structure):  # matrix.h (additive kind)
    _fields_ = [("handle", C.c_void_p), ("nnz", c_size_t)]


class _matrix_u(C.Union):
    _fields_ = [("full", bfm_matrix_full_t), ("band", bfm_matrix_band_t), ("sparse", bfm_matrix_sparse_t)]


class bfm_matrix_t(C.Structure):  # matrix.h:29-43
    _anonymous_ = ("u",)
    _fields_ = [("state", P_state), ("kind", C.c_int), ("major", C.c_int), ("m", c_size_t),
                ("u", _matrix_u)]


class bfm_perm_t(C.Structure):  # perm.h:6-14
    _fields_ = [("state", P_state), ("m", c_size_t), ("has_perm", C.c_bool),
                ("perm", c_size_p), ("inv_perm", c_size_p)]


class bfm_system_t(C.Structure):  # system.h:9-17
    _fields_ = [("state", P_state), ("n", c_size_t), ("perm", bfm_perm_t), ("A", bfm_matrix_t),
                ("b", bfm_vec_t)]


class bfm_ez_lepl1110_t(C.Structure):  # ez.h:11-24
    _fields_ = [("state", P_state), ("mesh", C.POINTER(bfm_mesh_t)), ("n_conditions", c_size_t),
                ("conditions", C.POINTER(bfm_condition_t)), ("gravity", bfm_force_t),
                ("material", bfm_material_t), ("rule", bfm_rule_t), ("obj", bfm_obj_t),
                ("instance", bfm_instance_t), ("sim", bfm_sim_t)]


P = C.POINTER
_I = C.c_int

# name -> (restype, argtypes); every prototype of the public headers
PROTOTYPES = {
    "bfm_state_create": (_I, [P_state]),
    "bfm_state_destroy": (_I, [P_state]),
    "bfm_set_alloc": (_I, [P_state, C.c_void_p]),
    "bfm_set_realloc": (_I, [P_state, C.c_void_p]),
    "bfm_set_free": (_I, [P_state, C.c_void_p]),
    "bfm_err_print": (_I, [P_state]),
    "bfm_vec_create": (_I, [P(bfm_vec_t), P_state, c_size_t]),
    "bfm_vec_copy": (_I, [P(bfm_vec_t), P(bfm_vec_t)]),
    "bfm_vec_destroy": (_I, [P(bfm_vec_t)]),
    "bfm_force_create": (_I, [P(bfm_force_t), P_state, c_size_t]),
    "bfm_force_destroy": (_I, [P(bfm_force_t)]),
    "bfm_force_set_none": (_I, [P(bfm_force_t)]),
    "bfm_force_set_linear": (_I, [P(bfm_force_t), P(bfm_vec_t)]),
    "bfm_force_set_funky": (_I, [P(bfm_force_t), C.c_void_p, C.c_void_p]),
    "bfm_force_eval": (_I, [P(bfm_force_t), P(bfm_vec_t), P(bfm_vec_t)]),
    "bfm_material_create": (_I, [P(bfm_material_t), P_state, C.c_char_p, C.c_double, C.c_double, C.c_double]),
    "bfm_material_destroy": (_I, [P(bfm_material_t)]),
    "bfm_material_set_colour": (_I, [P(bfm_material_t), C.c_double, C.c_double, C.c_double, C.c_double]),
    "bfm_matrix_full_create": (_I, [P(bfm_matrix_t), P_state, _I, c_size_t]),
    "bfm_matrix_band_create": (_I, [P(bfm_matrix_t), P_state, _I, c_size_t, c_size_t]),
    "bfm_matrix_copy": (_I, [P(bfm_matrix_t), P(bfm_matrix_t)]),
    "bfm_matrix_destroy": (_I, [P(bfm_matrix_t)]),
    "bfm_matrix_get": (C.c_double, [P(bfm_matrix_t), c_size_t, c_size_t]),
    "bfm_matrix_set": (_I, [P(bfm_matrix_t), c_size_t, c_size_t, C.c_double]),
    "bfm_matrix_add": (_I, [P(bfm_matrix_t), c_size_t, c_size_t, C.c_double]),
    "bfm_matrix_bandwidth": (c_size_t, [P(bfm_matrix_t)]),
    "bfm_matrix_lu": (_I, [P(bfm_matrix_t)]),
    "bfm_matrix_lu_solve": (_I, [P(bfm_matrix_t), P(bfm_vec_t)]),
    "bfm_matrix_solve": (_I, [P(bfm_matrix_t), P(bfm_vec_t)]),
    "bfm_mesh_create": (_I, [P(bfm_mesh_t), P_state, c_size_t, _I]),
    "bfm_mesh_destroy": (_I, [P(bfm_mesh_t)]),
    "bfm_mesh_read_lepl1110": (_I, [P(bfm_mesh_t), P_state, C.c_char_p]),
    "bfm_mesh_read_wavefront": (_I, [P(bfm_mesh_t), P_state, C.c_char_p, C.c_bool]),
    "bfm_condition_create": (_I, [P(bfm_condition_t), P_state, P(bfm_mesh_t), _I]),
    "bfm_condition_destroy": (_I, [P(bfm_condition_t)]),
    "bfm_shape_create": (_I, [P(bfm_shape_t), P_state, c_size_t, _I]),
    "bfm_shape_destroy": (_I, [P(bfm_shape_t)]),
    "bfm_rule_create": (_I, [P(bfm_rule_t), P_state, c_size_t, _I, c_size_t]),
    "bfm_rule_destroy": (_I, [P(bfm_rule_t)]),
    "bfm_rule_create_gauss_legendre": (_I, [P(bfm_rule_t), P_state, c_size_t, _I]),
    "bfm_obj_create": (_I, [P(bfm_obj_t), P_state, P(bfm_mesh_t), P(bfm_material_t), P(bfm_rule_t)]),
    "bfm_obj_destroy": (_I, [P(bfm_obj_t)]),
    "bfm_instance_create": (_I, [P(bfm_instance_t), P_state, P(bfm_obj_t)]),
    "bfm_instance_destroy": (_I, [P(bfm_instance_t)]),
    "bfm_instance_set_n_conditions": (_I, [P(bfm_instance_t), c_size_t]),
    "bfm_instance_add_condition": (_I, [P(bfm_instance_t), P(bfm_condition_t)]),
    "bfm_sim_create": (_I, [P(bfm_sim_t), P_state, _I]),
    "bfm_sim_destroy": (_I, [P(bfm_sim_t)]),
    "bfm_sim_set_n_instances": (_I, [P(bfm_sim_t), c_size_t]),
    "bfm_sim_add_instance": (_I, [P(bfm_sim_t), P(bfm_instance_t)]),
    "bfm_sim_set_n_forces": (_I, [P(bfm_sim_t), c_size_t]),
    "bfm_sim_add_force": (_I, [P(bfm_sim_t), P(bfm_force_t)]),
    "bfm_sim_run": (_I, [P(bfm_sim_t)]),
    "bfm_ez_lepl1110_create": (_I, [P(bfm_ez_lepl1110_t), P_state, P(bfm_mesh_t), C.c_char_p]),
    "bfm_ez_lepl1110_destroy": (_I, [P(bfm_ez_lepl1110_t)]),
    "bfm_ez_lepl1110_write": (_I, [P(bfm_ez_lepl1110_t), c_size_t, C.c_char_p]),
    "bfm_perm_create": (_I, [P(bfm_perm_t), P_state, c_size_t]),
    "bfm_perm_destroy": (_I, [P(bfm_perm_t)]),
    "bfm_perm_perm_matrix": (_I, [P(bfm_perm_t), P(bfm_matrix_t), C.c_bool]),
    "bfm_perm_perm_vec": (_I, [P(bfm_perm_t), P(bfm_vec_t), C.c_bool]),
    "bfm_perm_rcm": (_I, [P(bfm_perm_t), P(bfm_matrix_t)]),
    "bfm_system_create": (_I, [P(bfm_system_t), P_state, c_size_t]),
    "bfm_system_destroy": (_I, [P(bfm_system_t)]),
    "bfm_system_renumber": (_I, [P(bfm_system_t)]),
    "bfm_system_create_planar_strain": (_I, [P(bfm_system_t), P(bfm_instance_t), c_size_t, P(P(bfm_force_t))]),
    "bfm_system_create_planar_stress": (_I, [P(bfm_system_t), P(bfm_instance_t), c_size_t, P(P(bfm_force_t))]),
    "bfm_system_create_axisymmetric_strain": (_I, [P(bfm_system_t), P(bfm_instance_t), c_size_t, P(P(bfm_force_t))]),
}

# constants (condition.h:5-14, sim.h:6-11, mesh.h:7-11, force.h:6-10, matrix.h:10-18)
ELEM_SIMPLEX, ELEM_QUAD = 3, 4
SIM_NONE, SIM_PLANAR_STRAIN, SIM_PLANAR_STRESS, SIM_AXISYMMETRIC_STRAIN = 0, 1, 2, 3
DIRICHLET_X, DIRICHLET_Y, NEUMANN_X, NEUMANN_Y = 0, 1, 2, 3
NEUMANN_NORMAL, NEUMANN_TANGENT, DIRICHLET_NORMAL, DIRICHLET_TANGENT = 4, 5, 6, 7
FORCE_NONE, FORCE_LINEAR, FORCE_FUNKY = 0, 1, 2
MATRIX_FULL, MATRIX_BAND, MATRIX_SPARSE = 0, 1, 2
MAJOR_ROW, MAJOR_COLUMN = 0, 1


def bind(lib: C.CDLL, extra: dict | None = None) -> C.CDLL:
    """Declare restype/argtypes for every public prototype found in `lib`."""
    for name, (res, args) in {**PROTOTYPES, **(extra or {})}.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
