"""bfm_gb300: libbfm's FEM hot path on one GB300 (sm_103a).

`lib()` loads the in-tree GPU-backed ``libbfm.so`` (built by
``python -m bfm_gb300.build`` or ``__graft_entry__.build()``).  It exports the
reference's C API unchanged (include/bfm/*.h) plus the additive GPU API of
include/bfm/gpu.h.  There is no CPU fallback: a missing library raises.

`bfm_gb300.api` mirrors the reference's pybfm classes (Mesh_lepl1110,
Ez_lepl1110, Sim, Condition, ...) on top of this library through ctypes.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libbfm.so"

_lib: C.CDLL | None = None


class bfm_gpu_opts_t(C.Structure):  # include/bfm/gpu.h
    _fields_ = [("precision", C.c_int), ("precond", C.c_int), ("rtol", C.c_double), ("max_iters", C.c_int),
                ("replace_drop", C.c_double), ("deterministic", C.c_int), ("autotune", C.c_int),
                ("barrier_polls", C.c_int64), ("refine_restart", C.c_int)]


class bfm_gpu_stats_t(C.Structure):  # include/bfm/gpu.h
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("replacements", C.c_int), ("fallback", C.c_int),
                ("rel_residual", C.c_double), ("n_blocks", C.c_int64), ("n_dof", C.c_int64),
                ("ms_assemble", C.c_double), ("ms_solve", C.c_double)]


FP64, MIXED, MIXED_EXACT, FP64_DF = 0, 1, 2, 3
PC_JACOBI, PC_BLOCK_JACOBI, PC_LEARNED, PC_SSOR, PC_LEARNED_SSOR, PC_SSOR2, PC_LEARNED_SSOR2 = 0, 1, 2, 3, 4, 5, 6
PC_TWO_LEVEL_JACOBI = 7  # batched solver only: block Jacobi + per-part rigid-body coarse space
HOST, DEVICE = 0, 1
STATUS = {0: "ok", 1: "not converged", 2: "breakdown", 3: "bad mesh", 4: "cuda error", 5: "stagnated",
          6: "barrier timeout"}

_vp, _i, _d = C.c_void_p, C.c_int, C.c_double
_P = C.POINTER

GPU_PROTOTYPES = {
    "bfm_gpu_default_opts": (None, [_P(bfm_gpu_opts_t)]),
    "bfm_gpu_set_opts": (_i, [_P(bfm_gpu_opts_t)]),
    "bfm_gpu_get_opts": (_i, [_P(bfm_gpu_opts_t)]),
    "bfm_gpu_last_stats": (_i, [_P(bfm_gpu_stats_t)]),
    "bfm_gpu_last_error": (C.c_char_p, []),
    "bfm_gpu_device_count": (_i, []),
    "bfm_gpu_set_system_storage": (_i, [_i]),
    "bfm_gpu_instance_set_elem_material": (_i, [_P(abi.bfm_instance_t), _vp, _vp]),
    "bfm_gpu_problem_create": (_i, [_P(_vp), _i, _i, _i, _i, _i, _vp]),
    "bfm_gpu_problem_destroy": (_i, [_vp]),
    "bfm_gpu_problem_set_geometry": (_i, [_vp, _vp, _vp, _i]),
    "bfm_gpu_problem_set_material": (_i, [_vp, _d, _d, _d, _i, _vp, _vp, _i]),
    "bfm_gpu_problem_set_rule": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "bfm_gpu_problem_set_forces": (_i, [_vp, _i, _vp, _vp, _i]),
    "bfm_gpu_problem_set_conditions": (_i, [_vp, _i, _vp, _vp, _vp, _i, _vp, _i]),
    "bfm_gpu_problem_assemble": (_i, [_vp, _i]),
    "bfm_gpu_problem_solve": (_i, [_vp, _P(bfm_gpu_opts_t)]),
    "bfm_gpu_problem_stats": (_i, [_vp, _P(bfm_gpu_stats_t)]),
    "bfm_gpu_problem_solution": (_i, [_vp, _vp, _i]),
    "bfm_gpu_problem_n_blocks": (_i, [_vp, _P(C.c_int64)]),
    "bfm_gpu_problem_download": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "bfm_gpu_problem_stream": (_vp, [_vp]),
    "bfm_gpu_problem_time_kernels": (_i, [_vp, _i, _P(_d), _P(_d)]),
    "bfm_gpu_problem_autotune": (_i, [_vp, _P(_i)]),
    "bfm_gpu_problem_shape": (_i, [_vp, _P(_i)]),
    "bfm_gpu_problem_set_shape": (_i, [_vp, _i]),
    "bfm_gpu_pcg_solve_noalloc": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _d, _i, _P(_i), _P(_d), _vp]),
    "bfm_gpu_problem_set_edge_loads": (_i, [_vp, _i, _vp, _vp, _i]),
    "bfm_gpu_problem_set_edge_boundary": (_i, [_vp, _vp, _i]),
    "bfm_gpu_problem_set_parts": (_i, [_vp, _i, _vp]),
    "bfm_gpu_problem_solve_parts": (_i, [_vp, _P(bfm_gpu_opts_t)]),
    "bfm_gpu_problem_step_parts": (_i, [_vp, _i, _P(bfm_gpu_opts_t)]),
    "bfm_gpu_problem_part_stats": (_i, [_vp, _vp, _vp, _vp, _vp, _P(_i), _P(_i), _P(_d)]),
    "bfm_gpu_problem_parts_coarse": (_i, [_vp, _vp, _vp, _vp]),
    "bfm_gpu_rcm_csr": (_i, [C.c_int64, _vp, _vp, _vp, _vp, _vp]),
    "bfm_gpu_problem_apply": (_i, [_vp, _vp, _vp, _i]),
    "bfm_gpu_problem_ordering": (_i, [_vp, _vp, _vp, _vp]),
    "bfm_gpu_problem_time_precond": (_i, [_vp, _i, _vp, _vp, _vp]),
    "bfm_gpu_problem_coarse_info": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "bfm_gpu_mpnn_param_count": (_i, []),
    "bfm_gpu_mpnn_create": (_i, [_P(_vp), C.c_uint]),
    "bfm_gpu_mpnn_destroy": (_i, [_vp]),
    "bfm_gpu_mpnn_get_weights": (_i, [_vp, _vp]),
    "bfm_gpu_mpnn_set_weights": (_i, [_vp, _vp]),
    "bfm_gpu_mpnn_save": (_i, [_vp, C.c_char_p]),
    "bfm_gpu_mpnn_load": (_i, [_vp, C.c_char_p]),
    "bfm_gpu_mpnn_forward": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "bfm_gpu_mpnn_gradient": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _P(_d), _vp]),
    "bfm_gpu_mpnn_train_step": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _d, _P(_d)]),
    "bfm_gpu_mpnn_use": (_i, [_vp]),
}


def lib() -> C.CDLL:
    """The GPU-backed libbfm, loaded once.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m bfm_gb300.build` "
                              "(the GPU path has no CPU fallback)")
        _lib = abi.bind(C.CDLL(str(LIB_PATH)), GPU_PROTOTYPES)
    return _lib


def default_opts(**kw) -> bfm_gpu_opts_t:
    o = bfm_gpu_opts_t()
    lib().bfm_gpu_default_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def last_error() -> str:
    return (lib().bfm_gpu_last_error() or b"").decode()
