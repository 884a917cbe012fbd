"""Double-float path (FP64-accurate CG on the FP32 pipe): same parity bar
as the FP64 path, and an iteration count close to FP64 CG's."""
import ctypes as C

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api, meshgen as M
from common import CASES, load, rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run(lib, p, precision, rtol):
    lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=rtol, precision=precision)))
    try:
        h = api.SimHandle.from_problem(lib, p)
        rc = h.run()
        s = bfm_gb300.bfm_gpu_stats_t()
        lib.bfm_gpu_last_stats(C.byref(s))
        return rc, h, s
    finally:
        lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


@pytest.mark.parametrize("name", CASES)
def test_df_matches_reference(libbfm, name):
    p, d = load(name)
    rc, h, s = run(libbfm, p, bfm_gb300.FP64_DF, 1e-12)
    assert rc == 0, h.error()
    assert rel(h.effects(), d["effects"]) < 1e-10


def test_df_converges_like_fp64(libbfm):
    p = M.cfg_perforated(nx=256, ny=64, n_holes=25, seed=3)
    x, _, _ = O.solve_direct(p)
    rc, h, s64 = run(libbfm, p, bfm_gb300.FP64, 1e-8)
    assert rc == 0
    rc, h, sdf = run(libbfm, p, bfm_gb300.FP64_DF, 1e-8)
    assert rc == 0, h.error()
    assert sdf.rel_residual <= 1.5e-8
    assert rel(h.effects(), x) <= 1e-6
    assert abs(sdf.iterations - s64.iterations) <= 0.05 * s64.iterations + 5
