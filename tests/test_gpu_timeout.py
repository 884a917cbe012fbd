"""Bounded waits of the persistent kernels.

The SSOR sweep kernel, the coarse correction of the two-level preconditioner
and the batched solver synchronise their blocks with grid barriers that give
up after opts.barrier_polls polls.  Here the limit is one poll, so a block
that arrives before the others gives up at once (the GPU holds every block of
a cooperative launch, and no barrier can complete between one block's arrival
and its first poll for all of them): the solve must end with the timeout
status and an error, without hanging, and the same problem must solve
normally right after with the default limit."""
import ctypes as C
import os

import numpy as np
import pytest

import bfm_gb300
from bfm_gb300 import api, batch as BA, meshgen as M
from common import rel
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def stats(lib):
    s = bfm_gb300.bfm_gpu_stats_t()
    lib.bfm_gpu_last_stats(C.byref(s))
    return s


@pytest.mark.parametrize("precision", [bfm_gb300.FP64, bfm_gb300.FP64_DF])
def test_barrier_timeout_reports_and_recovers(libbfm, precision):
    p = M.plate(64, 16, 3, traction=1e6)
    x, _, _ = O.solve_direct(p)
    h = api.SimHandle.from_problem(libbfm, p)
    try:
        libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-10, precision=precision,
                                                               precond=bfm_gb300.PC_SSOR2, barrier_polls=1)))
        assert h.run() == -1
        assert "timed out" in h.error()
        assert stats(libbfm).status == 6  # BFM_GPU_TIMEOUT
        libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts(rtol=1e-10, precision=precision,
                                                               precond=bfm_gb300.PC_SSOR2)))
        assert h.run() == 0, h.error()
        s = stats(libbfm)
        assert s.status == 0 and s.rel_residual <= 1e-10
        assert rel(h.effects(), x) < 1e-8
    finally:
        libbfm.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))


def test_batch_barrier_timeout_reports_and_recovers(libbfm):
    """The tiled persistent batch kernel (the one with grid barriers; the
    block-per-part kernel has none) gives up a barrier after one poll, the
    statistics call reports it, and the next solve of the same batch runs."""
    ps = M.batch_uneven(4, seed=11)
    old = os.environ.get("BFM_GPU_BATCH_KERNEL")
    os.environ["BFM_GPU_BATCH_KERNEL"] = "tiled"
    try:
        B = BA.Batch(libbfm, ps)
    finally:
        if old is None:
            del os.environ["BFM_GPU_BATCH_KERNEL"]
        else:
            os.environ["BFM_GPU_BATCH_KERNEL"] = old
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        o = bfm_gb300.default_opts(rtol=1e-8, autotune=0, barrier_polls=1)
        assert libbfm.bfm_gpu_problem_solve_parts(B.P, C.byref(o)) == 0, bfm_gb300.last_error()
        it = np.zeros(len(ps), np.int32)
        rc = libbfm.bfm_gpu_problem_part_stats(B.P, it.ctypes.data, None, None, None, None, None, None)
        assert rc == -1 and "timed out" in bfm_gb300.last_error()
        B.solve(bfm_gb300.default_opts(rtol=1e-8, autotune=0))
        st = B.stats()
        assert np.all(st["status"] == 0) and np.all(st["rel_residual"] <= 1e-8)
    finally:
        B.close()
