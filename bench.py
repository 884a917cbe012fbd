"""Benchmark of the libbfm FEM hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                    [--workload perforated|q1|batch] [--method best|m1,m2,...] [--profile]

Workload (default): the perforated plate -- 2048x512 P1 triangles, 1,051,137
nodes, 2,102,274 DOF, 200 soft inclusions (E x 1e-3, seed 3), left edge
clamped, gravity, 1e6 Pa traction on the right edge, plane stress.  One step
= sparsity pattern + element loop + Dirichlet/Neumann + preconditioner set-up
+ PCG to relative residual 1e-8, with every input already in HBM (`value`).
`e2e` is the same step through the reference-facing C API, bfm_sim_run, with
host buffers: host->device upload of the mesh and conditions and
device->host copy of the displacements are inside its timed region.

Every default method (precision x preconditioner, bfm_gb300.methods) runs a
short selection pass (3 warm-up + 3 timed steps); the fastest one whose
displacements agree with a direct (SuperLU) solve of the FP64 system to 1e-6
is then timed with the requested W + K steps and reported, and `methods`
lists them all with their own step counts.  `roofline` describes the dominant kernel of that
method's iteration (the SSOR sweep kernel for the SSOR methods, with the SpMV in
`roofline_spmv`; the SpMV otherwise).

--impl reference times the reference's own algorithm (dense assembly, RCM,
band LU), restated in oracle/ and run on the host cores, on bounded samples
of the same plate; see `cpu_baseline()`.

Multi-GPU: the path solves one mesh per GPU (replicas, no collective); with
N ranks every rank solves its own copy and `value` is ms per solved plate of
the whole job (max time over ranks / N).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "solve ms to 1e-8 residual: learned+mixed PCG vs plain FP64 PCG; SpMV HBM GB/s"
RTOL = 1e-8

# methods timed by default (the bfm_gb300.methods table has them all): the
# plain FP64 Jacobi-PCG baseline, the benchmark spec's mixed precision with the
# learned preconditioner, and the fast preconditioners in every precision
DEFAULT_METHODS = ("fp64", "fp64_df", "mixed", "learned_mixed", "learned_df", "ssor_df", "ssor2_fp64", "ssor2_df",
                   "learned_ssor2_df", "ssor2_mixed", "learned_ssor2_mixed")
SELECT_STEPS = 3  # timed steps per method in the selection pass (after 3 warm-up steps)
SSOR_PCS = (3, 4, 5, 6)      # BFM_GPU_PC_SSOR, _LEARNED_SSOR, _SSOR2, _LEARNED_SSOR2
LEARNED_PCS = (2, 4, 6)
# fused SpMV kernel (K1) of each precision: the roofline kernel
SPMV_KERNEL = {0: "k_hs64_spmv", 1: "k_mx_spmv", 2: "k_mx_spmv", 3: "k_hsdf_spmv"}
# DRAM bytes (read + write) of one K1 launch on the 2048x512 perforated plate,
# from one ncu capture each (the profiles/ summaries named here)
SPMV_TRAFFIC = {0: (343_951_104, "profiles/spmv_fp64_hs_perforated_2048x512.md"),
                3: (329_563_136, "profiles/spmv_df_hs_perforated_2048x512.md"),
                1: (205_397_248, "profiles/spmv_fp32_mixed_perforated_2048x512.md"),
                2: (205_397_248, "profiles/spmv_fp32_mixed_perforated_2048x512.md")}
# the same for one launch of the SSOR sweep kernel, per (precision, two-level
# correction fused, kernel: 1 k_ssor_all, 2 k_ssor_tma), where a capture of the
# current kernel exists
SSOR_TRAFFIC = {(1, True, 1): (269_338_112, "profiles/ssor2_fused_mixed_perforated_2048x512.md"),
                (1, True, 2): (266_680_576, "profiles/ssor2_tma_mixed_perforated_2048x512.md")}


def algorithmic_bytes_ssor(n_blocks: int, n_nodes: int, precision: int) -> int:
    """One SSOR application: every off-diagonal block once (FP32 block +
    column index, 20 B), and per node the FP32 relaxation block (16 B), the
    residual read and z written (16 B each for FP64 and double-float, 8 B for
    the mixed precisions' FP32 vectors) and the double-float sweep vector
    written once (16 B)."""
    vec = 8 if precision in (1, 2) else 16
    return (n_blocks - n_nodes) * 20 + n_nodes * (16 + 2 * vec + 16)


def algorithmic_bytes_coarse(n_nodes: int, n_chunks: int, x_bytes: int) -> int:
    """The two-level correction's own reads inside the sweep kernel, per
    application (the residual and z are counted with the sweeps): per node its
    aggregate list entry and aggregate (4 B each) and its offset and free flags
    (16 B); per restriction chunk its start (4 B) and 3 partial sums (24 B);
    the rows of X and X^T (FP32, padded to 16 B)."""
    return n_nodes * (4 + 4 + 16) + n_chunks * (4 + 24) + x_bytes


def max_over_ranks(x: float, world: int) -> float:
    """Max of a per-rank number over all ranks (NCCL on GPUs, gloo on CPUs)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name: str):
    from bfm_gb300 import meshgen as M
    if name == "perforated":
        return M.cfg_perforated()
    if name == "q1":
        return M.cfg_q1_large()
    if name.startswith("small"):
        return M.plate(256, 64, 3, traction=1e6)
    raise SystemExit(f"unknown workload {name}")


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes_spmv(n_blocks: int, n_nodes: int, precision: int, block_pc: bool = False) -> int:
    """Bytes one launch of the fused SpMV kernel (K1: direction update, A p,
    (p, A p)) must move at least: block values + column indices + row
    pointers, plus its node vectors touched once.  FP64 and double-float
    (16 B per node vector): z and p read, p' and q written.  Mixed (8 B per
    node vector): r, p and the preconditioner read (Jacobi 8 B, block 16 B
    per node), the 16 B correction block read, p' and q written."""
    if precision in (0, 3):
        return n_blocks * (32 + 4) + 4 * (n_nodes + 1) + n_nodes * 64
    return n_blocks * (16 + 4) + 4 * (n_nodes + 1) + n_nodes * (8 + 8 + (16 if block_pc else 8) + 16 + 8 + 8)


def direct_solution(lib, D, p):
    """Displacements of a direct (SuperLU) solve of the FP64 system the GPU
    assembles, refined once with an extended-precision residual: the yardstick
    of every method's displacement error.  The FP64 system is bit-identical
    to the oracle's restatement of the reference assembly (the slow config
    tests check that at this size)."""
    import scipy.sparse.linalg as spla
    import bfm_gb300
    from bfm_gb300 import api
    D.assemble(bfm_gb300.FP64)
    rp, cols, vals, b = D.download()
    perm = np.zeros(p.n_nodes, np.int32)
    assert lib.bfm_gpu_problem_ordering(D.P, perm.ctypes.data, None, None) == 0
    K = api.scalar_csr(rp, cols, vals.reshape(-1), p.n_nodes, perm)
    bb = np.empty_like(b)
    bb[np.stack([2 * perm, 2 * perm + 1], 1).ravel()] = b
    t0 = time.perf_counter()
    lu = spla.splu(K.tocsc(), permc_spec="MMD_AT_PLUS_A", options=dict(SymmetricMode=True))
    x = lu.solve(bb)
    KL = K.astype(np.longdouble)
    r = bb.astype(np.longdouble) - KL @ x.astype(np.longdouble)
    x = (x.astype(np.longdouble) + lu.solve(r.astype(np.float64))).astype(np.float64)
    return x, time.perf_counter() - t0


def time_method(lib, D, stream, m, nets, warmup, steps, clocks=False):
    """W untimed + K timed steps of method m (assembly + solve, inputs in
    HBM), CUDA events on the problem's stream; then its statistics, solution
    and per-kernel durations."""
    import torch
    import bfm_gb300
    from bfm_gb300.methods import METHODS, opts
    prec, pc, _ = METHODS[m]
    if pc in nets:
        nets[pc].use()
    o = opts(m, RTOL)

    def step():
        assert lib.bfm_gpu_problem_assemble(D.P, prec) == 0, bfm_gb300.last_error()
        assert lib.bfm_gpu_problem_solve(D.P, C.byref(o)) == 0, bfm_gb300.last_error()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clk = Clocks(int(os.environ.get("LOCAL_RANK", 0))) if clocks else None
    if clk:
        clk.__enter__()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if clk:
        clk.__exit__()
    ms = ev0.elapsed_time(ev1) / steps
    s = bfm_gb300.bfm_gpu_stats_t()
    assert lib.bfm_gpu_problem_stats(D.P, C.byref(s)) == 0
    x = D.solution()
    # per-kernel durations for the roofline (same stream, CUDA events)
    t_spmv, t_upd = C.c_double(), C.c_double()
    assert lib.bfm_gpu_problem_time_kernels(D.P, 50, C.byref(t_spmv), C.byref(t_upd)) == 0
    shape = C.c_int()
    lib.bfm_gpu_problem_shape(D.P, C.byref(shape))
    ncol = C.c_int(0)
    lib.bfm_gpu_problem_ordering(D.P, None, None, C.byref(ncol))
    t_pc, t_sw, persist = C.c_double(0.0), C.c_double(0.0), C.c_int(0)
    n_coarse, n_chunks, x_bytes, fused = C.c_int64(0), C.c_int64(0), C.c_int64(0), C.c_int(0)
    if pc in SSOR_PCS:
        assert lib.bfm_gpu_problem_time_precond(D.P, 20, C.byref(t_pc), C.byref(t_sw), C.byref(persist)) == 0, \
            bfm_gb300.last_error()
        lib.bfm_gpu_problem_coarse_info(D.P, C.byref(n_coarse), C.byref(n_chunks), C.byref(x_bytes), C.byref(fused))
    if pc in nets:
        lib.bfm_gpu_mpnn_use(None)
    return dict(ms=ms, steps=steps, warmup=warmup, iters=s.iterations, status=s.status, rel_res=s.rel_residual,
                repl=s.replacements, ms_assemble=s.ms_assemble, ms_solve=s.ms_solve, n_blocks=s.n_blocks,
                fallback=s.fallback, ms_spmv=t_spmv.value, ms_update=t_upd.value,
                clocks=clk.summary() if clk else None, prec=prec, pc=pc, x=x, shape=shape.value, ncol=ncol.value,
                ms_precond=t_pc.value, ms_sweeps=t_sw.value, persistent=persist.value,
                coarse=dict(n_coarse=n_coarse.value, n_chunks=n_chunks.value, x_bytes=x_bytes.value,
                            fused=fused.value))


def run_gpu(args, rank: int, world: int):
    import torch
    import bfm_gb300
    from bfm_gb300 import api, learned
    from bfm_gb300.methods import METHODS, opts

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    lib = bfm_gb300.lib()
    p = workload(args.workload)
    # a dedicated stream: the problem's kernels and the timing events share it
    # (torch's default stream is the legacy NULL stream, which the library
    # would replace by a private one)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    # the networks: block-Jacobi blocks, and SSOR relaxation blocks (each
    # trained in its own context)
    nets = {pc: learned.Network(path=w) for pc, w in ((bfm_gb300.PC_LEARNED, learned.WEIGHTS),
                                                    (bfm_gb300.PC_LEARNED_SSOR, learned.WEIGHTS_SSOR)) if w.exists()}
    if bfm_gb300.PC_LEARNED_SSOR in nets:  # the relaxation blocks serve the two-level form too
        nets[bfm_gb300.PC_LEARNED_SSOR2] = nets[bfm_gb300.PC_LEARNED_SSOR]
    chosen = list(DEFAULT_METHODS) if args.method == "best" else args.method.split(",")
    missing = [m for m in chosen if METHODS[m][1] in LEARNED_PCS and METHODS[m][1] not in nets]
    if missing and args.method != "best":
        raise SystemExit(f"the weights of {missing} are missing: train them with python -m bfm_gb300.learned")
    chosen = [m for m in chosen if m not in missing]
    D = learned.DeviceProblem(p, stream=stream.cuda_stream, precision=None)
    x_direct, t_direct = (direct_solution(lib, D, p) if not args.no_direct else (None, 0.0))
    # selection pass: a few steps of every method; then the fastest one whose
    # displacements are within 1e-6 of the direct solve, W + K steps
    results = {}
    single = len(chosen) == 1
    for m in chosen:
        results[m] = time_method(lib, D, stream, m, nets, args.warmup if single else 3,
                                 args.steps if single else min(args.steps, SELECT_STEPS), clocks=single)
    for m, r in results.items():
        r["err_vs_direct"] = None if x_direct is None else float(np.linalg.norm(r["x"] - x_direct) /
                                                                   np.linalg.norm(x_direct))
    ok = [m for m, r in results.items() if r["status"] == 0 and (r["err_vs_direct"] is None or r["err_vs_direct"] <= 1e-6)]
    best = min(ok or results, key=lambda k: results[k]["ms"])
    if not single:
        if world > 1:
            torch.distributed.barrier()
        err = results[best]["err_vs_direct"]
        results[best] = time_method(lib, D, stream, best, nets, args.warmup, args.steps, clocks=True)
        results[best]["err_vs_direct"] = err
    D.close()

    # end-to-end through bfm_sim_run with host buffers (the learned methods use
    # the network selected above through the same global options); the first
    # run on the mesh is cold: it colours it, forms the coarse grid and tunes
    # the SpMV shape
    prec, pc, _ = METHODS[best]
    if pc in nets:
        nets[pc].use()
    lib.bfm_gpu_set_opts(C.byref(opts(best, RTOL)))
    h = api.SimHandle.from_problem(lib, p)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    assert h.run() == 0, h.error()
    cold_ms = (time.perf_counter() - t0) * 1e3
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_e2e = max(1, args.steps // 2)
    for _ in range(n_e2e):
        assert h.run() == 0, h.error()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / n_e2e
    n_masks = len(p.conds) * p.n_nodes
    h2d = p.n_nodes * 16 + p.n_elems * p.kind * 4 + n_masks + (0 if p.edges is None else 8 * len(p.edges)) + \
        (0 if p.elem_E is None else 8 * p.n_elems)
    d2h = p.n_dof * 8
    lib.bfm_gpu_set_opts(C.byref(bfm_gb300.default_opts()))
    lib.bfm_gpu_mpnn_use(None)
    for n_ in {id(v): v for v in nets.values()}.values():
        n_.close()
    return p, results, best, dict(ms=e2e_ms, cold_ms=cold_ms, h2d=h2d, d2h=d2h, steps=n_e2e), t_direct


def run_batch(steps=3, warmup=3, precond=None):
    """256 independent plates (nx ~ U{32..256}, ny ~ U{8..64}, per-element E
    log-uniform in [1e9, 2e11], seed 4): every step is one CUDA graph launch
    holding the assembly of the block-diagonal batch, the preconditioner's
    set-up and the persistent batched solve, every mesh to rtol 1e-8
    (MIXED_EXACT: FP64 assembly, FP32 iteration, FP64 residuals).  The
    reported preconditioner is the two-level block Jacobi (a rigid-body coarse
    space per mesh); plain Jacobi is timed beside it (`jacobi`)."""
    import torch
    import bfm_gb300
    from bfm_gb300 import batch as BA, meshgen as M
    if precond is None:
        line = run_batch(steps, warmup, bfm_gb300.PC_TWO_LEVEL_JACOBI)
        jac = run_batch(steps, warmup, bfm_gb300.PC_JACOBI)
        line["jacobi"] = {k: jac[k] for k in ("ms_per_step", "dof_per_s", "all_converged", "iterations_min",
                                              "iterations_median", "iterations_max")}
        return line
    lib = bfm_gb300.lib()
    ps = M.batch_uneven(256, seed=4)
    stream = torch.cuda.Stream()
    B = BA.Batch(lib, ps, stream=C.c_void_p(stream.cuda_stream))
    o = bfm_gb300.default_opts(rtol=RTOL, precond=precond)
    for _ in range(warmup):
        B.step(bfm_gb300.MIXED_EXACT, o)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        B.step(bfm_gb300.MIXED_EXACT, o)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    st = B.stats()
    B.close()
    dof = int(sum(p.n_dof for p in ps))
    it = st["iterations"]
    name = "two-level block Jacobi" if precond == bfm_gb300.PC_TWO_LEVEL_JACOBI else "Jacobi"
    return {"workload": "256 uneven P1 plates (seed 4), one graph launch per step (assembly + batched solve)",
            "preconditioner": name, "dof": dof, "steps": steps, "warmup": warmup, "ms_per_step": round(ms, 3),
            "dof_per_s": round(dof / (ms * 1e-3), 1), "all_converged": bool((st["status"] == 0).all()),
            "max_rel_residual": float(st["rel_residual"].max()), "iterations_min": int(it.min()),
            "iterations_median": int(np.median(it)), "iterations_max": int(it.max()),
            "rows_per_tile": st["rows_per_tile"], "lanes_per_row": st["lanes_per_row"]}


def profile_batch(args):
    """The batched workload's solve alone, for profilers: the 256 uneven
    plates assembled once (MIXED_EXACT), then `reps` solves with fixed shapes
    (512 threads per block, 2 lanes per row: no autotuning launches), the
    two-level block Jacobi preconditioner (`--method jacobi` for Jacobi)."""
    import bfm_gb300
    from bfm_gb300 import batch as BA, meshgen as M
    lib = bfm_gb300.lib()
    pc = bfm_gb300.PC_JACOBI if args.method == "jacobi" else bfm_gb300.PC_TWO_LEVEL_JACOBI
    B = BA.Batch(lib, M.batch_uneven(256, seed=4))
    try:
        B.assemble(bfm_gb300.MIXED_EXACT)
        o = bfm_gb300.default_opts(rtol=RTOL, precond=pc, autotune=0)
        ms = []
        for _ in range(max(args.reps, 1)):
            B.solve(o)
            st = B.stats()
            ms.append(st["ms_solve"])
    finally:
        B.close()
    it = st["iterations"]
    return {"workload": "256 uneven P1 plates (seed 4)", "preconditioner": "jacobi" if pc == 0 else "two-level block Jacobi",
            "ms_solve": min(ms), "threads_per_block": st["rows_per_tile"], "lanes_per_row": st["lanes_per_row"],
            "iterations_median": int(np.median(it)), "iterations_max": int(it.max()),
            "all_converged": bool((st["status"] == 0).all())}


def profile(args):
    """Assemble once, then the CG's SpMV+dots and update kernels as standalone
    launches (the solve itself runs them inside a CUDA graph), the SSOR
    preconditioner's applications and the network's inference where the
    method has them."""
    import bfm_gb300
    from bfm_gb300 import learned
    from bfm_gb300.methods import METHODS
    lib = bfm_gb300.lib()
    p = workload(args.workload)
    prec, pc, drop = METHODS.get(args.method, METHODS["fp64"])
    D = learned.DeviceProblem(p, precision=prec)
    s = bfm_gb300.bfm_gpu_stats_t()
    assert lib.bfm_gpu_problem_stats(D.P, C.byref(s)) == 0
    lpr = C.c_int(0)
    assert lib.bfm_gpu_problem_autotune(D.P, C.byref(lpr)) == 0, bfm_gb300.last_error()
    t_spmv, t_upd = C.c_double(), C.c_double()
    assert lib.bfm_gpu_problem_time_kernels(D.P, args.reps, C.byref(t_spmv), C.byref(t_upd)) == 0
    ms_net = None
    ms_pc, ms_sw, ncol, persist = None, None, C.c_int(0), C.c_int(0)
    if pc in SSOR_PCS:
        # two iterations form the colour order (and the coarse operator) and
        # the sweep graph; then the preconditioner alone, `reps` applications
        two = pc in (bfm_gb300.PC_SSOR2, bfm_gb300.PC_LEARNED_SSOR2)
        D.solve(precond=bfm_gb300.PC_SSOR2 if two else bfm_gb300.PC_SSOR, max_iters=2, replace_drop=drop)
        t, t_sw = C.c_double(), C.c_double()
        assert lib.bfm_gpu_problem_time_precond(D.P, args.reps, C.byref(t), C.byref(t_sw), C.byref(persist)) == 0, \
            bfm_gb300.last_error()
        ms_sw = t_sw.value
        lib.bfm_gpu_problem_ordering(D.P, None, None, C.byref(ncol))
        ms_pc = t.value
    if pc == bfm_gb300.PC_LEARNED:
        # the network's inference (features, 4 dense layers on the tensor cores, 3
        # aggregations, head), timed on the problem's stream with CUDA events
        import torch
        net = learned.Network(path=learned.WEIGHTS)
        stream = lib.bfm_gpu_problem_stream(D.P)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ext = torch.cuda.ExternalStream(stream)
        for _ in range(2):
            assert lib.bfm_gpu_mpnn_forward(net.h, D.P, None, None, None) == 0, bfm_gb300.last_error()
        e0.record(ext)
        for _ in range(args.reps):
            assert lib.bfm_gpu_mpnn_forward(net.h, D.P, None, None, None) == 0, bfm_gb300.last_error()
        e1.record(ext)
        torch.cuda.synchronize()
        ms_net = e0.elapsed_time(e1) / args.reps
        net.close()
    D.close()
    nbytes = algorithmic_bytes_spmv(s.n_blocks, p.n_nodes, prec)
    return {"workload": p.name, "method": args.method, "lanes_per_row": lpr.value, "n_blocks": s.n_blocks,
            "ms_assemble": s.ms_assemble,
            "spmv_ms": t_spmv.value, "update_ms": t_upd.value, "spmv_algorithmic_bytes": nbytes,
            "spmv_gbs": nbytes / (t_spmv.value * 1e-3) / 1e9, "network_forward_ms": ms_net,
            "precond_ms": ms_pc, "sweeps_ms": ms_sw, "colours": ncol.value, "persistent_sweeps": persist.value,
            "sweeps_algorithmic_bytes": algorithmic_bytes_ssor(s.n_blocks, p.n_nodes, prec) if ms_sw else None}


def run_reference(args, rank: int, world: int):
    """The reference algorithm (oracle port) on bounded samples, host cores."""
    from oracle.cpu_baseline import cpu_baseline
    p_full_dof = 2 * 2049 * 513 if args.workload == "perforated" else 2 * 1025 * 257
    return cpu_baseline(args.workload, p_full_dof, steps=args.steps, warmup=args.warmup)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="perforated")
    ap.add_argument("--method", default="best",
                    help="best (the default methods, fastest accurate one reported), or a comma-separated list of "
                         "bfm_gb300.methods names")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-direct", action="store_true", help="skip the direct solve (no err_vs_direct)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched workload's line (`batch`)")
    ap.add_argument("--profile", action="store_true",
                    help="assemble once and launch the two CG kernels --reps times each, standalone "
                         "(for ncu: one JSON line with their CUDA-event durations)")
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.profile:
        print(json.dumps(profile_batch(args) if args.workload == "batch" else profile(args)))
        return
    if args.workload == "batch":
        print(json.dumps(run_batch(steps=args.steps, warmup=args.warmup)))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        line = run_reference(args, rank, world)
        print(json.dumps(line))
        return

    # CPU baseline first: its worker processes start before any CUDA call
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle.cpu_baseline import cpu_baseline
        full = 2 * 2049 * 513 if args.workload == "perforated" else 2 * 1025 * 257
        cpu = cpu_baseline(args.workload, full, steps=3, warmup=1)["cpu_baseline"]

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    p, results, best, e2e, t_direct = run_gpu(args, rank, world)
    if rank != 0:
        return
    batch = run_batch() if args.workload == "perforated" and not args.no_batch else None
    from bfm_gb300.methods import ARITHMETIC, DESCRIPTION
    hbm, peak_kind = peaks()
    r = results[best]
    nb = r["n_blocks"]
    bytes_spmv = algorithmic_bytes_spmv(nb, p.n_nodes, r["prec"], r["pc"] != 0)
    achieved = bytes_spmv / (r["ms_spmv"] * 1e-3) / 1e9
    split = r["shape"] >= 1000
    traffic, traffic_src = (SPMV_TRAFFIC.get(r["prec"], (None, None))
                            if args.workload == "perforated" and r["pc"] == 0 and r["shape"] in (1, 2) else (None, None))
    kernel = SPMV_KERNEL[r["prec"]]
    if split:
        kernel = kernel.replace("_spmv", "_dir") + " + " + kernel + "_s"
    # assembly (pattern, Dirichlet marks, element loop, loads: about 24 kernels),
    # solve init + 2 kernels per iteration + replacement kernels, finish;
    # the learned preconditioner adds its 12 inference kernels per solve
    per_iter = 3 if split else 2
    ssor = r["pc"] in SSOR_PCS
    if ssor:
        # the SSOR sweeps after the init, every update and every replacement:
        # one cooperative launch (the two-level form's coarse correction runs
        # inside it), or 2 nc - 1 colour phases and four coarse kernels
        # (restriction, chunk sums, the products by X and X^T)
        coarse = (0 if r["persistent"] else 4) if r["pc"] in (5, 6) else 0
        per_pc = (1 if r["persistent"] else 2 * r["ncol"] - 1) + coarse
    else:
        per_pc = 0
    launches_per_step = 24 + 1 + (per_iter + per_pc) * r["iters"] + (2 + per_pc) * r["repl"] + per_pc + 2 + \
        (12 if r["pc"] in LEARNED_PCS else 0)
    spmv_roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                 "frac": round(achieved / hbm, 3), "traffic": traffic, "traffic_source": traffic_src,
                 "kernel": kernel, "spmv_shape": r["shape"], "algorithmic_bytes": bytes_spmv,
                 "kernel_ms": round(r["ms_spmv"], 5), "peak_source": peak_kind}
    if ssor:
        # the dominant kernel of an SSOR iteration is the sweep kernel, as the
        # solve launches it: with the two-level correction's stages inside when
        # they are fused (then its bytes count too), else the sweeps alone
        co = r["coarse"]
        fused = bool(co["fused"]) and bool(r["persistent"])
        b_pc = algorithmic_bytes_ssor(nb, p.n_nodes, r["prec"])
        t_pc = r["ms_sweeps"]
        if fused:
            b_pc += algorithmic_bytes_coarse(p.n_nodes, co["n_chunks"], co["x_bytes"])
            t_pc = r["ms_precond"]
        a_pc = b_pc / (t_pc * 1e-3) / 1e9
        tr = SSOR_TRAFFIC.get((r["prec"], fused, r["persistent"])) if args.workload == "perforated" else None
        roof = {"bound": "hbm", "achieved": round(a_pc, 1), "peak": hbm, "unit": "GB/s", "frac": round(a_pc / hbm, 3),
                "traffic": tr[0] if tr else None, "traffic_source": tr[1] if tr else None,
                "kernel": (("k_ssor_tma" if r["persistent"] == 2 else "k_ssor_all") +
                           (" (two-level correction fused)" if fused else "")) if r["persistent"]
                else "k_ssor_fwd + k_ssor_bwd",
                "algorithmic_bytes": b_pc, "kernel_ms": round(t_pc, 5), "peak_source": peak_kind,
                "coarse_dofs": co["n_coarse"]}
    else:
        roof = spmv_roof
    value = r["ms"] / world
    dtype = {0: "f64", 1: "f32", 2: "f32", 3: "f32x2 (double-float)"}[r["prec"]]
    line = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "ms",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(r["ms"], 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": dtype,
        "arithmetic": ARITHMETIC[r["prec"]],
        "data": "synthetic (seeded plate generator)",
        "config": {"workload": f"{p.name}: {p.n_dof} DOF, {p.n_elems} P{1 if p.kind == 3 else 2} elements",
                   "method": best, "method_description": DESCRIPTION[best], "rtol": RTOL,
                   "l2": "inputs larger than L2 (matrix %.0f MB)" % (nb * (4 * (8 if r['prec'] == 0 else 4) + 4) / 1e6),
                   "parallelism": f"replicas{world}"},
        "iterations": r["iters"],
        "rel_residual": r["rel_res"],
        "err_vs_direct": r.get("err_vs_direct"),
        "direct_solve_s": round(t_direct, 1),
        "ms_assemble": round(r["ms_assemble"], 3),
        "ms_solve": round(r["ms_solve"], 3),
        "methods": {k: {"ms": round(v["ms"], 3), "steps": v["steps"], "iterations": v["iters"], "status": v["status"],
                        "rel_residual": v["rel_res"], "err_vs_direct": v.get("err_vs_direct"),
                        "replacements": v["repl"], "fallback": v["fallback"], "ms_assemble": round(v["ms_assemble"], 3),
                        "spmv_ms": round(v["ms_spmv"], 5), "update_ms": round(v["ms_update"], 5),
                        "spmv_shape": v["shape"],
                        **({"precond_ms": round(v["ms_precond"], 5), "sweeps_ms": round(v["ms_sweeps"], 5),
                            "colours": v["ncol"],
                            "sweeps": {0: "per colour", 1: "persistent", 2: "persistent, TMA-staged"}[v["persistent"]]}
                           if v["pc"] in SSOR_PCS else {})}
                    for k, v in results.items()},
        "speedup_vs_fp64": (round(results["fp64"]["ms"] / r["ms"], 3) if "fp64" in results else None),
        "spmv_gbs": round(achieved, 1),
        "roofline": roof,
        **({"roofline_spmv": spmv_roof} if ssor else {}),
        "e2e": {"value": round(e2e["ms"], 3), "unit": "ms", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"], "steps": e2e["steps"]},
        "e2e_cold_ms": round(e2e["cold_ms"], 3),
        "gpu_launches": launches_per_step * args.steps,
        "clocks": r["clocks"],
        "cpu_baseline": cpu,
        "batch": batch,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
