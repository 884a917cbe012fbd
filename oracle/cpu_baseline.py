"""The reference's CPU algorithm, timed on the host cores (bench.py's CPU
baseline leg and its `--impl reference` arm; TEST/MEASUREMENT INFRASTRUCTURE).

What runs: oracle/bfm_oracle.c's orc_solve_reference -- the reference pipeline
restated (dense assembly + conditions, RCM renumbering, band LU without
pivoting, inverse permutation; libbfm/src/sim.c:103-135), bit-exact with the
reference on the golden fixtures.

Sample: the reference stores K densely (n^2 doubles: 35 TB for the 2.1M-DOF
plate), so the full workload cannot run.  Each step solves the same plate
problem at a bounded size (128x32 cells, 8,514 DOF) once per host core, in
parallel worker processes, and the measured time per DOF is scaled linearly
to the full workload's DOF count.  The reference's cost grows faster than
linearly (O(n^2) assembly storage and RCM scans, O(n k^2) band LU), so the
scaled number is a lower bound on its real time.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import time

SAMPLE = (128, 32)


def _sample_problem(workload: str):
    from bfm_gb300 import meshgen as M
    nx, ny = SAMPLE
    if workload == "perforated":
        return M.cfg_perforated(nx=nx, ny=ny, n_holes=max(1, 200 * nx * ny // (2048 * 512)), seed=3)
    if workload == "q1":
        return M.plate(nx, ny, 4, jitter_frac=0.2, seed=2, traction=1e6)
    return M.plate(nx, ny, 3, traction=1e6)


def _solve_one(workload: str) -> tuple[float, int]:
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from oracle import oracle as O
    p = _sample_problem(workload)
    t0 = time.perf_counter()
    O.solve_reference(p)
    return time.perf_counter() - t0, p.n_dof


def cpu_baseline(workload: str, full_dof: int, steps: int = 1, warmup: int = 0, cores: int | None = None) -> dict:
    from oracle import oracle as O
    O.orc()  # build the port before forking workers
    cores = cores or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(warmup):
            pool.map(_solve_one, [workload] * cores)
        walls, dofs = [], 0
        for _ in range(max(1, steps)):
            t0 = time.perf_counter()
            res = pool.map(_solve_one, [workload] * cores)
            walls.append(time.perf_counter() - t0)
            dofs = sum(n for _, n in res)
    wall = sorted(walls)[len(walls) // 2]
    per_dof_s = wall / dofs
    value_ms = per_dof_s * full_dof * 1e3
    n_sample = dofs // cores
    sample = (f"{cores} parallel solves of the same plate problem at {SAMPLE[0]}x{SAMPLE[1]} cells "
              f"({n_sample} DOF each) per step, {wall:.2f} s wall; time per DOF scaled linearly to "
              f"{full_dof} DOF (a lower bound: the reference path is O(n^2) in memory and time)")
    base = {"value": round(value_ms, 1), "unit": "ms", "cores": cores, "kind": "port", "sample": sample}
    return {
        "metric": "solve ms to 1e-8 residual: learned+mixed PCG vs plain FP64 PCG; SpMV HBM GB/s",
        "value": base["value"], "unit": "ms", "n_gpus": 0, "steps": max(1, steps), "warmup": warmup,
        "ms_per_step": round(wall * 1e3, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded plate generator)", "impl": "reference",
        "config": {"workload": f"{workload} plate (reference algorithm: dense + RCM + band LU)"},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
