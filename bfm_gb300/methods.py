"""Named solve methods: a precision, a preconditioner and the FP64 residual
replacement threshold tuned for them (the recurrence residual must drop by
this factor between two replacements; in the mixed precisions each
replacement is an FP64 iterative-refinement step).  The thresholds come from
sweeps on the 2048x512 perforated plate: FP64 is insensitive, the paths on
the FP32 pipe converge in fewer iterations with rarer replacements, and the
mixed two-level SSOR takes its fewest iterations with a step every 1e-1."""
from __future__ import annotations

from . import (FP64, FP64_DF, MIXED, MIXED_EXACT, PC_JACOBI, PC_LEARNED, PC_LEARNED_SSOR, PC_LEARNED_SSOR2,
               PC_SSOR, PC_SSOR2, default_opts)

# name: (precision, preconditioner, replace_drop)
METHODS = {
    "fp64": (FP64, PC_JACOBI, 0.1),
    "fp64_df": (FP64_DF, PC_JACOBI, 0.01),
    "mixed_exact": (MIXED_EXACT, PC_JACOBI, 0.001),
    "mixed": (MIXED, PC_JACOBI, 0.001),
    "learned_fp64": (FP64, PC_LEARNED, 0.1),
    "learned_df": (FP64_DF, PC_LEARNED, 0.01),
    "learned_mixed": (MIXED, PC_LEARNED, 0.001),
    "ssor_fp64": (FP64, PC_SSOR, 0.1),
    "ssor_df": (FP64_DF, PC_SSOR, 0.01),
    "learned_ssor_df": (FP64_DF, PC_LEARNED_SSOR, 0.01),
    "ssor2_fp64": (FP64, PC_SSOR2, 0.1),
    "ssor2_df": (FP64_DF, PC_SSOR2, 0.01),
    "learned_ssor2_df": (FP64_DF, PC_LEARNED_SSOR2, 0.01),
    "ssor2_mixed": (MIXED, PC_SSOR2, 0.1),
    "ssor2_mixed_exact": (MIXED_EXACT, PC_SSOR2, 0.1),
    "learned_ssor2_mixed": (MIXED, PC_LEARNED_SSOR2, 0.1),
}

# arithmetic of each precision, as the benchmark line states it
ARITHMETIC = {
    FP64: "fp64 assembly, fp64 SpMV and vectors",
    FP64_DF: "fp64 assembly, double-float (fp32 pairs) SpMV and vectors, fp64 dots and final residual",
    MIXED_EXACT: "fp64 assembly rounded to fp32, fp32 SpMV and vectors, fp64 dots and refinement",
    MIXED: "fp32 assembly, fp32 SpMV and vectors, fp64 dots and refinement",
}

# what each method is, as the benchmark line states it
_PC = {PC_JACOBI: "Jacobi", PC_LEARNED: "learned block-Jacobi (message-passing network)",
       PC_SSOR: "multicolour block SSOR", PC_LEARNED_SSOR: "multicolour block SSOR, learned relaxation blocks",
       PC_SSOR2: "two-level SSOR (multicolour block SSOR + rigid-body coarse space)",
       PC_LEARNED_SSOR2: "two-level SSOR, learned relaxation blocks"}
_PREC = {FP64: "FP64 PCG", FP64_DF: "double-float PCG, FP64 tail", MIXED: "FP32 PCG with FP64 iterative refinement",
         MIXED_EXACT: "FP32 PCG (FP64-assembled operator) with FP64 iterative refinement"}
DESCRIPTION = {k: f"{_PREC[p]}, {_PC[c]} preconditioner" for k, (p, c, _) in METHODS.items()}


def opts(name: str, rtol: float, **kw):
    """bfm_gpu_opts_t for a named method."""
    precision, precond, drop = METHODS[name]
    return default_opts(rtol=rtol, precision=precision, precond=precond, replace_drop=drop, **kw)
