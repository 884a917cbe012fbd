"""Shared helpers for the test suite: golden fixtures as meshgen.Problem."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from bfm_gb300 import meshgen as M

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["lepl8", "p1_64x16", "q1_24x8_jitter", "p1_12x6_conds", "p1_20x10_shuffled", "gear12", "p1_16x8_nt"]
# axisymmetric systems with the reference's own formulas (stress = 3): K is
# indefinite, so the fixtures pin the assembly, the RCM and the band solve only
AXI_CASES = ["axi_p1_12x8", "axi_q1_10x6"]


def load(name: str):
    d = np.load(GOLDEN / f"{name}.npz")
    n = d["coords"].shape[0]
    masks = np.unpackbits(d["cond_nodes"], axis=1)[:, :n].astype(bool)
    conds = [(int(k), float(v), masks[i]) for i, (k, v) in enumerate(zip(d["cond_kind"], d["cond_value"]))]
    edges = d["edges"] if d["edges"].shape[0] else None
    p = M.Problem(name, int(d["kind"]), d["coords"], d["elems"], E=float(d["E"]), nu=float(d["nu"]),
                  rho=float(d["rho"]), stress=int(d["stress"]), forces=[tuple(f) for f in d["forces"]],
                  conds=conds, edges=edges,
                  edge_boundary=d["edge_boundary"].astype(bool) if "edge_boundary" in d else None)
    return p, d


def dense_K(d, n):
    K = np.zeros((n, n))
    K[d["K_rows"], d["K_cols"]] = d["K_vals"]
    return K


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def gpu_available() -> bool:
    try:
        import bfm_gb300
        return bfm_gb300.lib().bfm_gpu_device_count() > 0
    except Exception:
        return False
