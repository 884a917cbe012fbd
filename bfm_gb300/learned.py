"""Learned block preconditioner: device problems, the network handle, training
pairs and the training loop.

The network and its kernels live in the library (bfm_gb300/csrc/mpnn.cu,
declared in include/bfm/gpu.h); this module drives them.  Training pairs
come from the plain solver itself: a Jacobi-PCG solve stopped after k
iterations gives x_k, a converged solve gives x*, and the pair is
(r, e) = (K e, x* - x_k), formed on the device (bfm_gpu_problem_apply).
Small batches of uneven plates (the batched workload's generator, solved as
one block-diagonal system) and scaled-down perforated plates provide the
meshes.  The loss is the log of a condition-number estimate of the
preconditioned operator B K: log R(v) - log R(e) with the Rayleigh quotient
R(x) = (x.Kx) / (x.B^-1 x), v a power-iteration vector of B K kept per mesh,
e the solver's error (smooth, so R(e) approaches the bottom of the spectrum).
In the SSOR context (BFM_GPU_PC_LEARNED_SSOR) the blocks are the relaxation
block inverses of the multicolour SSOR preconditioner M, the pairs come from
SSOR-PCG solves, and x.B^-1 x becomes x.M x (mpnn.cu, k_loss_terms).

Device memory for pairs is held in torch tensors (plumbing only): every
computation is a library kernel.

    python -m bfm_gb300.learned --out weights.bin --pairs 20000
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time
from pathlib import Path

import numpy as np

from . import (DEVICE, FP64, PC_BLOCK_JACOBI, PC_JACOBI, PC_LEARNED, PC_LEARNED_SSOR, PC_SSOR, bfm_gpu_stats_t, default_opts,
               last_error, lib)
from . import meshgen as M

WEIGHTS = Path(__file__).resolve().parent / "weights" / "mpnn_plate.bin"
WEIGHTS_SSOR = Path(__file__).resolve().parent / "weights" / "mpnn_ssor.bin"


class DeviceProblem:
    """One meshgen.Problem uploaded into a bfm_gpu_problem (inputs copied once)."""

    def __init__(self, p: M.Problem, stream: int | None = None, precision: int = FP64):
        self.lib = lib()
        self.p = p
        L = self.lib
        P = C.c_void_p()
        n_edges = 0 if p.edges is None else len(p.edges)
        rc = L.bfm_gpu_problem_create(C.byref(P), p.kind, p.n_nodes, p.n_elems, n_edges, len(p.conds), stream)
        assert rc == 0, last_error()
        self.P = P
        keep = []

        def a(x, dt):
            x = np.ascontiguousarray(x, dtype=dt)
            keep.append(x)
            return x.ctypes.data

        ok = L.bfm_gpu_problem_set_geometry(P, a(p.coords, np.float64), a(p.elems, np.int32), 0) == 0
        ok = ok and L.bfm_gpu_problem_set_material(
            P, p.E, p.nu, p.rho, int(p.stress), None if p.elem_E is None else a(p.elem_E, np.float64),
            None if p.elem_nu is None else a(p.elem_nu, np.float64), 0) == 0
        w, ph, dx, de = M.gauss_tables(p.kind)
        ok = ok and L.bfm_gpu_problem_set_rule(P, len(w), a(w, np.float64), a(ph, np.float64), a(dx, np.float64),
                                               a(de, np.float64)) == 0
        f = np.array(p.forces, np.float64).reshape(-1)
        ok = ok and L.bfm_gpu_problem_set_forces(P, len(p.forces), a(f, np.float64) if len(f) else None, None, 0) == 0
        kinds = a([c[0] for c in p.conds], np.int32)
        vals = a([c[1] for c in p.conds], np.float64)
        masks = a(np.stack([c[2] for c in p.conds]).astype(np.uint8), np.uint8)
        edges = a(p.edges, np.int32) if p.edges is not None else None
        ok = ok and L.bfm_gpu_problem_set_conditions(P, len(p.conds), kinds, vals, masks, n_edges, edges, 0) == 0
        if n_edges and p.edge_boundary is not None:
            ok = ok and L.bfm_gpu_problem_set_edge_boundary(P, a(p.edge_boundary, np.uint8), 0) == 0
        if p.edge_loads is not None:
            le, ll = p.edge_loads
            ok = ok and L.bfm_gpu_problem_set_edge_loads(P, len(le), a(le, np.int32), a(ll, np.float64), 0) == 0
        assert ok, last_error()
        self.keep = keep
        self.precision = None
        if precision is not None:
            self.assemble(precision)

    @property
    def n_nodes(self) -> int:
        return self.p.n_nodes

    def assemble(self, precision: int = FP64):
        assert self.lib.bfm_gpu_problem_assemble(self.P, precision) == 0, last_error()
        self.precision = precision

    def solve(self, **opts) -> bfm_gpu_stats_t:
        o = default_opts(**opts)
        assert self.lib.bfm_gpu_problem_solve(self.P, C.byref(o)) == 0, last_error()
        s = bfm_gpu_stats_t()
        assert self.lib.bfm_gpu_problem_stats(self.P, C.byref(s)) == 0, last_error()
        return s

    def solution(self, out=None):
        """Host copy (numpy), or into a device pointer `out` (on the problem's stream)."""
        if out is None:
            x = np.zeros(2 * self.n_nodes)
            assert self.lib.bfm_gpu_problem_solution(self.P, x.ctypes.data, 0) == 0, last_error()
            return x
        assert self.lib.bfm_gpu_problem_solution(self.P, C.c_void_p(out), DEVICE) == 0, last_error()
        return out

    def apply(self, x_ptr: int, y_ptr: int):
        """y = K x on the device (FP64 operator)."""
        assert self.lib.bfm_gpu_problem_apply(self.P, C.c_void_p(x_ptr), C.c_void_p(y_ptr), DEVICE) == 0, last_error()

    def download(self):
        """(row_ptr, cols, vals (nb, 2, 2), b) of the assembled system."""
        nb = C.c_int64()
        assert self.lib.bfm_gpu_problem_n_blocks(self.P, C.byref(nb)) == 0
        rp = np.zeros(self.n_nodes + 1, np.int32)
        cols = np.zeros(nb.value, np.int32)
        vals = np.zeros((nb.value, 2, 2))
        b = np.zeros(2 * self.n_nodes)
        assert self.lib.bfm_gpu_problem_download(self.P, rp.ctypes.data, cols.ctypes.data, vals.ctypes.data,
                                                 b.ctypes.data) == 0, last_error()
        return rp, cols, vals, b

    def stream(self) -> int:
        return self.lib.bfm_gpu_problem_stream(self.P) or 0

    def close(self):
        if self.P:
            self.lib.bfm_gpu_problem_destroy(self.P)
            self.P = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Network:
    """Handle of a bfm_gpu_mpnn (weights on the device)."""

    def __init__(self, seed: int = 0, path: str | Path | None = None):
        self.lib = lib()
        h = C.c_void_p()
        assert self.lib.bfm_gpu_mpnn_create(C.byref(h), seed) == 0, last_error()
        self.h = h
        self.n_params = self.lib.bfm_gpu_mpnn_param_count()
        if path is not None:
            self.load(path)

    def load(self, path):
        assert self.lib.bfm_gpu_mpnn_load(self.h, str(path).encode()) == 0, last_error()

    def save(self, path):
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        assert self.lib.bfm_gpu_mpnn_save(self.h, str(path).encode()) == 0, last_error()

    def weights(self) -> np.ndarray:
        w = np.zeros(self.n_params, np.float32)
        assert self.lib.bfm_gpu_mpnn_get_weights(self.h, w.ctypes.data) == 0, last_error()
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == self.n_params
        assert self.lib.bfm_gpu_mpnn_set_weights(self.h, w.ctypes.data) == 0, last_error()

    def forward(self, prob: DeviceProblem):
        n = prob.n_nodes
        f = np.zeros((n, 16), np.float32)
        c = np.zeros((n, 3), np.float32)
        B = np.zeros((n, 2, 2))
        assert self.lib.bfm_gpu_mpnn_forward(self.h, prob.P, f.ctypes.data, c.ctypes.data, B.ctypes.data) == 0, \
            last_error()
        return f, c, B

    def gradient(self, prob: DeviceProblem, r_ptr: int, e_ptr: int, v_ptr: int, power_iters: int = 0):
        loss = C.c_double()
        g = np.zeros(self.n_params, np.float32)
        assert self.lib.bfm_gpu_mpnn_gradient(self.h, prob.P, C.c_void_p(r_ptr), C.c_void_p(e_ptr), C.c_void_p(v_ptr),
                                              power_iters, C.byref(loss), g.ctypes.data) == 0, last_error()
        return loss.value, g

    def train_step(self, prob: DeviceProblem, r_ptr: int, e_ptr: int, v_ptr: int, lr: float,
                   power_iters: int = 4) -> float:
        loss = C.c_double()
        assert self.lib.bfm_gpu_mpnn_train_step(self.h, prob.P, C.c_void_p(r_ptr), C.c_void_p(e_ptr),
                                                C.c_void_p(v_ptr), power_iters, lr, C.byref(loss)) == 0, last_error()
        return loss.value

    def use(self):
        assert self.lib.bfm_gpu_mpnn_use(self.h) == 0

    def close(self):
        if self.h:
            self.lib.bfm_gpu_mpnn_use(None)
            self.lib.bfm_gpu_mpnn_destroy(self.h)
            self.h = None


# ---------------------------------------------------------------- training data

def training_meshes(seed: int, n_plates: int = 2, n_batch: int = 1, batch_parts: int = 12):
    """Meshes of the training set: perforated plates at a quarter of the
    benchmark's resolution with their own hole seeds, and block-diagonal
    batches of uneven plates from the batched workload's generator."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_plates):
        nx = int(rng.choice([256, 384, 512]))
        out.append(M.cfg_perforated(nx=nx, ny=nx // 4, n_holes=200, seed=int(rng.integers(1 << 30))))
    for k in range(n_batch):
        parts = M.batch_uneven(batch_parts, seed=int(rng.integers(1 << 30)))
        out.append(concat(parts))
    return out


def concat(problems) -> M.Problem:
    """Block-diagonal union of P1 problems as one Problem: per-element E and
    nu, the Dirichlet masks of each kind merged (homogeneous values only),
    every Neumann condition carried as per-edge loads (each mesh keeps its
    own magnitude; loads skip constrained DOFs)."""
    off = np.cumsum([0] + [p.n_nodes for p in problems])
    n = int(off[-1])
    coords = np.concatenate([p.coords for p in problems])
    elems = np.concatenate([p.elems + off[k] for k, p in enumerate(problems)])
    eE = np.concatenate([p.elem_E if p.elem_E is not None else np.full(p.n_elems, p.E) for p in problems])
    enu = np.concatenate([p.elem_nu if p.elem_nu is not None else np.full(p.n_elems, p.nu) for p in problems])
    masks = {M.DIRICHLET_X: np.zeros(n, bool), M.DIRICHLET_Y: np.zeros(n, bool)}
    for k, p in enumerate(problems):
        for kind, v, mask in p.conds:
            if kind in masks:
                if v != 0.0:
                    raise ValueError("concatenated Dirichlet conditions must be homogeneous")
                masks[kind][off[k]:off[k + 1]] |= mask
    loads = [M.neumann_edge_loads(p, off[k]) for k, p in enumerate(problems)]
    return M.Problem(name=f"concat{len(problems)}", kind=problems[0].kind, coords=coords, elems=elems,
                     elem_E=eE, elem_nu=enu, forces=list(problems[0].forces),
                     conds=[(kind, 0.0, m) for kind, m in masks.items()],
                     edge_loads=(np.concatenate([e for e, _ in loads]), np.concatenate([l for _, l in loads])))


def working_index(prob: DeviceProblem):
    """Device index of the problem's working order per DOF (None for the
    caller's order): x_working = x_caller[index]."""
    import torch
    perm = np.zeros(prob.n_nodes, np.int32)
    nc = C.c_int(0)
    assert prob.lib.bfm_gpu_problem_ordering(prob.P, perm.ctypes.data, None, C.byref(nc)) == 0, last_error()
    if nc.value == 0:
        return None
    d = np.stack([2 * perm, 2 * perm + 1], 1).reshape(-1).astype(np.int64)
    return torch.from_numpy(d).cuda()


def pairs(prob: DeviceProblem, stops=(32, 64, 128, 256, 512, 1024, 2048), rtol: float = 1e-10, ssor: bool = False):
    """(r, e) device pairs (torch float64 tensors) from partial PCG solves:
    Jacobi, or with ssor the multicolour SSOR (vectors in the problem's
    colour-major working order, as the loss kernels read them)."""
    import torch
    n = 2 * prob.n_nodes
    pc = PC_SSOR if ssor else PC_JACOBI
    st = prob.solve(precond=pc, rtol=rtol)
    assert st.status in (0, 5), (st.status, last_error())
    xs = torch.empty(n, dtype=torch.float64, device="cuda")
    prob.solution(xs.data_ptr())
    idx = working_index(prob) if ssor else None
    out = []
    for k in stops:
        prob.solve(precond=pc, rtol=rtol, max_iters=k)
        xk = torch.empty(n, dtype=torch.float64, device="cuda")
        prob.solution(xk.data_ptr())
        torch.cuda.synchronize()
        e = xs - xk
        if idx is not None:
            e = e[idx].contiguous()
        if float(torch.linalg.vector_norm(e)) == 0.0:
            continue
        r = torch.empty_like(e)
        torch.cuda.synchronize()
        prob.apply(e.data_ptr(), r.data_ptr())
        torch.cuda.synchronize()
        out.append((r, e))
    return out


def train(net: Network, probs, n_pairs: int, lr: float = 3e-4, epochs: int = 1, seed: int = 0, log=None,
          power_iters: int = 4, warm_power: int = 60, ssor: bool = False):
    """Adam over the pairs of `probs` (a list of DeviceProblem); returns the
    mean loss of each epoch and the number of distinct pairs.  Each problem
    keeps its power-iteration vector: `warm_power` steps before training,
    `power_iters` more at every training step on it.  ssor: train the
    relaxation blocks of the SSOR preconditioner (the problems are left in
    its colour order)."""
    import torch
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    data, vecs = [], []
    for i, pr in enumerate(probs):
        for r, e in pairs(pr, ssor=ssor):
            data.append((i, r, e))
        v = torch.rand(2 * pr.n_nodes, dtype=torch.float64, device="cuda", generator=gen) - 0.5
        torch.cuda.synchronize()
        vecs.append(v)
    if not data:
        raise RuntimeError("no training pairs")
    for i, pr in enumerate(probs):
        r, e = next((r, e) for j, r, e in data if j == i)
        net.gradient(pr, r.data_ptr(), e.data_ptr(), vecs[i].data_ptr(), warm_power)
    hist = []
    steps = max(n_pairs, len(data)) * epochs
    order = rng.integers(0, len(data), steps)
    losses = []
    for t, j in enumerate(order):
        i, r, e = data[j]
        losses.append(net.train_step(probs[i], r.data_ptr(), e.data_ptr(), vecs[i].data_ptr(), lr, power_iters))
        if log and (t + 1) % 500 == 0:
            log(f"step {t + 1}/{steps} loss {np.mean(losses[-500:]):.5f}")
    n_ep = max(1, epochs)
    per = len(losses) // n_ep
    for k in range(n_ep):
        hist.append(float(np.mean(losses[k * per:(k + 1) * per])))
    return hist, len(data)


def evaluate(net: Network, prob: DeviceProblem, rtol: float = 1e-8, precision: int | None = None, ssor: bool = False):
    """Iterations and ms of Jacobi, block-Jacobi (the untrained network) and
    learned PCG on one problem; ssor: Jacobi, block SSOR (the untrained
    network) and learned SSOR."""
    if precision is not None and precision != prob.precision:
        prob.assemble(precision)
    net.use()
    res = {}
    methods = ((("jacobi", PC_JACOBI), ("block_ssor", PC_SSOR), ("learned", PC_LEARNED_SSOR)) if ssor else
               (("jacobi", PC_JACOBI), ("block_jacobi", PC_BLOCK_JACOBI), ("learned", PC_LEARNED)))
    for name, pc in methods:
        s = prob.solve(precond=pc, rtol=rtol)
        res[name] = dict(iterations=s.iterations, status=s.status, fallback=s.fallback, ms=s.ms_solve,
                         rel_residual=s.rel_residual)
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--context", choices=["jacobi", "ssor"], default="jacobi",
                    help="blocks of the block-Jacobi preconditioner, or relaxation blocks of the multicolour SSOR")
    ap.add_argument("--out", default=None, help="weights file (default: the package's file for the context)")
    ap.add_argument("--pairs", type=int, default=20000, help="training steps (one pair each)")
    ap.add_argument("--meshes", type=int, default=6, help="training meshes (each gives several pairs)")
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--seed", type=int, default=5)
    args = ap.parse_args(argv)
    ssor = args.context == "ssor"
    out = args.out or str(WEIGHTS_SSOR if ssor else WEIGHTS)
    import torch
    torch.cuda.init()
    t0 = time.time()
    meshes = training_meshes(args.seed, n_plates=args.meshes - args.meshes // 3, n_batch=args.meshes // 3)
    probs = [DeviceProblem(p) for p in meshes]
    net = Network(seed=args.seed)
    hist, n_data = train(net, probs, args.pairs, lr=args.lr, seed=args.seed, log=print, ssor=ssor)
    net.save(out)
    held = DeviceProblem(M.cfg_perforated(nx=512, ny=128, n_holes=200, seed=3))
    ev = evaluate(net, held, ssor=ssor)
    print(json.dumps({"context": args.context, "pairs_distinct": n_data, "steps": args.pairs, "loss": hist,
                      "held_out": ev, "seconds": round(time.time() - t0, 1), "out": out}))


if __name__ == "__main__":
    main()
