// Krylov kernels of the GB300 libbfm solver: grid reductions, the FP64 and
// mixed-precision PCG iterations and residual checks.  Included by every
// translation unit that launches them (internal linkage: each gets its own
// instantiations).
#pragma once

#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>

#include <bfm/gpu.h>

#include "reduce.cuh"

namespace {

// ------------------------------------------------------------------ CG (Chronopoulos-Gear PCG)
//
// One reduction point per iteration:
//   u = M r, w = A u, gamma = (r,u), delta = (w,u), rho = (r,r)
//   beta = gamma/gamma_old, alpha = gamma/(delta - beta*gamma/alpha_old)
//   p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s
// Kernel A: SpMV on u = M r (formed on the fly) + the three inner products;
// its last block computes alpha, beta and the stopping test.
// Kernel B: the four vector updates.

struct CgState {
	double bnorm2;
	double gamma;      // (r, M r) of the current residual
	double gamma_old, alpha_old;
	double alpha, beta;
	double rho;        // (r,r) of the current recurrence residual
	double rho_ref;    // mixed: (r,r) right after the last residual replacement
	double true_res2;  // ||b - A x||^2 after the solve
	double rtol, drop2;
	double best_true2;  // smallest true residual seen at a replacement
	int iter, max_iters;
	int done, status;
	int replacements;
	int stall;          // replacements in a row without halving best_true2's norm
	double ssor_acc;    // SSOR: (r, z) summed over the sweep phases
	int ssor_err;       // SSOR: a grid barrier of the persistent sweep kernel timed out
	int repl_req;       // outside a graph: the last K2 asked for a residual replacement
};

// After an FP64 true residual: converged, or stagnating at the roundoff floor
// of the arithmetic (five replacements in a row without halving the best
// residual), or keep going.  Returns 1 when the solve should stop.
__device__ __forceinline__ int true_residual_verdict(CgState* st, double res2) {
	st->replacements += 1;
	st->rho_ref = res2;
	st->true_res2 = res2;
	if (res2 <= st->rtol * st->rtol * st->bnorm2) return 1;
	if (st->replacements == 1 || res2 < 0.25 * st->best_true2) {
		st->best_true2 = res2;
		st->stall = 0;
		return 0;
	}
	if (++st->stall >= 5) {
		st->status = BFM_GPU_STAGNATED;
		return 1;
	}
	return 0;
}

struct CgOpts {
	double rtol;
	double drop2;  // mixed: replace when (r,r) has dropped by this factor since the last replacement
	int max_iters;
	int restart;   // mixed: each FP64 refinement step restarts the inner PCG (beta = 0)
};

// Vectors are interleaved (u,v) per node and accessed as pairs.
template <typename V>
struct CgArgs {
	int N;
	const int* row_ptr;
	const int* cols;
	const V* vals;          // iteration operator (2x2 blocks)
	const double* vals64;   // FP64 operator for true residuals (nullptr: `vals` widened)
	const V* dinv;          // Jacobi: 2 per node; block Jacobi: 4 per node
	const float* corr;      // mixed: per-node 2x2 row-sum block S of the operator (difference form)
	int block_pc;
	const double* b;
	double* x;
	V* r;
	V* u;   // FP64 path: u = M r (materialized); mixed path: dx, the grouped solution update
	V* p;   // FP64 path: direction; mixed path: direction read this iteration
	V* pn;  // mixed path: direction written this iteration (ping-pong with p)
	V* s;   // FP64 path: s = A p by recurrence
	V* w;   // FP64 path: w = A u; mixed path: q = A p
	V* z;   // mixed path with SSOR sweeps: z = M r, formed by the sweeps (no_pc)
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgOpts opts;
	cudaGraphConditionalHandle cond;       // while-node: keep iterating
	cudaGraphConditionalHandle cond_repl;  // if-node: replace the residual this iteration
	int use_cond;  // launched inside the solve graph: drive its conditional nodes
	int timing;    // measurement launches: ignore the stop flag, never set it
	int no_pc;     // the SSOR sweeps form z = M r and gamma after this kernel
};

// 2x2 block k of the matrix: m0 m1 / m2 m3 (one 32-byte or 16-byte vector load)
__device__ __forceinline__ void ld_block(const double* v, long k, double& m0, double& m1, double& m2, double& m3) {
	double2 const a = reinterpret_cast<const double2*>(v)[2 * k];
	double2 const b = reinterpret_cast<const double2*>(v)[2 * k + 1];
	m0 = a.x; m1 = a.y; m2 = b.x; m3 = b.y;
}
__device__ __forceinline__ void ld_block(const float* v, long k, float& m0, float& m1, float& m2, float& m3) {
	float4 const a = reinterpret_cast<const float4*>(v)[k];
	m0 = a.x; m1 = a.y; m2 = a.z; m3 = a.w;
}

template <typename V>
__device__ __forceinline__ void precond_apply(const V* dinv, int block_pc, int c, V r0, V r1, V& u0, V& u1) {
	if (block_pc) {
		V m0, m1, m2, m3;
		ld_block(dinv, c, m0, m1, m2, m3);
		u0 = m0 * r0 + m1 * r1;
		u1 = m2 * r0 + m3 * r1;
	}
	else {
		auto const d = ld2(dinv, c);
		u0 = d.x * r0;
		u1 = d.y * r1;
	}
}

// One block row of y = A g with LPR lanes per row: lane `sub` takes blocks
// sub, sub+LPR, ... (adjacent lanes read adjacent blocks: coalesced vector
// loads), then the group adds its partial sums with shuffles.  Every lane of
// the warp must call this (rows past the end pass ks == ke).
template <int LPR, typename A, typename V, typename G>
__device__ __forceinline__ void row_product(const int* __restrict__ cols, const V* __restrict__ vals, int ks, int ke, int sub,
                                            G gather, A& y0, A& y1) {
	y0 = A(0);
	y1 = A(0);
#pragma unroll 2
	for (int k = ks + sub; k < ke; k += LPR) {
		int const c = cols[k];
		A g0, g1;
		gather(c, g0, g1);
		V m0, m1, m2, m3;
		ld_block(vals, k, m0, m1, m2, m3);
		y0 += A(m0) * g0 + A(m1) * g1;
		y1 += A(m2) * g0 + A(m3) * g1;
	}
#pragma unroll
	for (int o = LPR / 2; o; o >>= 1) {
		y0 += __shfl_xor_sync(0xffffffffu, y0, o);
		y1 += __shfl_xor_sync(0xffffffffu, y1, o);
	}
}

// True residual of one block row, r = b - A x with the FP64 matrix, in
// compensated arithmetic: every product split exactly by an FMA
// (TwoProduct), the sums carried as (sum, error) pairs (TwoSum), the lanes'
// pairs combined the same way, and b - (s + c) formed with a TwoSum.  An
// FP64 residual carries an error near eps |A| |x|, which on the perforated
// plates is a third of 1e-8 relative; computed this way it is accurate to
// about eps |r|, so replacements and the convergence test see the residual
// of the stored x rather than rounding noise.  Every lane must call it.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
	s = __dadd_rn(a, b);
	double const z = __dsub_rn(s, a);
	e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, z)), __dsub_rn(b, z));
}
__device__ __forceinline__ void dd_acc(double& s, double& c, double a, double b) {
	double const p = __dmul_rn(a, b);
	double const pe = __fma_rn(a, b, -p);
	double t, te;
	two_sum(s, p, t, te);
	s = t;
	c = __dadd_rn(c, __dadd_rn(te, pe));
}
template <int LPR>
__device__ __forceinline__ void residual_dd(const int* __restrict__ cols, const double* __restrict__ vals, int ks, int ke, int sub,
                                            const double* __restrict__ x, double2 bb, double& r0, double& r1) {
	double s0 = 0.0, c0 = 0.0, s1 = 0.0, c1 = 0.0;
	for (int k = ks + sub; k < ke; k += LPR) {
		double2 const g = ld2(x, cols[k]);
		double m0, m1, m2, m3;
		ld_block(vals, k, m0, m1, m2, m3);
		dd_acc(s0, c0, m0, g.x);
		dd_acc(s0, c0, m1, g.y);
		dd_acc(s1, c1, m2, g.x);
		dd_acc(s1, c1, m3, g.y);
	}
#pragma unroll
	for (int o = LPR / 2; o; o >>= 1) {
		double t, e;
		two_sum(s0, __shfl_xor_sync(0xffffffffu, s0, o), t, e);
		c0 = __dadd_rn(__dadd_rn(c0, __shfl_xor_sync(0xffffffffu, c0, o)), e);
		s0 = t;
		two_sum(s1, __shfl_xor_sync(0xffffffffu, s1, o), t, e);
		c1 = __dadd_rn(__dadd_rn(c1, __shfl_xor_sync(0xffffffffu, c1, o)), e);
		s1 = t;
	}
	double h, e;
	two_sum(bb.x, -s0, h, e);
	r0 = __dadd_rn(h, __dsub_rn(e, c0));
	two_sum(bb.y, -s1, h, e);
	r1 = __dadd_rn(h, __dsub_rn(e, c1));
}

// Same product with the loads batched: each lane first reads NB column
// indices, then issues the NB neighbour gathers and the NB block loads, then
// does the arithmetic, so NB independent memory chains are in flight per lane
// instead of one (the kernels are bound by gather latency, not bandwidth).
// Entries are summed in the order k = ks+sub, ks+sub+LPR, ... as above.
template <int LPR, int NB, typename A, typename V, typename G>
__device__ __forceinline__ void row_product_pf(const int* __restrict__ cols, const V* __restrict__ vals, int ks, int ke,
                                               int sub, G gather, A& y0, A& y1) {
	y0 = A(0);
	y1 = A(0);
	for (int k0 = ks + sub; k0 < ke; k0 += LPR * NB) {
		int c[NB];
#pragma unroll
		for (int j = 0; j < NB; j++) c[j] = k0 + j * LPR < ke ? cols[k0 + j * LPR] : -1;
		A g0[NB], g1[NB];
#pragma unroll
		for (int j = 0; j < NB; j++) {
			g0[j] = g1[j] = A(0);
			if (c[j] >= 0) gather(c[j], g0[j], g1[j]);
		}
		V m[NB][4];
#pragma unroll
		for (int j = 0; j < NB; j++) {
			m[j][0] = m[j][1] = m[j][2] = m[j][3] = V(0);
			if (c[j] >= 0) ld_block(vals, k0 + j * LPR, m[j][0], m[j][1], m[j][2], m[j][3]);
		}
#pragma unroll
		for (int j = 0; j < NB; j++) {
			y0 += A(m[j][0]) * g0[j] + A(m[j][1]) * g1[j];
			y1 += A(m[j][2]) * g0[j] + A(m[j][3]) * g1[j];
		}
	}
#pragma unroll
	for (int o = LPR / 2; o; o >>= 1) {
		y0 += __shfl_xor_sync(0xffffffffu, y0, o);
		y1 += __shfl_xor_sync(0xffffffffu, y1, o);
	}
}

template <int LPR, int NB, typename A, typename V, typename G>
__device__ __forceinline__ void row_product_nb(const int* __restrict__ cols, const V* __restrict__ vals, int ks, int ke,
                                               int sub, G gather, A& y0, A& y1) {
	if constexpr (NB == 1) row_product<LPR, A>(cols, vals, ks, ke, sub, gather, y0, y1);
	else row_product_pf<LPR, NB, A>(cols, vals, ks, ke, sub, gather, y0, y1);
}

// row loop shared by the SpMV kernels: every warp runs the same number of trips
#define FOR_ROWS(LPR)                                                                          \
	int const sub_ = threadIdx.x % (LPR);                                                       \
	int const rows_per_block_ = blockDim.x / (LPR);                                             \
	for (int base_ = blockIdx.x * rows_per_block_; base_ < a.N; base_ += gridDim.x * rows_per_block_) \
		for (int row_ = base_ + threadIdx.x / (LPR), once_ = 1; once_; once_ = 0)

// ---------------------------------------------------------------- init

template <typename V>
__global__ void __launch_bounds__(TPB_K) k_cg_init(CgArgs<V> a, int mixed) {
	double v[2] = {0.0, 0.0};  // (b,b), (b, M b)
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const bb = ld2(a.b, i);
		V const r0 = (V) bb.x, r1 = (V) bb.y;
		V u0 = (V) 0, u1 = (V) 0;
		if (!a.no_pc) precond_apply(a.dinv, a.block_pc, i, r0, r1, u0, u1);
		st2(a.x, i, 0.0, 0.0);
		st2(a.r, i, r0, r1);
		st2(a.p, i, (V) 0, (V) 0);
		if (!mixed) {
			st2(a.u, i, u0, u1);
			st2(a.s, i, (V) 0, (V) 0);
		}
		else {
			st2(a.u, i, (V) 0, (V) 0);
		}
		v[0] += bb.x * bb.x + bb.y * bb.y;
		v[1] += (double) r0 * (double) u0 + (double) r1 * (double) u1;
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		CgState* st = a.st;
		st->bnorm2 = out[0];
		st->gamma = out[1];
		st->rtol = a.opts.rtol;
		st->drop2 = a.opts.drop2;
		st->max_iters = a.opts.max_iters;
		st->iter = 0;
		st->replacements = 0;
		st->stall = 0;
		st->best_true2 = out[0];
		st->status = BFM_GPU_OK;
		st->done = out[0] == 0.0;  // b = 0: x = 0 is exact
		st->gamma_old = 0; st->alpha_old = 0;
		st->alpha = 0; st->beta = 0;
		st->rho = out[0];
		st->rho_ref = out[0];
		st->true_res2 = out[0];
		st->ssor_err = 0;
		st->repl_req = 0;
		if (a.use_cond) cudaGraphSetConditional(a.cond, st->done ? 0u : 1u);
	}
}

// ---------------------------------------------------------------- FP64, single reduction
// (bfm_gpu_pcg_solve_noalloc) Chronopoulos-Gear PCG: one reduction per iteration and only the SpMV's
// 4 FP64 FMAs per block in the gathered loop (FP64 issue rate bounds this
// path on GB300, so u = M r is materialized once per node instead of being
// formed per neighbour).
//   A: w = A u; gamma = (r,u), delta = (w,u), rho = (r,r); alpha, beta
//   B: p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = M r

template <int LPR>
__global__ void __launch_bounds__(TPB_K) k_cg64_spmv(CgArgs<double> a) {
	CgState* st = a.st;
	// The loop continues only if this launch's finisher says so: block 0
	// clears the condition first, the last block sets it after the stopping
	// test.  A launch whose finisher did not run therefore ends the loop.
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(a.cond, 0u);
	if (st->done && !a.timing) return;
	double v[3] = {0.0, 0.0, 0.0};
	const double* __restrict__ u = a.u;
	auto gather = [u](int c, double& g0, double& g1) {
		double2 const t = ld2(u, c);
		g0 = t.x;
		g1 = t.y;
	};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		double y0, y1;
		row_product<LPR, double>(a.cols, a.vals, ks, ke, sub_, gather, y0, y1);
		if (ok && sub_ == 0) {
			st2(a.w, row_, y0, y1);
			double2 const ri = ld2(a.r, row_), ui = ld2(u, row_);
			v[0] += ri.x * ui.x + ri.y * ui.y;
			v[1] += y0 * ui.x + y1 * ui.y;
			v[2] += ri.x * ri.x + ri.y * ri.y;
		}
	}
	double out[3];
	if (grid_sum<3>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		double const gamma = out[0], delta = out[1], rho = out[2];
		st->rho = rho;
		int stop = 0;
		if (rho <= st->rtol * st->rtol * st->bnorm2) {
			stop = 1;
		}
		else if (st->iter >= st->max_iters) {
			stop = 1;
			if (!a.timing) st->status = BFM_GPU_NOT_CONVERGED;
		}
		else {
			double beta = 0.0, den = delta;
			if (st->iter > 0) {
				beta = gamma / st->gamma_old;
				den = delta - beta * gamma / st->alpha_old;
			}
			if (!(den > 0.0) || !(gamma > 0.0)) {
				stop = 1;
				if (!a.timing) st->status = BFM_GPU_BREAKDOWN;
			}
			else {
				double const alpha = gamma / den;
				st->alpha = alpha;
				st->beta = beta;
				st->gamma_old = gamma;
				st->alpha_old = alpha;
				st->iter += 1;
			}
		}
		if (a.timing) return;
		st->done = stop;
		if (a.use_cond && !stop) cudaGraphSetConditional(a.cond, 1u);
	}
}

__global__ void __launch_bounds__(TPB_K) k_cg64_update(CgArgs<double> a) {
	CgState const* st = a.st;
	if (st->done && !a.timing) return;
	double const alpha = st->alpha, beta = st->beta;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const u = ld2(a.u, i), p = ld2(a.p, i), s = ld2(a.s, i), w = ld2(a.w, i);
		double2 const x = ld2(a.x, i), r = ld2(a.r, i);
		double const p0 = u.x + beta * p.x, p1 = u.y + beta * p.y;
		double const s0 = w.x + beta * s.x, s1 = w.y + beta * s.y;
		double const r0 = r.x - alpha * s0, r1 = r.y - alpha * s1;
		st2(a.p, i, p0, p1);
		st2(a.s, i, s0, s1);
		st2(a.x, i, x.x + alpha * p0, x.y + alpha * p1);
		st2(a.r, i, r0, r1);
		double u0, u1;
		precond_apply(a.dinv, a.block_pc, i, r0, r1, u0, u1);
		st2(a.u, i, u0, u1);
	}
}

// ---------------------------------------------------------------- mixed path
// Hestenes-Stiefel PCG with an FP32 operator, FP32 Krylov vectors and FP64
// only where accuracy needs it.  GB300 issues FP64 at a small fraction of its
// FP32 rate, so the iteration does no per-entry FP64 arithmetic at all:
//   - inner products accumulate in double-float pairs (error-free FP32
//     transformations, about 48 significant bits) and become FP64 once per
//     thread;
//   - the solution update is grouped: dx += alpha p' in FP32, flushed into the
//     FP64 x only before each FP64 residual replacement and at the end;
//   - the FP32 operator is applied in difference form,
//         (A g)_r = S_r g_r + sum_c A32_rc (g_c - g_r),
//     with S_r the node's 2x2 block row sum of the operator (zero for an
//     interior node, kept from the FP64 sums or as a double-float sum).  It
//     keeps the rigid translation modes exact (without them the FP32 operator
//     loses definiteness on ill-conditioned meshes and CG diverges), and for a
//     smooth g the differences are small and exact, so the cancellation of a
//     stiffness row (its terms sum to about zero) costs no FP32 accuracy.
//   K1: p' = M r + beta p; q = A p' (difference form); alpha = gamma / (p', q)
//   K2: dx += alpha p'; r -= alpha q; gamma' = (r, M r), rho = (r, r); beta
//   on request (IF node): x += dx, dx = 0; r = b - A64 x in FP64; gamma = (r, M r)

// K2 finisher when the SSOR sweeps come next: the iteration count, the cap
// and the replacement request (from rho alone); beta and gamma follow from
// the sweeps' (r, z)
__device__ __forceinline__ void hs_rho(CgState* st, double rho, int timing, int use_cond, cudaGraphConditionalHandle cond,
                                       cudaGraphConditionalHandle cond_repl) {
	if (timing) return;
	double const tol2 = st->rtol * st->rtol * st->bnorm2;
	st->rho = rho;
	st->iter += 1;
	if (st->iter >= st->max_iters) {
		st->status = BFM_GPU_NOT_CONVERGED;
		st->done = 1;
		if (use_cond) cudaGraphSetConditional(cond, 0u);
	}
	else if (use_cond && (rho <= st->drop2 * st->rho_ref || rho <= tol2)) {
		cudaGraphSetConditional(cond_repl, 1u);
	}
}

struct DF {
	float hi, lo;
};

// s += a*b without rounding loss (TwoProduct via FMA, TwoSum); the _rn
// intrinsics keep the compiler from contracting or reassociating
__device__ __forceinline__ void df_add_prod(DF& s, float a, float b) {
	float const p = __fmul_rn(a, b);
	float const e = __fmaf_rn(a, b, -p);
	float const t = __fadd_rn(s.hi, p);
	float const z = __fsub_rn(t, s.hi);
	float const err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, z)), __fsub_rn(p, z));
	s.hi = t;
	s.lo = __fadd_rn(s.lo, __fadd_rn(err, e));
}

__device__ __forceinline__ double df_value(DF const& s) { return (double) s.hi + (double) s.lo; }

template <int LPR, int NB = 1>
__global__ void __launch_bounds__(TPB_K) k_mx_spmv(CgArgs<float> a) {
	CgState* st = a.st;
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	float const beta = (float) st->beta;
	const float* __restrict__ r = a.r;
	const float* __restrict__ p = a.p;
	const float* __restrict__ dinv = a.dinv;
	const float* __restrict__ zv = a.z;
	int const bpc = a.block_pc, zpc = a.no_pc;
	auto gather = [=](int c, float& g0, float& g1) {
		float2 const pc = ld2(p, c);
		float z0, z1;
		if (zpc) {  // z = M r from the SSOR sweeps
			float2 const zc = ld2(zv, c);
			z0 = zc.x;
			z1 = zc.y;
		}
		else {      // z = M r of the point or block Jacobi preconditioner, on the fly
			float2 const rc = ld2(r, c);
			precond_apply(dinv, bpc, c, rc.x, rc.y, z0, z1);
		}
		g0 = z0 + beta * pc.x;
		g1 = z1 + beta * pc.y;
	};
	DF pq = {0.f, 0.f};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		// difference form: y = S g_r + sum_c K_rc (g_c - g_r); for a smooth g
		// the differences are small and exact, so nothing cancels in FP32
		float g0 = 0.f, g1 = 0.f;
		if (ok) gather(row_, g0, g1);
		auto dgather = [=](int c, float& d0, float& d1) {
			gather(c, d0, d1);
			d0 -= g0;
			d1 -= g1;
		};
		float y0, y1;
		row_product_nb<LPR, NB, float>(a.cols, a.vals, ks, ke, sub_, dgather, y0, y1);
		if (ok && sub_ == 0) {
			float4 const cc = reinterpret_cast<const float4*>(a.corr)[row_];
			y0 += cc.x * g0 + cc.y * g1;
			y1 += cc.z * g0 + cc.w * g1;
			st2(a.pn, row_, g0, g1);
			st2(a.w, row_, y0, y1);
			df_add_prod(pq, g0, y0);
			df_add_prod(pq, g1, y1);
		}
	}
	double v[1] = {df_value(pq)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		double const d = out[0];
		if (!(d > 0.0)) {
			if (!a.timing) {
				st->done = 1;
				st->status = BFM_GPU_BREAKDOWN;
			}
			return;  // the while condition stays cleared
		}
		st->alpha = st->gamma / d;
		if (a.use_cond) cudaGraphSetConditional(a.cond, 1u);
	}
}

__global__ void __launch_bounds__(TPB_K) k_mx_update(CgArgs<float> a) {
	CgState* st = a.st;
	if (st->done && !a.timing) return;
	float const alpha = (float) st->alpha;
	DF g = {0.f, 0.f}, rr = {0.f, 0.f};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		float2 const pn = ld2(a.pn, i), q = ld2(a.w, i), r = ld2(a.r, i), dx = ld2(a.u, i);
		st2(a.u, i, dx.x + alpha * pn.x, dx.y + alpha * pn.y);
		float const r0 = r.x - alpha * q.x, r1 = r.y - alpha * q.y;
		st2(a.r, i, r0, r1);
		if (!a.no_pc) {
			float z0, z1;
			precond_apply(a.dinv, a.block_pc, i, r0, r1, z0, z1);
			df_add_prod(g, r0, z0);
			df_add_prod(g, r1, z1);
		}
		df_add_prod(rr, r0, r0);
		df_add_prod(rr, r1, r1);
	}
	double v[2] = {df_value(g), df_value(rr)};
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (a.no_pc) {  // the SSOR sweeps come next: gamma and beta follow from their (r, z)
			hs_rho(st, out[1], a.timing, a.use_cond, a.cond, a.cond_repl);
			return;
		}
		if (a.timing) return;
		double const gamma = out[0], rho = out[1];
		double const tol2 = st->rtol * st->rtol * st->bnorm2;
		st->rho = rho;
		st->iter += 1;
		st->beta = gamma / st->gamma;
		st->gamma = gamma;
		int stop = 0, repl = 0;
		if (st->iter >= st->max_iters) {
			stop = 1;
			st->status = BFM_GPU_NOT_CONVERGED;
		}
		else if (!(gamma > 0.0)) {
			// r = 0 exactly, or NaN: let the FP64 residual decide
			repl = gamma == 0.0;
			if (!repl) {
				stop = 1;
				st->status = BFM_GPU_BREAKDOWN;
			}
		}
		else {
			// the FP32 recurrence has lost `drop` since the last FP64
			// residual, or claims convergence: refresh from FP64
			repl = rho <= st->drop2 * st->rho_ref || rho <= tol2;
		}
		if (stop) {
			st->done = 1;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
		else if (repl && a.use_cond) {
			cudaGraphSetConditional(a.cond_repl, 1u);
		}
	}
}

// x += dx (FP64), dx = 0
__global__ void __launch_bounds__(TPB_K) k_mx_flush(CgArgs<float> a) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		float2 const dx = ld2(a.u, i);
		if (dx.x == 0.f && dx.y == 0.f) continue;
		double2 const x = ld2(a.x, i);
		st2(a.x, i, x.x + (double) dx.x, x.y + (double) dx.y);
		st2(a.u, i, 0.f, 0.f);
	}
}

// y = A_res x in FP64, LPR lanes per row.  The residual operator is the FP64
// matrix when present, else the iteration matrix widened plus its
// correction blocks.
template <int LPR, typename V>
__device__ __forceinline__ void residual_row(const CgArgs<V>& a, int row, int sub, double& e0, double& e1) {
	bool const ok = row < a.N;
	int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
	const double* __restrict__ x = a.x;
	auto gather = [x](int c, double& g0, double& g1) {
		double2 const t = ld2(x, c);
		g0 = t.x;
		g1 = t.y;
	};
	double2 const xi = ok ? ld2(x, row) : make_double2(0.0, 0.0);
	auto dgather = [x, xi](int c, double& g0, double& g1) {  // difference form of the FP32 operator
		double2 const t = ld2(x, c);
		g0 = t.x - xi.x;
		g1 = t.y - xi.y;
	};
	if (a.vals64) {
		double2 const bb = ok ? ld2(a.b, row) : make_double2(0.0, 0.0);
		residual_dd<LPR>(a.cols, a.vals64, ks, ke, sub, x, bb, e0, e1);
		if (!ok) e0 = e1 = 0.0;
		return;
	}
	double y0, y1;
	row_product<LPR, double>(a.cols, a.vals, ks, ke, sub, dgather, y0, y1);
	e0 = e1 = 0.0;
	if (ok) {
		if (!a.vals64 && a.corr) {
			float4 const cc = reinterpret_cast<const float4*>(a.corr)[row];
			y0 += (double) cc.x * xi.x + (double) cc.y * xi.y;
			y1 += (double) cc.z * xi.x + (double) cc.w * xi.y;
		}
		double2 const bb = ld2(a.b, row);
		e0 = bb.x - y0;
		e1 = bb.y - y1;
	}
}

template <int LPR>
__global__ void __launch_bounds__(TPB_K) k_mx_replace(CgArgs<float> a) {
	CgState* st = a.st;
	if (st->done) return;
	double v[2] = {0.0, 0.0};  // (r,r), (r, M r)
	FOR_ROWS(LPR) {
		double e0, e1;
		residual_row<LPR>(a, row_, sub_, e0, e1);
		if (row_ < a.N && sub_ == 0) {
			float const r0 = (float) e0, r1 = (float) e1;
			st2(a.r, row_, r0, r1);
			v[0] += e0 * e0 + e1 * e1;
			if (!a.no_pc) {
				float z0, z1;
				precond_apply(a.dinv, a.block_pc, row_, r0, r1, z0, z1);
				v[1] += (double) r0 * (double) z0 + (double) r1 * (double) z1;
			}
		}
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (!a.no_pc) st->gamma = out[1];  // else the SSOR sweeps (mode 1) set it
		// iterative refinement with restarts: the inner PCG starts afresh from this residual
		if (a.opts.restart) st->beta = 0.0;
		if (true_residual_verdict(st, out[0])) {
			st->done = 1;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
	}
}

// ||b - A_res x||^2 in FP64
template <int LPR, typename V>
__global__ void __launch_bounds__(TPB_K) k_true_residual(CgArgs<V> a) {
	double v[1] = {0.0};
	FOR_ROWS(LPR) {
		double e0, e1;
		residual_row<LPR>(a, row_, sub_, e0, e1);
		if (sub_ == 0) v[0] += e0 * e0 + e1 * e1;
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) a.st->true_res2 = out[0];
}

// ---------------------------------------------------------------- double-float path
// FP64-accurate PCG computed on the FP32 pipe (BFM_GPU_FP64_DF).  GB300 issues
// FP64 at a small fraction of its FP32 rate, and the FP64 SpMV is bound by
// that issue rate, not by memory.  Here every value is an unevaluated sum of
// two floats (hi + lo, about 48 significant bits): the matrix (two FP32
// copies, 32 bytes per block as in FP64), the Krylov vectors and the
// solution; products and sums use error-free transformations (TwoProduct by
// FMA, TwoSum), so the iteration behaves like FP64 CG at memory-bound speed.
// Same single-reduction iteration as the FP64 path (u = M r materialized).

struct dfl {
	float hi, lo;
};

__device__ __forceinline__ dfl df_make(double v) {
	float const h = (float) v;
	return {h, (float) (v - (double) h)};
}
__device__ __forceinline__ double df_dbl(dfl a) { return (double) a.hi + (double) a.lo; }

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
	float const s = __fadd_rn(a.hi, b.hi);
	float const bb = __fsub_rn(s, a.hi);
	float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
	e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
	float const h = __fadd_rn(s, e);
	return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
	float const p = __fmul_rn(a.hi, b.hi);
	float e = __fmaf_rn(a.hi, b.hi, -p);
	e = __fmaf_rn(a.hi, b.lo, e);
	e = __fmaf_rn(a.lo, b.hi, e);
	float const h = __fadd_rn(p, e);
	return {h, __fsub_rn(e, __fsub_rn(h, p))};
}
// a*b + c
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) { return df_add(df_mul(a, b), c); }



// node vector element: (u_hi, v_hi, u_lo, v_lo) in one float4
__device__ __forceinline__ void df_ld(const float* v, int i, dfl& a, dfl& b) {
	float4 const t = reinterpret_cast<const float4*>(v)[i];
	a = {t.x, t.z};
	b = {t.y, t.w};
}
__device__ __forceinline__ void df_st(float* v, int i, dfl a, dfl b) {
	reinterpret_cast<float4*>(v)[i] = make_float4(a.hi, b.hi, a.lo, b.lo);
}

// z = M r in double-float: Jacobi (one float4 per node) or a 2x2 block (two)
__device__ __forceinline__ void df_precond(const float* dinv, int block, int i, dfl r0, dfl r1, dfl& z0, dfl& z1) {
	if (block) {
		float4 const h = reinterpret_cast<const float4*>(dinv)[2 * i];
		float4 const l = reinterpret_cast<const float4*>(dinv)[2 * i + 1];
		z0 = df_add(df_mul({h.x, l.x}, r0), df_mul({h.y, l.y}, r1));
		z1 = df_add(df_mul({h.z, l.z}, r0), df_mul({h.w, l.w}, r1));
	}
	else {
		dfl d0, d1;
		df_ld(dinv, i, d0, d1);
		z0 = df_mul(d0, r0);
		z1 = df_mul(d1, r1);
	}
}

struct DfArgs {
	int N;
	const int* row_ptr;
	const int* cols;
	const float* hi;    // 2x2 blocks, FP32 rounding of the FP64 value
	const float* lo;    // FP32 rounding of the remainder
	const float* srow;  // per node: FP64 block row sum of the matrix as a df pair (4 hi, then 4 lo)
	const double* vals64;  // the FP64 matrix, for the replacement residuals
	const float* dinv;  // per node, df pair layout: Jacobi (u_hi, v_hi, u_lo, v_lo); block (4 hi, 4 lo)
	int block_pc;
	const double* b;
	float* x;           // df solution update since the last flush (grouped, like the mixed path's dx)
	double* x64;        // the FP64 solution: every flush adds the update in FP64
	float* r;
	float* u;
	float* p;
	float* s;
	float* w;
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgOpts opts;
	cudaGraphConditionalHandle cond;
	cudaGraphConditionalHandle cond_repl;
	int use_cond;
	int timing;
	int no_pc;  // the SSOR sweeps form z = M r and gamma after this kernel
};

__global__ void __launch_bounds__(TPB_K) k_df_init(DfArgs a) {
	double v[2] = {0.0, 0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const bb = ld2(a.b, i);
		dfl const r0 = df_make(bb.x), r1 = df_make(bb.y);
		dfl u0 = {0.f, 0.f}, u1 = {0.f, 0.f};
		if (!a.no_pc) df_precond(a.dinv, a.block_pc, i, r0, r1, u0, u1);
		dfl const z = {0.f, 0.f};
		df_st(a.x, i, z, z);
		st2(a.x64, i, 0.0, 0.0);
		df_st(a.r, i, r0, r1);
		df_st(a.u, i, u0, u1);
		df_st(a.p, i, z, z);
		df_st(a.s, i, z, z);
		v[0] += bb.x * bb.x + bb.y * bb.y;
		v[1] += df_dbl(df_add(df_mul(r0, u0), df_mul(r1, u1)));
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		CgState* st = a.st;
		st->bnorm2 = out[0];
		st->gamma = out[1];
		st->rtol = a.opts.rtol;
		st->drop2 = a.opts.drop2;
		st->max_iters = a.opts.max_iters;
		st->iter = 0;
		st->replacements = 0;
		st->stall = 0;
		st->best_true2 = out[0];
		st->status = BFM_GPU_OK;
		st->done = out[0] == 0.0;
		st->gamma_old = 0; st->alpha_old = 0;
		st->alpha = 0; st->beta = 0;
		st->rho = out[0];
		st->rho_ref = out[0];
		st->true_res2 = out[0];
		st->ssor_err = 0;
		st->repl_req = 0;
		if (a.use_cond) cudaGraphSetConditional(a.cond, st->done ? 0u : 1u);
	}
}

// x64 += dx in FP64, dx = 0: before every FP64 residual and at the end.  The
// update since the last flush is small next to x, so its 48 bits are plenty,
// while x itself keeps FP64's 53 (a 48-bit x would put its rounding, times
// the stiffness, into every true residual).
__global__ void k_df_flush(DfArgs a) {
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		dfl x0, x1;
		df_ld(a.x, i, x0, x1);
		double2 const x = ld2(a.x64, i);
		st2(a.x64, i, x.x + df_dbl(x0), x.y + df_dbl(x1));
		dfl const z = {0.f, 0.f};
		df_st(a.x, i, z, z);
	}
}

// FP64 preconditioner (Jacobi: 2 per node; block: 4 per node) in double-float layout
// the FP32 halves of the double-float relaxation blocks packed 16 bytes per
// node for the SSOR sweeps, which use no low halves (read in place they
// would take every other 16 bytes of 32-byte sectors)
__global__ void k_pack_hi(int N, const float4* __restrict__ dinv, float4* __restrict__ out) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < N) out[i] = dinv[2 * i];
}

__global__ void k_df_dinv(int N, const double* __restrict__ dinv64, float* __restrict__ dinv, int block) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	if (!block) {
		df_st(dinv, i, df_make(dinv64[2 * i]), df_make(dinv64[2 * i + 1]));
		return;
	}
	dfl m[4];
	for (int k = 0; k < 4; k++) m[k] = df_make(dinv64[4 * i + k]);
	reinterpret_cast<float4*>(dinv)[2 * i] = make_float4(m[0].hi, m[1].hi, m[2].hi, m[3].hi);
	reinterpret_cast<float4*>(dinv)[2 * i + 1] = make_float4(m[0].lo, m[1].lo, m[2].lo, m[3].lo);
}

// ---------------------------------------------------------------- Hestenes-Stiefel, FP64 and double-float
// The default iteration of the FP64 and double-float paths: two reductions
// per iteration, A p formed afresh every iteration (no nested recurrences,
// so the recurrence residual tracks the true one), reliable updates through
// an IF node, convergence decided on the true residual only.
//   K1: p' = z + beta p (neighbours formed on the fly, own row stored in the
//       other ping-pong buffer); q = A p'; alpha = gamma / (p', q)
//   K2: x += alpha p'; r -= alpha q; z = M r; gamma' = (r, z), rho = (r, r);
//       beta; request a replacement when rho dropped by `drop` or claims rtol
//   R:  r = b - A x; z = M r; gamma; verdict on the true residual
// FP64: vectors double2 per node, z materialized so a neighbour costs 2 FMAs
// on top of the SpMV's 4.  Double-float: pairs of floats, FP32 pipe only.

// shared K1 finisher: alpha from (p', q); breakdown if not positive
__device__ __forceinline__ void hs_alpha(CgState* st, double pq, int timing, int use_cond,
                                         cudaGraphConditionalHandle cond) {
	if (!(pq > 0.0)) {
		if (!timing) {
			st->done = 1;
			st->status = BFM_GPU_BREAKDOWN;
		}
		return;
	}
	st->alpha = st->gamma / pq;
	if (use_cond && !timing) cudaGraphSetConditional(cond, 1u);
}

// shared K2 finisher: beta, max_iters, breakdown, replacement request
__device__ __forceinline__ void hs_beta(CgState* st, double gamma, double rho, int timing, int use_cond,
                                        cudaGraphConditionalHandle cond, cudaGraphConditionalHandle cond_repl) {
	if (timing) return;
	double const tol2 = st->rtol * st->rtol * st->bnorm2;
	st->rho = rho;
	st->iter += 1;
	st->beta = gamma / st->gamma;
	st->gamma = gamma;
	int stop = 0, repl = 0;
	if (st->iter >= st->max_iters) {
		stop = 1;
		st->status = BFM_GPU_NOT_CONVERGED;
	}
	else if (!(gamma > 0.0)) {
		repl = gamma == 0.0;
		if (!repl) {
			stop = 1;
			st->status = BFM_GPU_BREAKDOWN;
		}
	}
	else {
		repl = rho <= st->drop2 * st->rho_ref || rho <= tol2;
	}
	if (stop) {
		st->done = 1;
		if (use_cond) cudaGraphSetConditional(cond, 0u);
	}
	else if (repl && use_cond) {
		cudaGraphSetConditional(cond_repl, 1u);
	}
	// launched from a host loop (no conditional nodes): the replacement
	// kernel, launched after every K2, reads the request from the state
	if (!use_cond) st->repl_req = repl && !stop;
}

template <int LPR, int NB = 1>
__global__ void __launch_bounds__(TPB_K) k_hs64_spmv(CgArgs<double> a) {
	CgState* st = a.st;
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	double const beta = st->beta;
	const double* __restrict__ z = a.u;
	const double* __restrict__ pp = a.p;
	auto gather = [=](int c, double& g0, double& g1) {
		double2 const zc = ld2(z, c), pc = ld2(pp, c);
		g0 = zc.x + beta * pc.x;
		g1 = zc.y + beta * pc.y;
	};
	double v[1] = {0.0};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		double y0, y1;
		row_product_nb<LPR, NB, double>(a.cols, a.vals, ks, ke, sub_, gather, y0, y1);
		if (ok && sub_ == 0) {
			double g0, g1;
			gather(row_, g0, g1);
			st2(a.pn, row_, g0, g1);
			st2(a.w, row_, y0, y1);
			v[0] += g0 * y0 + g1 * y1;
		}
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) hs_alpha(st, out[0], a.timing, a.use_cond, a.cond);
}

__global__ void __launch_bounds__(TPB_K) k_hs64_update(CgArgs<double> a) {
	CgState* st = a.st;
	if (st->done && !a.timing) return;
	double const alpha = st->alpha;
	double v[2] = {0.0, 0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const pn = ld2(a.pn, i), q = ld2(a.w, i), r = ld2(a.r, i), x = ld2(a.x, i);
		st2(a.x, i, x.x + alpha * pn.x, x.y + alpha * pn.y);
		double const r0 = r.x - alpha * q.x, r1 = r.y - alpha * q.y;
		st2(a.r, i, r0, r1);
		if (!a.no_pc) {
			double z0, z1;
			precond_apply(a.dinv, a.block_pc, i, r0, r1, z0, z1);
			st2(a.u, i, z0, z1);
			v[0] += r0 * z0 + r1 * z1;
		}
		v[1] += r0 * r0 + r1 * r1;
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (a.no_pc) hs_rho(st, out[1], a.timing, a.use_cond, a.cond, a.cond_repl);
		else hs_beta(st, out[0], out[1], a.timing, a.use_cond, a.cond, a.cond_repl);
	}
}

template <int LPR>
__global__ void __launch_bounds__(TPB_K) k_hs64_replace(CgArgs<double> a) {
	CgState* st = a.st;
	if (st->done) return;
	// outside a graph this kernel follows every K2 and works only on request
	if (!a.use_cond && !st->repl_req) return;
	double v[2] = {0.0, 0.0};
	const double* __restrict__ x = a.x;
	auto gx = [x](int c, double& g0, double& g1) {
		double2 const t = ld2(x, c);
		g0 = t.x;
		g1 = t.y;
	};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		double r0, r1;
		residual_dd<LPR>(a.cols, a.vals, ks, ke, sub_, x, ok ? ld2(a.b, row_) : make_double2(0.0, 0.0), r0, r1);
		if (ok && sub_ == 0) {
			st2(a.r, row_, r0, r1);
			v[0] += r0 * r0 + r1 * r1;
			if (!a.no_pc) {
				double z0, z1;
				precond_apply(a.dinv, a.block_pc, row_, r0, r1, z0, z1);
				st2(a.u, row_, z0, z1);
				v[1] += r0 * z0 + r1 * z1;
			}
		}
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		st->repl_req = 0;
		if (!a.no_pc) st->gamma = out[1];
		if (true_residual_verdict(st, out[0])) {
			st->done = 1;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
	}
}

// ---- double-float HS kernels: x, r, z (in u), p, p' (in s), q (in w)
// Difference form of the double-float SpMV:
//     (A g)_r = S_r g_r + sum_c A_rc (g_c - g_r),
// S_r the node's block row sum taken from the FP64 matrix.  The stored values
// hold 48 of the FP64 values' 53 bits; applied directly that 48-bit operator
// costs about 13-40% more CG iterations on the perforated plates, applied in
// this form (exact row sums, and small exact differences for smooth g) it
// converges like FP64.
__device__ __forceinline__ void df_srow(const float* srow, int r, dfl g0, dfl g1, dfl& y0, dfl& y1) {
	float4 const h = reinterpret_cast<const float4*>(srow)[2 * r];
	float4 const l = reinterpret_cast<const float4*>(srow)[2 * r + 1];
	y0 = df_fma({h.x, l.x}, g0, y0);
	y0 = df_fma({h.y, l.y}, g1, y0);
	y1 = df_fma({h.z, l.z}, g0, y1);
	y1 = df_fma({h.w, l.w}, g1, y1);
}

template <int LPR, int NB = 1>
__global__ void __launch_bounds__(TPB_K) k_hsdf_spmv(DfArgs a) {
	CgState* st = a.st;
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	dfl const beta = df_make(st->beta);
	dfl dot = {0.f, 0.f};  // per-thread double-float sum of (p', q)
	int const sub = threadIdx.x % LPR;
	int const rpb = blockDim.x / LPR;
	for (int base = blockIdx.x * rpb; base < a.N; base += gridDim.x * rpb) {
		int const row = base + threadIdx.x / LPR;
		bool const ok = row < a.N;
		int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
		dfl gr0 = {0.f, 0.f}, gr1 = {0.f, 0.f};
		if (ok) {
			dfl z0, z1, p0, p1;
			df_ld(a.u, row, z0, z1);
			df_ld(a.p, row, p0, p1);
			gr0 = df_fma(beta, p0, z0);
			gr1 = df_fma(beta, p1, z1);
		}
		dfl const ng0 = df_neg(gr0), ng1 = df_neg(gr1);
		dfl y0 = {0.f, 0.f}, y1 = {0.f, 0.f};
		for (int k0 = ks + sub; k0 < ke; k0 += LPR * NB) {
			// NB entries per trip: indices, then gathers and block loads, then arithmetic
			int c[NB];
#pragma unroll
			for (int j = 0; j < NB; j++) c[j] = k0 + j * LPR < ke ? a.cols[k0 + j * LPR] : -1;
			float4 zv[NB], pv[NB], h[NB], l[NB];
#pragma unroll
			for (int j = 0; j < NB; j++) {
				zv[j] = pv[j] = h[j] = l[j] = make_float4(0.f, 0.f, 0.f, 0.f);
				if (c[j] >= 0) {
					zv[j] = reinterpret_cast<const float4*>(a.u)[c[j]];
					pv[j] = reinterpret_cast<const float4*>(a.p)[c[j]];
					h[j] = reinterpret_cast<const float4*>(a.hi)[k0 + j * LPR];
					l[j] = reinterpret_cast<const float4*>(a.lo)[k0 + j * LPR];
				}
			}
#pragma unroll
			for (int j = 0; j < NB; j++) {
				if (c[j] < 0) continue;
				dfl const g0 = df_add(df_fma(beta, {pv[j].x, pv[j].z}, {zv[j].x, zv[j].z}), ng0);
				dfl const g1 = df_add(df_fma(beta, {pv[j].y, pv[j].w}, {zv[j].y, zv[j].w}), ng1);
				y0 = df_fma({h[j].x, l[j].x}, g0, y0);
				y0 = df_fma({h[j].y, l[j].y}, g1, y0);
				y1 = df_fma({h[j].z, l[j].z}, g0, y1);
				y1 = df_fma({h[j].w, l[j].w}, g1, y1);
			}
		}
#pragma unroll
		for (int o = LPR / 2; o; o >>= 1) {
			y0 = df_add(y0, {__shfl_xor_sync(0xffffffffu, y0.hi, o), __shfl_xor_sync(0xffffffffu, y0.lo, o)});
			y1 = df_add(y1, {__shfl_xor_sync(0xffffffffu, y1.hi, o), __shfl_xor_sync(0xffffffffu, y1.lo, o)});
		}
		if (ok && sub == 0) {
			df_srow(a.srow, row, gr0, gr1, y0, y1);
			df_st(a.s, row, gr0, gr1);
			df_st(a.w, row, y0, y1);
			dot = df_add(dot, df_add(df_mul(gr0, y0), df_mul(gr1, y1)));
		}
	}
	double v[1] = {df_dbl(dot)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) hs_alpha(st, out[0], a.timing, a.use_cond, a.cond);
}

__global__ void __launch_bounds__(TPB_K) k_hsdf_update(DfArgs a) {
	CgState* st = a.st;
	if (st->done && !a.timing) return;
	dfl const alpha = df_make(st->alpha), nalpha = df_neg(alpha);
	// per-thread double-float sums, one FP64 conversion per thread (FP64 is scarce on GB300)
	dfl d0 = {0.f, 0.f}, d1 = {0.f, 0.f};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		dfl pn0, pn1, q0, q1, r0, r1, x0, x1;
		df_ld(a.s, i, pn0, pn1);
		df_ld(a.w, i, q0, q1);
		df_ld(a.r, i, r0, r1);
		df_ld(a.x, i, x0, x1);
		df_st(a.x, i, df_fma(alpha, pn0, x0), df_fma(alpha, pn1, x1));
		r0 = df_fma(nalpha, q0, r0);
		r1 = df_fma(nalpha, q1, r1);
		df_st(a.r, i, r0, r1);
		if (!a.no_pc) {
			dfl z0, z1;
			df_precond(a.dinv, a.block_pc, i, r0, r1, z0, z1);
			df_st(a.u, i, z0, z1);
			d0 = df_add(d0, df_add(df_mul(r0, z0), df_mul(r1, z1)));
		}
		d1 = df_add(d1, df_add(df_mul(r0, r0), df_mul(r1, r1)));
	}
	double v[2] = {df_dbl(d0), df_dbl(d1)};
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (a.no_pc) hs_rho(st, out[1], a.timing, a.use_cond, a.cond, a.cond_repl);
		else hs_beta(st, out[0], out[1], a.timing, a.use_cond, a.cond, a.cond_repl);
	}
}

// Replacement of the double-float path: the true residual in FP64 from the
// FP64 matrix (the rare FP64 SpMV sets the attainable accuracy; the
// iteration itself stays on the FP32 pipe), r and z = M r back in pairs.
template <int LPR>
__global__ void __launch_bounds__(TPB_K) k_hsdf_replace(DfArgs a) {
	CgState* st = a.st;
	if (st->done) return;
	double v[2] = {0.0, 0.0};
	int const sub = threadIdx.x % LPR;
	int const rpb = blockDim.x / LPR;
	const double* __restrict__ x64 = a.x64;  // flushed just before
	auto gx = [x64](int c, double& g0, double& g1) {
		double2 const t = ld2(x64, c);
		g0 = t.x;
		g1 = t.y;
	};
	for (int base = blockIdx.x * rpb; base < a.N; base += gridDim.x * rpb) {
		int const row = base + threadIdx.x / LPR;
		bool const ok = row < a.N;
		int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
		double e0, e1;
		residual_dd<LPR>(a.cols, a.vals64, ks, ke, sub, x64, ok ? ld2(a.b, row) : make_double2(0.0, 0.0), e0, e1);
		if (ok && sub == 0) {
			dfl const r0 = df_make(e0), r1 = df_make(e1);
			df_st(a.r, row, r0, r1);
			v[0] += e0 * e0 + e1 * e1;
			if (!a.no_pc) {
				dfl z0, z1;
				df_precond(a.dinv, a.block_pc, row, r0, r1, z0, z1);
				df_st(a.u, row, z0, z1);
				v[1] += df_dbl(df_add(df_mul(r0, z0), df_mul(r1, z1)));
			}
		}
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (!a.no_pc) st->gamma = out[1];
		if (true_residual_verdict(st, out[0])) {
			st->done = 1;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
	}
}

// ---- split form of K1: a direction kernel forms p' = z + beta p for every
// node (and clears the graph's conditions), then the SpMV gathers p' alone:
// one gathered vector instead of two and no direction arithmetic per
// neighbour (FP64: 4 DFMA per block instead of 6).
__global__ void __launch_bounds__(TPB_K) k_hs64_dir(CgArgs<double> a) {
	CgState* st = a.st;
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	double const beta = st->beta;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const z = ld2(a.u, i), p = ld2(a.p, i);
		st2(a.pn, i, z.x + beta * p.x, z.y + beta * p.y);
	}
}

template <int LPR, int NB = 1>
__global__ void __launch_bounds__(TPB_K) k_hs64_spmv_s(CgArgs<double> a) {
	CgState* st = a.st;
	if (st->done && !a.timing) return;
	const double* __restrict__ pn = a.pn;
	auto gather = [=](int c, double& g0, double& g1) {
		double2 const t = ld2(pn, c);
		g0 = t.x;
		g1 = t.y;
	};
	double v[1] = {0.0};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		double y0, y1;
		row_product_nb<LPR, NB, double>(a.cols, a.vals, ks, ke, sub_, gather, y0, y1);
		if (ok && sub_ == 0) {
			double2 const g = ld2(pn, row_);
			st2(a.w, row_, y0, y1);
			v[0] += g.x * y0 + g.y * y1;
		}
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) hs_alpha(st, out[0], a.timing, a.use_cond, a.cond);
}

__global__ void __launch_bounds__(TPB_K) k_hsdf_dir(DfArgs a) {
	CgState* st = a.st;
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	dfl const beta = df_make(st->beta);
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		dfl z0, z1, p0, p1;
		df_ld(a.u, i, z0, z1);
		df_ld(a.p, i, p0, p1);
		df_st(a.s, i, df_fma(beta, p0, z0), df_fma(beta, p1, z1));
	}
}

template <int LPR, int NB = 1>
__global__ void __launch_bounds__(TPB_K) k_hsdf_spmv_s(DfArgs a) {
	CgState* st = a.st;
	if (st->done && !a.timing) return;
	dfl dot = {0.f, 0.f};  // per-thread double-float sum of (p', q)
	int const sub = threadIdx.x % LPR;
	int const rpb = blockDim.x / LPR;
	for (int base = blockIdx.x * rpb; base < a.N; base += gridDim.x * rpb) {
		int const row = base + threadIdx.x / LPR;
		bool const ok = row < a.N;
		int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
		dfl gr0 = {0.f, 0.f}, gr1 = {0.f, 0.f};
		if (ok) df_ld(a.s, row, gr0, gr1);
		dfl const ng0 = df_neg(gr0), ng1 = df_neg(gr1);
		dfl y0 = {0.f, 0.f}, y1 = {0.f, 0.f};
		for (int k0 = ks + sub; k0 < ke; k0 += LPR * NB) {
			int c[NB];
#pragma unroll
			for (int j = 0; j < NB; j++) c[j] = k0 + j * LPR < ke ? a.cols[k0 + j * LPR] : -1;
			float4 gv[NB], h[NB], l[NB];
#pragma unroll
			for (int j = 0; j < NB; j++) {
				gv[j] = h[j] = l[j] = make_float4(0.f, 0.f, 0.f, 0.f);
				if (c[j] >= 0) {
					gv[j] = reinterpret_cast<const float4*>(a.s)[c[j]];
					h[j] = reinterpret_cast<const float4*>(a.hi)[k0 + j * LPR];
					l[j] = reinterpret_cast<const float4*>(a.lo)[k0 + j * LPR];
				}
			}
#pragma unroll
			for (int j = 0; j < NB; j++) {
				if (c[j] < 0) continue;
				dfl const g0 = df_add({gv[j].x, gv[j].z}, ng0), g1 = df_add({gv[j].y, gv[j].w}, ng1);
				y0 = df_fma({h[j].x, l[j].x}, g0, y0);
				y0 = df_fma({h[j].y, l[j].y}, g1, y0);
				y1 = df_fma({h[j].z, l[j].z}, g0, y1);
				y1 = df_fma({h[j].w, l[j].w}, g1, y1);
			}
		}
#pragma unroll
		for (int o = LPR / 2; o; o >>= 1) {
			y0 = df_add(y0, {__shfl_xor_sync(0xffffffffu, y0.hi, o), __shfl_xor_sync(0xffffffffu, y0.lo, o)});
			y1 = df_add(y1, {__shfl_xor_sync(0xffffffffu, y1.hi, o), __shfl_xor_sync(0xffffffffu, y1.lo, o)});
		}
		if (ok && sub == 0) {
			df_srow(a.srow, row, gr0, gr1, y0, y1);
			df_st(a.w, row, y0, y1);
			dot = df_add(dot, df_add(df_mul(gr0, y0), df_mul(gr1, y1)));
		}
	}
	double v[1] = {df_dbl(dot)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) hs_alpha(st, out[0], a.timing, a.use_cond, a.cond);
}

// ---- precision switch: double-float iterations, then an FP64 tail
// The double-float recurrence tracks FP64 PCG's residual history to about
// 1e-7 on the perforated plates, then its attainable accuracy levels off near
// 1e-8.  So the double-float loop stops at a looser tolerance, and this
// kernel hands its state to FP64 HS-PCG without a restart: the latest
// direction converted to FP64 (into the FP64 loop's first direction buffer),
// r = b - A x in FP64 from the flushed solution, z = M r, gamma, and the
// final tolerance.  beta stays from the last double-float step, exactly as
// after a residual replacement.  A stagnated double-float loop continues in
// FP64; a breakdown or the iteration cap ends the solve.
__global__ void __launch_bounds__(TPB_K) k_df_switch(CgArgs<double> a, const float* __restrict__ dir_a,
                                                      const float* __restrict__ dir_b, double rtol_final) {
	CgState* st = a.st;
	bool const go = st->iter > 0 && (st->status == BFM_GPU_OK || st->status == BFM_GPU_STAGNATED);
	if (!go) {
		if (blockIdx.x == 0 && threadIdx.x == 0 && a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		return;
	}
	// K1 of half (iter - 1) % 2 wrote the latest direction: half 0 into dir_a, half 1 into dir_b
	const float* __restrict__ src = ((st->iter - 1) & 1) ? dir_b : dir_a;
	double v[2] = {0.0, 0.0};
	const double* __restrict__ x = a.x;
	auto gx = [x](int c, double& g0, double& g1) {
		double2 const t = ld2(x, c);
		g0 = t.x;
		g1 = t.y;
	};
	FOR_ROWS(1) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		double r0, r1;
		residual_dd<1>(a.cols, a.vals, ks, ke, sub_, x, ok ? ld2(a.b, row_) : make_double2(0.0, 0.0), r0, r1);
		if (ok) {
			dfl p0, p1;
			df_ld(src, row_, p0, p1);
			st2(a.p, row_, df_dbl(p0), df_dbl(p1));  // same 16 bytes per node when src is a.p
			st2(a.r, row_, r0, r1);
			v[0] += r0 * r0 + r1 * r1;
			if (!a.no_pc) {
				double z0, z1;
				precond_apply(a.dinv, a.block_pc, row_, r0, r1, z0, z1);
				st2(a.u, row_, z0, z1);
				v[1] += r0 * z0 + r1 * z1;
			}
		}
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		if (!a.no_pc) st->gamma = out[1];
		st->rtol = rtol_final;
		st->status = BFM_GPU_OK;
		st->done = 0;
		st->stall = 0;
		st->best_true2 = 1e300;  // a fresh start for the stagnation test
		st->done = true_residual_verdict(st, out[0]);
		if (a.use_cond) cudaGraphSetConditional(a.cond, st->done ? 0u : 1u);
	}
}

// ---------------------------------------------------------------- multicolour block SSOR
// z = M^-1 r with M = (D~ + L) D~^-1 (D~ + U): A = L + D + U in the
// colour-major node order (L: blocks of lower-colour neighbours, U: higher),
// D~ the 2x2 relaxation blocks (the diagonal blocks, or the network's).
//   forward, colours 0 .. nc-1:   y_i = D~_i^-1 (r_i - sum_L A_ij y_j)
//   backward, colours nc-2 .. 0:  z_i = y_i - D~_i^-1 sum_U A_ij z_j
// (the backward solve of (D~ + U) z = D~ y, written without D~ itself; the
// last colour has no U neighbours, so its z is its y).  Nodes of one colour
// share no element, so each colour is one parallel phase.  The blocks and
// D~^-1 are read in FP32 (rounding them only moves M a little, and M stays
// fixed), but the vectors and sums are double-float: FP32 rounding there
// makes M^-1 r vary from one application to the next at the 1e-7 level, which
// cost the perforated plates half again as many CG iterations at 1e-10.  y is
// overwritten by z colour by colour.  Every phase that finishes rows adds
// their (r, z) to the state; the last phase turns the sum into beta and
// gamma (after an update) or gamma (after a replacement).

struct CoarseArgs {
	int na, nc;               // aggregates (cells), coarse DOFs (3 na)
	int gx, gy, xfast;        // cell grid; cell (cx, cy) is cx + gx cy when xfast, else cy + gy cx
	int bw;                   // half-bandwidth of A_c
	const int* agg_ptr;       // nodes of aggregate I: agg_nodes[agg_ptr[I] .. agg_ptr[I + 1]), ascending
	const int* agg_nodes;
	const int* agg;
	const float4* pnode;
	float2* band;             // A_c, then L in place (double-float pairs): entry (i, i - t) at band[i (bw + 1) + t], 1 / L_ii on the diagonal
	double* diag0;            // A_c's diagonal (the pivot test)
	float* xl;                // X = L^-1 by rows: row i (columns 0..i) at xrow(i), rows padded to 4 floats
	float* xu;                // X^T by rows: row j (columns j..nc-1) at xrow(nc - 1 - j)
	float2* rc;               // P^T r          (double-float pairs, 4 zero pads after the last)
	float2* yt;               // X rc           (the same)
	float2* yc;               // X^T X rc
	const void* r;
	int df;                   // layout of r: VT_F64 (double2 per node), VT_DF (float4) or VT_F32 (float2)
	const int* row_ptr;
	const int* cols;
	const double* vals64;     // the operator A_c is formed from: FP64 blocks, or (nullptr)
	const float* vals32;      // the FP32 blocks in difference form with the row-sum blocks
	const float* corr32;      // corr32 (the MIXED precision)
	int* err;
	unsigned* bar;       // grid barrier words of the one-launch form (k_coarse_apply)
	int* berr;           // its timeout flag
	long polls;          // polls per grid barrier before it gives up
	// chunks of at most COARSE_CHUNK nodes of one aggregate: chunk q covers
	// agg_nodes[chunk_start[q] .. chunk_start[q + 1]) of aggregate chunk_agg[q];
	// the chunks of aggregate I are [agg_chunk[I], agg_chunk[I + 1])
	int nchunk;
	const int* chunk_start;
	const int* chunk_agg;
	const int* agg_chunk;
	double* part;        // per chunk: 3 (restriction) or 81 (coarse matrix) partial sums
	// the triangular products' work list of the TMA sweep kernel (built for
	// a grid of tri_g blocks; tri_g 0: none): block b's segments
	// tri_seg[tri_sp[b] .. tri_sp[b + 1]) as (row, first entry, entries,
	// slot), its rows tri_row[tri_rp[b] .. tri_rp[b + 1]) as (row, first
	// slot, slots, 0)
	int tri_g;
	int tables;          // 0: the TMA sweep kernel's fallbacks (per-warp rows of X, global restriction arrays)
	const int* tri_sp;
	const int* tri_rp;
	const int4* tri_seg;
	const int4* tri_row;
};

constexpr int TRI_SEG = 512;    // entries of a triangle row per segment (4 groups per lane)
constexpr int TRI_SLOTS = 128;  // segment sums a block holds in shared memory

struct SsorArgs {
	const int* row_ptr;
	const int* cols;
	const int* dpos;    // per row: first block at or after the diagonal
	const float* hi;    // FP32 2x2 blocks
	const float* dinv;  // FP32 relaxation block inverses, 16 bytes per node (k_pack_hi)
	const void* r;      // residual: double-float float4 (u_hi, v_hi, u_lo, v_lo) or FP64 double2 per node
	void* z;            // z = M^-1 r, same layout
	float* y;           // double-float float4 per node
	double* partials;
	unsigned* ticket;
	CgState* st;
	int lo, hi_row;     // the rows of this phase's colour
	int fwd_last;       // forward phase of the last colour: its z is its y
	int first_acc;      // first phase that finishes rows: (r, z) starts from zero
	int final_phase;    // last phase: beta and gamma
	int mode;           // 0 after an update (beta = gamma' / gamma), 1 after a residual replacement
	cudaGraphConditionalHandle cond, cond_repl;
	int use_cond;
	int timing;
	// persistent form: every phase in one cooperative launch
	unsigned* bar;      // grid barrier: arrivals, generation
	long polls;         // polls per grid barrier before it gives up
	int ncol;
	int off[65];        // colour c: rows [off[c], off[c + 1])
	// two-level form: z += P yc, the coarse correction (yc == nullptr: none)
	const int* agg;      // aggregate of each node
	const float4* pnode; // per node: (dx / H, dy / H, u free, v free)
	const float2* yc;    // A_c^-1 P^T r, double-float pair per coarse DOF
	// the sweeps' blocks, apart from the CSR matrix: sliced ELL over slices
	// of 32 consecutive rows of one colour, the slice's k-th block of row
	// `lane` at [ptr[s] + 32 k + lane] (padding: column -1), so a warp reads
	// 32 consecutive blocks per step.  Lower-colour blocks (forward sweep) and
	// higher-colour blocks (backward) are kept apart: each phase streams only
	// the blocks it uses, each once.
	const float4* lv;
	const int* lc;
	const int* lp;
	const float4* uv;
	const int* uc;
	const int* up;
	int slice0;          // per-phase kernels: first slice of this phase's colour
	int sbase[65];       // persistent kernel: first slice of colour c
	// persistent kernel, at least 3 colours: the coarse correction's four
	// stages run inside the sweep phases (restriction, chunk sums, X rc, X^T yt
	// in phases 0-3, between the sweeps' own grid barriers); the rows
	// finished before the last phase get their P yc term in the last one
	int fuse;
	CoarseArgs co;
	// persistent kernel: at the start of each phase, thread 0 of each block
	// asks the TMA unit to prefetch into L2 what the block's rows read in
	// the next phase and what no phase writes (sliced-ELL blocks and
	// columns, relaxation blocks, the coarse stages' rows of X), so those
	// reads hit L2 after the grid barrier
	int pf;
	// TMA-staged persistent kernel (k_ssor_tma): slices per tile of each
	// phase and the bytes of one ring stage
	int spt[127];
	int stage_bytes;
};


// a * b for a float and a double-float (TwoProduct of the high part)
__device__ __forceinline__ dfl df_mul_f(float a, dfl b) {
	float const p = __fmul_rn(a, b.hi);
	float e = __fmaf_rn(a, b.hi, -p);
	e = __fmaf_rn(a, b.lo, e);
	float const h = __fadd_rn(p, e);
	return {h, __fsub_rn(e, __fsub_rn(h, p))};
}

// D~^-1 (s0, s1) with the FP32 block d
__device__ __forceinline__ void ssor_blk(float4 d, dfl s0, dfl s1, dfl& o0, dfl& o1) {
	o0 = df_add(df_mul_f(d.x, s0), df_mul_f(d.y, s1));
	o1 = df_add(df_mul_f(d.z, s0), df_mul_f(d.w, s1));
}

// sum of A_ij y_j over the sliced-ELL blocks of row `lane` of slice s, y
// double-float float4 per node (written by other blocks of the persistent
// kernel: read past L1).  SSOR_CHUNK blocks at a time: their column indices
// and values are loaded together, then their gathers.  The slice's width is
// the same for the whole warp.
constexpr int SSOR_CHUNK = 2;  // with 8 resident blocks per SM (32 registers)

__device__ __forceinline__ void sell_row(const float4* __restrict__ v, const int* __restrict__ cidx,
                                         const int* __restrict__ ptr, int s, int lane, const float* y, dfl& t0, dfl& t1) {
	int const k0 = ptr[s] + lane, w = (ptr[s + 1] - ptr[s]) >> 5;
	for (int kb = 0; kb < w; kb += SSOR_CHUNK) {
		int c[SSOR_CHUNK];
		float4 m[SSOR_CHUNK];
#pragma unroll
		for (int j = 0; j < SSOR_CHUNK; j++) {
			bool const in = kb + j < w;
			int const e = k0 + 32 * (kb + j);
			c[j] = in ? __ldcs(cidx + e) : -1;
			m[j] = in ? __ldcs(v + e) : make_float4(0.f, 0.f, 0.f, 0.f);
		}
		float4 g[SSOR_CHUNK];
#pragma unroll
		for (int j = 0; j < SSOR_CHUNK; j++)
			g[j] = c[j] >= 0 ? __ldcg(reinterpret_cast<const float4*>(y) + c[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
		for (int j = 0; j < SSOR_CHUNK; j++) {
			dfl const g0 = {g[j].x, g[j].z}, g1 = {g[j].y, g[j].w};
			t0 = df_add(t0, df_add(df_mul_f(m[j].x, g0), df_mul_f(m[j].y, g1)));
			t1 = df_add(t1, df_add(df_mul_f(m[j].z, g0), df_mul_f(m[j].w, g1)));
		}
	}
}

// vector layouts of the residual r and z = M^-1 r the sweeps read and write
enum : int {
	VT_F64 = 0,  // double2 per node (FP64 path)
	VT_DF = 1,   // double-float float4 per node (u_hi, v_hi, u_lo, v_lo)
	VT_F32 = 2,  // float2 per node (mixed path); the sweeps still sum in double-float
};

template <int VT>
__device__ __forceinline__ void ssor_ld_r(const void* r, int i, dfl& r0, dfl& r1, double& q0, double& q1) {
	if constexpr (VT == VT_DF) {
		df_ld((const float*) r, i, r0, r1);
	}
	else if constexpr (VT == VT_F32) {
		float2 const t = ld2((const float*) r, i);
		r0 = {t.x, 0.f};
		r1 = {t.y, 0.f};
	}
	else {
		double2 const t = ld2((const double*) r, i);
		q0 = t.x;
		q1 = t.y;
		r0 = df_make(q0);
		r1 = df_make(q1);
	}
}

// the coarse correction of node i, (P yc)_i = [f0 (y0 - dy y2), f1 (y1 + dx y2)]
__device__ __forceinline__ void coarse_term(const int* agg, const float4* pnode, const float2* yc, int i, dfl& c0, dfl& c1) {
	int const I = agg[i];
	float4 const q = pnode[i];
	float2 const a = yc[3 * I], b = yc[3 * I + 1], c = yc[3 * I + 2];
	dfl const y2 = {c.x, c.y};
	c0 = q.z != 0.f ? df_add({a.x, a.y}, df_mul_f(-q.y, y2)) : dfl{0.f, 0.f};
	c1 = q.w != 0.f ? df_add({b.x, b.y}, df_mul_f(q.x, y2)) : dfl{0.f, 0.f};
}

template <int VT>
__device__ __forceinline__ void ssor_st_z(const SsorArgs& a, int i, dfl z0, dfl z1, dfl r0, dfl r1, double q0, double q1,
                                          dfl& acc, double& acc64) {
	if (a.yc) {
		dfl c0, c1;
		coarse_term(a.agg, a.pnode, a.yc, i, c0, c1);
		z0 = df_add(z0, c0);
		z1 = df_add(z1, c1);
	}
	if constexpr (VT == VT_DF) {
		df_st((float*) a.z, i, z0, z1);
		acc = df_add(acc, df_add(df_mul(r0, z0), df_mul(r1, z1)));
	}
	else if constexpr (VT == VT_F32) {
		// (r, z) of the rounded z the iteration will use
		dfl const w0 = {__fadd_rn(z0.hi, z0.lo), 0.f}, w1 = {__fadd_rn(z1.hi, z1.lo), 0.f};
		st2((float*) a.z, i, w0.hi, w1.hi);
		acc = df_add(acc, df_add(df_mul(r0, w0), df_mul(r1, w1)));
	}
	else {
		double const w0 = df_dbl(z0), w1 = df_dbl(z1);
		st2((double*) a.z, i, w0, w1);
		acc64 += q0 * w0 + q1 * w1;
	}
}

// store z without the coarse term (fused two-level form, before yc exists)
template <int VT>
__device__ __forceinline__ void ssor_st_plain(const SsorArgs& a, int i, dfl z0, dfl z1) {
	if constexpr (VT == VT_DF) df_st((float*) a.z, i, z0, z1);
	else if constexpr (VT == VT_F32) st2((float*) a.z, i, __fadd_rn(z0.hi, z0.lo), __fadd_rn(z1.hi, z1.lo));
	else st2((double*) a.z, i, df_dbl(z0), df_dbl(z1));
}

// z_i += (P yc)_i for a row stored by ssor_st_plain, and its (r, z)
template <int VT>
__device__ __forceinline__ void ssor_add_coarse(const SsorArgs& a, int i, dfl& acc, double& acc64) {
	// z was stored by other blocks in an earlier phase: read it from L2
	dfl z0, z1;
	if constexpr (VT == VT_DF) {
		float4 const t = __ldcg(reinterpret_cast<const float4*>(a.z) + i);
		z0 = {t.x, t.z};
		z1 = {t.y, t.w};
	}
	else if constexpr (VT == VT_F32) {
		float2 const t = __ldcg(reinterpret_cast<const float2*>(a.z) + i);
		z0 = {t.x, 0.f};
		z1 = {t.y, 0.f};
	}
	else {
		double2 const t = __ldcg(reinterpret_cast<const double2*>(a.z) + i);
		z0 = df_make(t.x);
		z1 = df_make(t.y);
	}
	dfl r0, r1;
	double q0 = 0.0, q1 = 0.0;
	ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
	ssor_st_z<VT>(a, i, z0, z1, r0, r1, q0, q1, acc, acc64);
}

__device__ __forceinline__ void ssor_finish(const SsorArgs& a, double part) {
	CgState* st = a.st;
	st->ssor_acc = a.first_acc ? part : st->ssor_acc + part;
	if (!a.final_phase || a.timing) return;
	double const g = st->ssor_acc;
	if (st->ssor_err) {
		st->done = 1;
		st->status = BFM_GPU_TIMEOUT;
		if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		return;
	}
	if (a.mode == 1) {
		st->gamma = g;
		return;
	}
	// as hs_beta: a zero (r, z) asks for a replacement, a negative one is a breakdown
	st->beta = g / st->gamma;
	st->gamma = g;
	if (!(g > 0.0)) {
		if (g == 0.0) {
			if (a.use_cond) cudaGraphSetConditional(a.cond_repl, 1u);
		}
		else {
			st->done = 1;
			st->status = BFM_GPU_BREAKDOWN;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
	}
}

template <int VT>
__global__ void __launch_bounds__(TPB_K) k_ssor_fwd(SsorArgs a) {
	if (a.st->done && !a.timing) return;
	dfl acc = {0.f, 0.f};
	double acc64 = 0.0;
	for (int i = a.lo + blockIdx.x * blockDim.x + threadIdx.x; i < a.hi_row; i += gridDim.x * blockDim.x) {
		dfl r0, r1;
		double q0 = 0.0, q1 = 0.0;
		ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
		dfl t0 = {0.f, 0.f}, t1 = {0.f, 0.f};
		sell_row(a.lv, a.lc, a.lp, a.slice0 + ((i - a.lo) >> 5), (i - a.lo) & 31, a.y, t0, t1);
		dfl y0, y1;
		ssor_blk(reinterpret_cast<const float4*>(a.dinv)[i], df_add(r0, df_neg(t0)), df_add(r1, df_neg(t1)), y0, y1);
		df_st(a.y, i, y0, y1);
		if (a.fwd_last) ssor_st_z<VT>(a, i, y0, y1, r0, r1, q0, q1, acc, acc64);
	}
	if (!a.fwd_last) return;
	double v[1] = {VT == VT_F64 ? acc64 : df_dbl(acc)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) ssor_finish(a, out[0]);
}

template <int VT>
__global__ void __launch_bounds__(TPB_K) k_ssor_bwd(SsorArgs a) {
	if (a.st->done && !a.timing) return;
	dfl acc = {0.f, 0.f};
	double acc64 = 0.0;
	for (int i = a.lo + blockIdx.x * blockDim.x + threadIdx.x; i < a.hi_row; i += gridDim.x * blockDim.x) {
		dfl t0 = {0.f, 0.f}, t1 = {0.f, 0.f};
		sell_row(a.uv, a.uc, a.up, a.slice0 + ((i - a.lo) >> 5), (i - a.lo) & 31, a.y, t0, t1);
		dfl w0, w1, y0, y1;
		ssor_blk(reinterpret_cast<const float4*>(a.dinv)[i], t0, t1, w0, w1);
		df_ld(a.y, i, y0, y1);
		dfl const z0 = df_add(y0, df_neg(w0)), z1 = df_add(y1, df_neg(w1));
		df_st(a.y, i, z0, z1);
		dfl r0, r1;
		double q0 = 0.0, q1 = 0.0;
		ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
		ssor_st_z<VT>(a, i, z0, z1, r0, r1, q0, q1, acc, acc64);
	}
	double v[1] = {VT == VT_F64 ? acc64 : df_dbl(acc)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) ssor_finish(a, out[0]);
}

// Grid barrier of the persistent sweep kernel (cooperative launch: every
// block is resident).  Arrivals count up; the last one resets the count and
// advances the generation the others wait for.  The wait is bounded: past
// the limit (polls per barrier, a kernel argument: bfm_gpu_opts_t's
// barrier_polls, this default when 0) the kernel records the timeout, and
// the blocks stop sweeping.
constexpr long BARRIER_POLLS_DEFAULT = 1l << 24;

// Grid barrier words: the arrival count at word 0 and the generation at word
// 32 (separate 128-byte lines, so the polling does not slow the arrivals)
constexpr int BAR_WORDS = 96;  // count (word 0), generation (32), the TMA sweep kernel's arrival counter (64)

// the generation this block waits past at its next grid barrier
__device__ __forceinline__ unsigned& bar_expect() {
	__shared__ unsigned g;
	return g;
}

// at kernel start, before the first grid_barrier: no block can pass a
// barrier before every block has arrived, so the generation read here is
// the one before the first barrier
__device__ __forceinline__ void grid_barrier_init(unsigned* bar) {
	if (threadIdx.x == 0) {
		unsigned v;
		asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar + 32) : "memory");
		bar_expect() = v;
	}
}

// Grid-wide barrier of a cooperative launch: thread 0 of each block arrives
// with one acquire-release atomic (the block's writes, ordered before it by
// __syncthreads, are released with it); the last to arrive resets the count
// and publishes the next generation with a release store; the others poll it
// with acquire loads.  Bounded: after `polls` polls, or when another block
// has given up (*err, checked every 1024 polls), *err is set and false
// returned.
__device__ bool grid_barrier(unsigned* bar, int* err, long polls) {
	__shared__ int ok;
	__syncthreads();
	if (threadIdx.x == 0) {
		unsigned* count = bar;
		unsigned* gen = bar + 32;
		unsigned const target = bar_expect() + 1;
		int good = 1;
		unsigned old;
		asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(count) : "memory");
		if (old == gridDim.x - 1) {
			asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(count) : "memory");
			asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(gen), "r"(target) : "memory");
		}
		else {
			long spins = 0;
			unsigned cur;
			while (true) {
				asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(gen) : "memory");
				if (cur == target) break;
				++spins;
				if (spins > polls || ((spins & 1023) == 0 && *(volatile int*) err != 0)) {
					atomicExch(err, 1);
					good = 0;
					break;
				}
			}
		}
		bar_expect() = target;
		ok = good;
	}
	__syncthreads();
	return ok;
}

__device__ __forceinline__ bool ssor_barrier(const SsorArgs& a) { return grid_barrier(a.bar, &a.st->ssor_err, a.polls); }

// ---------------------------------------------------------------- coarse space (two-level SSOR)
// M^-1 = M_SSOR^-1 + P A_c^-1 P^T, A_c = P^T A P: one aggregate per cell of a
// grid laid over the mesh's bounding box, three coarse DOFs per aggregate
// (the two translations and the rotation about the cell centre, scaled by
// the cell size H), rows of constrained DOFs zero.  The cells are numbered
// along the grid's shorter side first, so A_c, which couples each cell with
// the 8 around it, is a band matrix of half-width bw = 3 (short side + 1) + 2.
// Its band Cholesky factor L gives X = L^-1 (a dense lower triangle, stored
// in FP32), and the correction is applied as yc = X^T (X P^T r) with
// double-float sums: symmetric positive (semi)definite by construction,
// whatever the rounding of X.  The sweeps add P yc to z when they store it,
// so the recursion itself stays M_SSOR^-1.


constexpr int COARSE_CHUNK = 128;
constexpr int COARSE_MAX_BW = 101;  // widest band: the factorisation's shared window and the solve's registers
constexpr int CHOL_T = 512;         // threads of the factorisation block
constexpr int LINV_C = 2;           // columns per warp of the inversion
constexpr int LINV_L = 32 / LINV_C;  // lanes per column
constexpr int LINV_W = 4;           // warps per block of the inversion

__host__ __device__ __forceinline__ void cell_xy(int I, int gx, int gy, int xfast, int& cx, int& cy) {
	if (xfast) {
		cx = I % gx;
		cy = I / gx;
	}
	else {
		cy = I % gy;
		cx = I / gy;
	}
}
__host__ __device__ __forceinline__ int cell_id(int cx, int cy, int gx, int gy, int xfast) {
	return xfast ? cx + gx * cy : cy + gy * cx;
}
// start of row i of a triangle whose row i has i + 1 entries, each row padded
// to a multiple of 4 floats (16-byte rows): rows 4q .. 4q + 3 take 4 (q + 1) each
__host__ __device__ __forceinline__ long xrow(int i) {
	long const q = i / 4, r = i % 4;
	return 4 * (q + 1) * (2 * q + r);
}

// shared memory of the factorisation (n coarse DOFs): the (bw + 2)^2
// window, the scaled column, the pivot (double-float pairs), the pivots'
// drop thresholds, the update's (row, column) pairs
__host__ __device__ constexpr size_t chol_smem(int bw, int n) {
	return sizeof(float2) * ((size_t) (bw + 2) * (bw + 2) + (bw + 2) + 2) + sizeof(float) * ((size_t) n + 1) +
	       sizeof(short2) * ((size_t) bw * (bw + 1) / 2);
}
// shared memory of the inversion: per warp LINV_C column rings and two staged rows of L
__host__ __device__ constexpr size_t linv_smem(int bw) {
	return sizeof(float2) * LINV_W * ((size_t) LINV_C * (bw + 2) + 2 * (bw + 1));
}

// 1 / sqrt(p) of a double-float pivot above the drop threshold (else 0: a
// dropped DOF): the FP32 estimate y = rsqrtf(p) refined by one
// Newton-Raphson step y + y (1 - p y^2) / 2 in double-float arithmetic
// (quadratic convergence: about 23 -> 46 bits, the width of the pair)
__device__ __forceinline__ dfl pivot_rsqrt(dfl p, float thr) {
	if (!(p.hi > thr)) return {0.f, 0.f};
	float const y = rsqrtf(p.hi);
	float const yy = __fmul_rn(y, y);
	dfl const y2 = {yy, __fmaf_rn(y, y, -yy)};
	dfl const e = df_add({1.f, 0.f}, df_neg(df_mul(p, y2)));
	return df_add({y, 0.f}, df_mul_f(0.5f * y, e));
}

// per node its offset from its cell's centre (scaled by the cell size H) and
// which of its DOFs are free (constrained ones get no coarse correction)
// (the offsets times 1 / H, which the host forms once: two FP64 divisions
// per node cost more than the rest of the kernel on this GPU's FP64 pipe,
// and the offsets are rounded to FP32 anyway)
__global__ void k_pnode(int N, const double* __restrict__ coords, const int* __restrict__ agg, const int* __restrict__ last_ci,
                        double x0, double y0, double cw, double ch, int gx, int gy, int xfast, double invH,
                        float4* __restrict__ pnode) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	int cx, cy;
	cell_xy(agg[i], gx, gy, xfast, cx, cy);
	double const xc = x0 + (cx + 0.5) * cw, yc = y0 + (cy + 0.5) * ch;
	pnode[i] = make_float4((float) ((coords[2l * i] - xc) * invH), (float) ((coords[2l * i + 1] - yc) * invH),
	                       last_ci[2l * i] < 0 ? 1.f : 0.f, last_ci[2l * i + 1] < 0 ? 1.f : 0.f);
}

// rc = P^T r in two deterministic stages: one warp per chunk of an
// aggregate (lane l takes the chunk's nodes l, l + 32, ..: their indices
// first, then their values, then double-float sums in that order and a fixed
// shuffle tree), then per coarse DOF the chunks' sums in chunk order
__device__ __forceinline__ void restrict_chunk(const CoarseArgs& a, int q, int lane) {
	constexpr int PER = COARSE_CHUNK / 32;
	int const k0 = a.chunk_start[q], k1 = a.chunk_start[q + 1];
	int idx[PER];
#pragma unroll
	for (int u = 0; u < PER; u++) {
		int const k = k0 + lane + 32 * u;
		idx[u] = k < k1 ? a.agg_nodes[k] : -1;
	}
	dfl r0[PER], r1[PER];
	float4 pq[PER];
#pragma unroll
	for (int u = 0; u < PER; u++) {
		r0[u] = r1[u] = {0.f, 0.f};
		pq[u] = make_float4(0.f, 0.f, 0.f, 0.f);
		int const i = idx[u];
		if (i < 0) continue;
		if (a.df == VT_DF) df_ld((const float*) a.r, i, r0[u], r1[u]);
		else if (a.df == VT_F32) {
			float2 const t = ld2((const float*) a.r, i);
			r0[u] = {t.x, 0.f};
			r1[u] = {t.y, 0.f};
		}
		else {
			double2 const t = ld2((const double*) a.r, i);
			r0[u] = df_make(t.x);
			r1[u] = df_make(t.y);
		}
		pq[u] = a.pnode[i];
	}
	dfl s0 = {0.f, 0.f}, s1 = {0.f, 0.f}, s2 = {0.f, 0.f};
#pragma unroll
	for (int u = 0; u < PER; u++) {
		if (idx[u] < 0) continue;
		dfl const x0 = pq[u].z == 0.f ? dfl{0.f, 0.f} : r0[u];
		dfl const x1 = pq[u].w == 0.f ? dfl{0.f, 0.f} : r1[u];
		s0 = df_add(s0, x0);
		s1 = df_add(s1, x1);
		s2 = df_add(s2, df_add(df_mul_f(-pq[u].y, x0), df_mul_f(pq[u].x, x1)));
	}
#pragma unroll
	for (int o = 16; o; o >>= 1) {
		s0 = df_add(s0, {__shfl_xor_sync(0xffffffffu, s0.hi, o), __shfl_xor_sync(0xffffffffu, s0.lo, o)});
		s1 = df_add(s1, {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)});
		s2 = df_add(s2, {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)});
	}
	if (lane == 0) {
		a.part[3l * q] = df_dbl(s0);
		a.part[3l * q + 1] = df_dbl(s1);
		a.part[3l * q + 2] = df_dbl(s2);
	}
}

// restrict_chunk with one node in flight per lane (for a kernel with few
// registers): the same sums in the same order
__device__ __forceinline__ void restrict_chunk_lean(const CoarseArgs& a, int q, int lane) {
	int const k0 = a.chunk_start[q], k1 = a.chunk_start[q + 1];
	dfl s0 = {0.f, 0.f}, s1 = {0.f, 0.f}, s2 = {0.f, 0.f};
	for (int k = k0 + lane; k < k1; k += 32) {
		int const i = a.agg_nodes[k];
		dfl r0, r1;
		if (a.df == VT_DF) df_ld((const float*) a.r, i, r0, r1);
		else if (a.df == VT_F32) {
			float2 const t = ld2((const float*) a.r, i);
			r0 = {t.x, 0.f};
			r1 = {t.y, 0.f};
		}
		else {
			double2 const t = ld2((const double*) a.r, i);
			r0 = df_make(t.x);
			r1 = df_make(t.y);
		}
		float4 const pq = a.pnode[i];
		dfl const x0 = pq.z == 0.f ? dfl{0.f, 0.f} : r0;
		dfl const x1 = pq.w == 0.f ? dfl{0.f, 0.f} : r1;
		s0 = df_add(s0, x0);
		s1 = df_add(s1, x1);
		s2 = df_add(s2, df_add(df_mul_f(-pq.y, x0), df_mul_f(pq.x, x1)));
	}
#pragma unroll
	for (int o = 16; o; o >>= 1) {
		s0 = df_add(s0, {__shfl_xor_sync(0xffffffffu, s0.hi, o), __shfl_xor_sync(0xffffffffu, s0.lo, o)});
		s1 = df_add(s1, {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)});
		s2 = df_add(s2, {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)});
	}
	if (lane == 0) {
		a.part[3l * q] = df_dbl(s0);
		a.part[3l * q + 1] = df_dbl(s1);
		a.part[3l * q + 2] = df_dbl(s2);
	}
}

__device__ __forceinline__ void restrict_sum_one(const CoarseArgs& a, int t) {
	int const I = t / 3, m = t % 3;
	double v = 0.0;
	for (int c = a.agg_chunk[I]; c < a.agg_chunk[I + 1]; c++) v += a.part[3l * c + m];
	dfl const d = df_make(v);
	a.rc[t] = make_float2(d.hi, d.lo);
}

__global__ void __launch_bounds__(256) k_restrict(CoarseArgs a) {
	int const q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (q < a.nchunk) restrict_chunk(a, q, lane);
}

__global__ void k_restrict_sum(CoarseArgs a) {
	int const t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < a.nc) restrict_sum_one(a, t);
}

constexpr int CX_T = 256;  // threads per row of the coarse products

// one row of a padded FP32 triangle times a double-float vector, one block:
// thread t takes the 16-byte groups t, t + CX_T, .. (loads first, then
// double-float products and sums), then a fixed shuffle tree per warp and
// the warps' sums in order (deterministic); the result in thread 0
template <int U = 4>  // groups per thread in flight
__device__ __forceinline__ dfl coarse_row_dot(const float* __restrict__ row, int len, const float2* __restrict__ v) {
	__shared__ float2 ws[CX_T / 32];
	int const tx = threadIdx.x, lane = tx & 31, w = tx >> 5;
	dfl s = {0.f, 0.f};
	int const ng = (len + 3) >> 2;
	const float4* r4 = reinterpret_cast<const float4*>(row);
	for (int g0 = tx; g0 < ng; g0 += CX_T * U) {
		float4 x[U];
		float2 vv[U][4];
#pragma unroll
		for (int u = 0; u < U; u++) {
			int const g = g0 + CX_T * u;
			x[u] = g < ng ? __ldg(r4 + g) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
			for (int c = 0; c < 4; c++) vv[u][c] = g < ng ? v[4 * g + c] : make_float2(0.f, 0.f);
		}
#pragma unroll
		for (int u = 0; u < U; u++) {
			if (g0 + CX_T * u >= ng) continue;
			s = df_add(s, df_mul_f(x[u].x, {vv[u][0].x, vv[u][0].y}));
			s = df_add(s, df_mul_f(x[u].y, {vv[u][1].x, vv[u][1].y}));
			s = df_add(s, df_mul_f(x[u].z, {vv[u][2].x, vv[u][2].y}));
			s = df_add(s, df_mul_f(x[u].w, {vv[u][3].x, vv[u][3].y}));
		}
	}
#pragma unroll
	for (int o = 16; o; o >>= 1) s = df_add(s, {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
	if (lane == 0) ws[w] = make_float2(s.hi, s.lo);
	__syncthreads();
	dfl t = {0.f, 0.f};
	if (tx == 0)
		for (int k = 0; k < CX_T / 32; k++) t = df_add(t, {ws[k].x, ws[k].y});
	return t;
}

// yt = X rc: one block per row of X (the padding of a row is zero, and rc has
// zero pads past its end)
__global__ void __launch_bounds__(CX_T) k_coarse_x(CoarseArgs a) {
	int const i = blockIdx.x;
	if (i >= a.nc) return;
	dfl const s = coarse_row_dot(a.xl + xrow(i), i + 1, a.rc);
	if (threadIdx.x == 0) a.yt[i] = make_float2(s.hi, s.lo);
}

// yc = X^T yt, the same way over the rows of X^T (row j starts at column j)
__global__ void __launch_bounds__(CX_T) k_coarse_xt(CoarseArgs a) {
	int const j = blockIdx.x;
	if (j >= a.nc) return;
	dfl const s = coarse_row_dot(a.xu + xrow(a.nc - 1 - j), a.nc - j, a.yt + j);
	if (threadIdx.x == 0) a.yc[j] = make_float2(s.hi, s.lo);
}

// The four stages above in one cooperative launch, grid barriers between
// them (bounded waits: a timeout sets *berr and every block returns), the
// same arithmetic: restriction chunks by warps, chunk sums by threads, the
// two triangular products by blocks (one row at a time)
__global__ void __launch_bounds__(CX_T) k_coarse_apply(CoarseArgs a) {
	int const nw = gridDim.x * (CX_T / 32), wid = blockIdx.x * (CX_T / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
	if (*(volatile int*) a.berr) return;  // an earlier barrier of this solve timed out: the solve has stopped
	grid_barrier_init(a.bar);
	for (int q = wid; q < a.nchunk; q += nw) restrict_chunk(a, q, lane);
	if (!grid_barrier(a.bar, a.berr, a.polls)) return;
	for (int t = blockIdx.x * CX_T + threadIdx.x; t < a.nc; t += gridDim.x * CX_T) restrict_sum_one(a, t);
	if (!grid_barrier(a.bar, a.berr, a.polls)) return;
	for (int i = blockIdx.x; i < a.nc; i += gridDim.x) {
		dfl const s = coarse_row_dot(a.xl + xrow(i), i + 1, a.rc);
		if (threadIdx.x == 0) a.yt[i] = make_float2(s.hi, s.lo);
		__syncthreads();
	}
	if (!grid_barrier(a.bar, a.berr, a.polls)) return;
	for (int j = blockIdx.x; j < a.nc; j += gridDim.x) {
		dfl const s = coarse_row_dot(a.xu + xrow(a.nc - 1 - j), a.nc - j, a.yt + j);
		if (threadIdx.x == 0) a.yc[j] = make_float2(s.hi, s.lo);
		__syncthreads();
	}
}

// bulk prefetch of [p, p + bytes) into L2 (p 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
	if (bytes) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// the inputs of phase ph of k_ssor_all that this block reads and no phase
// writes: the rows it takes (the same grid-stride split as the sweeps, whole
// slices: a block's rows start 32-aligned within the colour), and for the
// fused coarse stages the rows of X and X^T it takes
__device__ void ssor_prefetch_phase(const SsorArgs& a, int ph, int nc, int stride) {
	bool const forward = ph < nc;
	int const c = forward ? ph : 2 * nc - 2 - ph;
	int const lo = a.off[c], hi = a.off[c + 1];
	const float4* v = forward ? a.lv : a.uv;
	const int* ci = forward ? a.lc : a.uc;
	const int* ptr = forward ? a.lp : a.up;
	for (int s0 = lo + blockIdx.x * (int) blockDim.x; s0 < hi; s0 += stride) {
		int const e0 = min(s0 + (int) blockDim.x, hi);
		int const sa = a.sbase[c] + ((s0 - lo) >> 5), sb = a.sbase[c] + ((e0 - lo + 31) >> 5);
		int const k0 = __ldg(ptr + sa), k1 = __ldg(ptr + sb);
		l2_prefetch(v + k0, 16u * (unsigned) (k1 - k0));
		l2_prefetch(ci + k0, 4u * (unsigned) (k1 - k0));
		l2_prefetch(reinterpret_cast<const float4*>(a.dinv) + s0, 16u * (unsigned) (e0 - s0));
	}
	if (!a.fuse) return;
	CoarseArgs const& co = a.co;
	if (ph == 2)
		for (int i = blockIdx.x; i < co.nc; i += gridDim.x) l2_prefetch(co.xl + xrow(i), 4u * (unsigned) ((i + 4) & ~3));
	else if (ph == 3)
		for (int j = blockIdx.x; j < co.nc; j += gridDim.x)
			l2_prefetch(co.xu + xrow(co.nc - 1 - j), 4u * (unsigned) ((co.nc - j + 3) & ~3));
}

template <int VT>
__global__ void __launch_bounds__(TPB_K, 8) k_ssor_all(SsorArgs a) {
	if (a.st->done && !a.timing) return;
	grid_barrier_init(a.bar);
	int const nc = a.ncol > 0 ? a.ncol : 1;
	dfl acc = {0.f, 0.f};
	double acc64 = 0.0;
	bool alive = true;
	int const stride = gridDim.x * blockDim.x, tid = blockIdx.x * blockDim.x + threadIdx.x;
	bool const fuse = a.fuse && nc >= 3;
	for (int ph = 0; ph < 2 * nc - 1 && alive; ph++) {
		bool const forward = ph < nc;
		bool const last = ph == 2 * nc - 2;
		int const c = forward ? ph : 2 * nc - 2 - ph;
		bool const final_rows = !forward || c == nc - 1;
		int const lo = a.off[c], hi = a.off[c + 1];
		if (a.pf && threadIdx.x == 0 && ph + 1 < 2 * nc - 1) ssor_prefetch_phase(a, ph + 1, nc, stride);
		for (int i = lo + tid; i < hi; i += stride) {
			dfl r0, r1;
			double q0 = 0.0, q1 = 0.0;
			dfl t0 = {0.f, 0.f}, t1 = {0.f, 0.f};
			float4 const d = reinterpret_cast<const float4*>(a.dinv)[i];
			dfl z0, z1;
			int const sl = a.sbase[c] + ((i - lo) >> 5), lane = (i - lo) & 31;
			if (forward) {
				ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
				sell_row(a.lv, a.lc, a.lp, sl, lane, a.y, t0, t1);
				ssor_blk(d, df_add(r0, df_neg(t0)), df_add(r1, df_neg(t1)), z0, z1);
			}
			else {
				sell_row(a.uv, a.uc, a.up, sl, lane, a.y, t0, t1);
				dfl w0, w1;
				ssor_blk(d, t0, t1, w0, w1);
				float4 const yv = __ldcg(reinterpret_cast<const float4*>(a.y) + i);
				z0 = df_add({yv.x, yv.z}, df_neg(w0));
				z1 = df_add({yv.y, yv.w}, df_neg(w1));
				ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
			}
			__stcg(reinterpret_cast<float4*>(a.y) + i, make_float4(z0.hi, z1.hi, z0.lo, z1.lo));
			if (final_rows) {
				if (fuse && !last) ssor_st_plain<VT>(a, i, z0, z1);
				else ssor_st_z<VT>(a, i, z0, z1, r0, r1, q0, q1, acc, acc64);
			}
		}
		if (fuse) {
			CoarseArgs const& co = a.co;
			if (ph == 0) {  // r_c = P^T r: chunk partial sums, a warp per chunk
				int const nw = stride >> 5, wid = tid >> 5;
				for (int q = wid; q < co.nchunk; q += nw) restrict_chunk_lean(co, q, threadIdx.x & 31);
			}
			else if (ph == 1) {  // the chunks of each coarse DOF, in order
				for (int t = tid; t < co.nc; t += stride) restrict_sum_one(co, t);
			}
			else if (ph == 2) {  // y_t = X r_c, a block per row
				for (int i = blockIdx.x; i < co.nc; i += gridDim.x) {
					dfl const s = coarse_row_dot<1>(co.xl + xrow(i), i + 1, co.rc);
					if (threadIdx.x == 0) co.yt[i] = make_float2(s.hi, s.lo);
					__syncthreads();
				}
			}
			else if (ph == 3) {  // y_c = X^T y_t
				for (int j = blockIdx.x; j < co.nc; j += gridDim.x) {
					dfl const s = coarse_row_dot<1>(co.xu + xrow(co.nc - 1 - j), co.nc - j, co.yt + j);
					if (threadIdx.x == 0) co.yc[j] = make_float2(s.hi, s.lo);
					__syncthreads();
				}
			}
			if (last)  // the rows finished before y_c existed: every colour but colour 0
				for (int i = a.off[1] + tid; i < a.off[nc]; i += stride) ssor_add_coarse<VT>(a, i, acc, acc64);
		}
		if (!last) alive = ssor_barrier(a);
	}
	// every block reaches the reduction, finished or not
	double v[1] = {VT == VT_F64 ? acc64 : df_dbl(acc)};
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) ssor_finish(a, out[0]);
}

// the 2x3 block P_i = [[f0, 0, -f0 dy], [0, f1, f1 dx]] of a node with
// q = (dx, dy, f0, f1), or zero
__device__ __forceinline__ void p_block(float4 q, bool on, double p[2][3]) {
	double const f0 = on ? q.z : 0.f, f1 = on ? q.w : 0.f;
	p[0][0] = f0;  p[0][1] = 0.0; p[0][2] = -f0 * (double) q.y;
	p[1][0] = 0.0; p[1][1] = f1;  p[1][2] = f1 * (double) q.x;
}

// acc += P_r^T (M d), M a 2x2 block, d and P_r 2x3
__device__ __forceinline__ void acc_ptmd(double acc[9], const double pr[2][3], double m0, double m1, double m2, double m3,
                                         const double d[2][3]) {
#pragma unroll
	for (int b = 0; b < 3; b++) {
		double const t0 = m0 * d[0][b] + m1 * d[1][b];
		double const t1 = m2 * d[0][b] + m3 * d[1][b];
#pragma unroll
		for (int q = 0; q < 3; q++) acc[3 * q + b] += pr[0][q] * t0 + pr[1][q] * t1;
	}
}

// A_c = P^T A P in two deterministic stages.  One warp per chunk of
// aggregate I: every lane keeps the 3x3 blocks of the 9 cells around I (slot
// = cell offset), so the lanes' partial sums line up and are reduced in a
// fixed order into the chunk's 81 values; then per aggregate and entry the
// chunks in chunk order.  A neighbour outside those 9 cells sets *err (the
// caller then drops the coarse correction).
// The sums run in double-float on the FP32 pipe (GB300 issues FP64 at a small
// fraction of that rate): the FP32 operator's products are exact (TwoProduct
// by FMA), FP64 operator values enter as pairs.
__global__ void k_coarse_ac(CoarseArgs a) {
	int const q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (q >= a.nchunk) return;
	int cx, cy;
	cell_xy(a.chunk_agg[q], a.gx, a.gy, a.xfast, cx, cy);
	dfl acc[9][9];
	for (int s = 0; s < 9; s++)
		for (int t = 0; t < 9; t++) acc[s][t] = {0.f, 0.f};
	for (int k = a.chunk_start[q] + lane; k < a.chunk_start[q + 1]; k += 32) {
		int const i = a.agg_nodes[k];
		float4 const pi = a.pnode[i];
		float const fi0 = pi.z, fi1 = pi.w;
		float const p20 = -fi0 * pi.y, p21 = fi1 * pi.x;  // the rotation row of P_i^T (exact: f is 0 or 1)
		// the FP32 operator in difference form, (A g)_i = S_i g_i + sum_j A_ij (g_j - g_i):
		// its diagonal block is S_i - sum_{j != i} A_ij
		dfl deff[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
		if (!a.vals64) {
			float4 const sr = reinterpret_cast<const float4*>(a.corr32)[i];
			deff[0] = {sr.x, 0.f}; deff[1] = {sr.y, 0.f}; deff[2] = {sr.z, 0.f}; deff[3] = {sr.w, 0.f};
			for (int e = a.row_ptr[i]; e < a.row_ptr[i + 1]; e++) {
				if (a.cols[e] == i) continue;
				float4 const v = reinterpret_cast<const float4*>(a.vals32)[e];
				deff[0] = df_add(deff[0], {-v.x, 0.f}); deff[1] = df_add(deff[1], {-v.y, 0.f});
				deff[2] = df_add(deff[2], {-v.z, 0.f}); deff[3] = df_add(deff[3], {-v.w, 0.f});
			}
		}
		for (int e = a.row_ptr[i]; e < a.row_ptr[i + 1]; e++) {
			int const j = a.cols[e];
			int jx, jy;
			cell_xy(a.agg[j], a.gx, a.gy, a.xfast, jx, jy);
			int const ox = jx - cx, oy = jy - cy;
			if (ox < -1 || ox > 1 || oy < -1 || oy > 1) {
				atomicOr(a.err, 1);
				continue;
			}
			int const slot = (oy + 1) * 3 + (ox + 1);
			float4 const pj = a.pnode[j];
			float const gj0 = pj.z, gj1 = pj.w, r0 = -gj0 * pj.y, r1 = gj1 * pj.x;  // exact: g is 0 or 1
			dfl m[4];
			if (a.vals64) {
				for (int t = 0; t < 4; t++) m[t] = df_make(a.vals64[4l * e + t]);
			}
			else if (j == i) {
				for (int t = 0; t < 4; t++) m[t] = deff[t];
			}
			else {
				float4 const v = reinterpret_cast<const float4*>(a.vals32)[e];
				m[0] = {v.x, 0.f}; m[1] = {v.y, 0.f}; m[2] = {v.z, 0.f}; m[3] = {v.w, 0.f};
			}
			// A P_j (2x3), then P_i^T (3x2) times it
			dfl const ap[2][3] = {{df_mul_f(gj0, m[0]), df_mul_f(gj1, m[1]), df_add(df_mul_f(r0, m[0]), df_mul_f(r1, m[1]))},
			                      {df_mul_f(gj0, m[2]), df_mul_f(gj1, m[3]), df_add(df_mul_f(r0, m[2]), df_mul_f(r1, m[3]))}};
#pragma unroll
			for (int v = 0; v < 3; v++) {
				acc[slot][v] = df_add(acc[slot][v], df_mul_f(fi0, ap[0][v]));
				acc[slot][3 + v] = df_add(acc[slot][3 + v], df_mul_f(fi1, ap[1][v]));
				acc[slot][6 + v] = df_add(acc[slot][6 + v], df_add(df_mul_f(p20, ap[0][v]), df_mul_f(p21, ap[1][v])));
			}
		}
	}
	for (int s = 0; s < 9; s++)
		for (int t = 0; t < 9; t++) {
			dfl x = acc[s][t];
#pragma unroll
			for (int o = 16; o; o >>= 1) x = df_add(x, {__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)});
			if (lane == 0) a.part[81l * q + 9 * s + t] = df_dbl(x);
		}
}

// The chunks' sums per aggregate into the lower band of A_c, each entry the
// mean of itself and its transpose (the same coupling seen from the other
// cell: the mirrored slot, u and v swapped), and the diagonal saved for the
// pivot test.  Coarse DOFs without any coupling -- empty cells, all-constrained
// or degenerate modes -- get a zero diagonal, which the pivot test drops.
__global__ void k_coarse_ac_sum(CoarseArgs a) {
	long const t = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (t >= 81l * a.na) return;
	int const I = (int) (t / 81), e = (int) (t % 81), s = e / 9, u = (e % 9) / 3, v = e % 3;
	int cx, cy;
	cell_xy(I, a.gx, a.gy, a.xfast, cx, cy);
	int const jx = cx + s % 3 - 1, jy = cy + s / 3 - 1;
	if (jx < 0 || jx >= a.gx || jy < 0 || jy >= a.gy) return;
	int const J = cell_id(jx, jy, a.gx, a.gy, a.xfast);
	int const row = 3 * I + u, col = 3 * J + v;
	if (row < col) return;
	if (row - col > a.bw) {
		atomicOr(a.err, 1);
		return;
	}
	double x = 0.0, y = 0.0;
	for (int q = a.agg_chunk[I]; q < a.agg_chunk[I + 1]; q++) x += a.part[81l * q + e];
	int const et = 9 * (8 - s) + 3 * v + u;
	for (int q = a.agg_chunk[J]; q < a.agg_chunk[J + 1]; q++) y += a.part[81l * q + et];
	double const m = 0.5 * (x + y);
	dfl const d = df_make(m);
	a.band[(long) row * (a.bw + 1) + (row - col)] = make_float2(d.hi, d.lo);
	if (row == col) a.diag0[row] = m;
}

// Band Cholesky A_c = L L^T in place, one block, in double-float arithmetic
// on the FP32 pipe (FP64 issues at a small fraction of that rate on this
// GPU).  The active part of the trailing matrix (rows k .. k + bw, their band)
// lives in a (bw + 2)^2 window in shared memory, rows in a ring.  Step k: the
// pivot p = S_kk; p at or below 1e-12 of A_c's diagonal entry (a coarse mode
// that A barely sees: an empty cell, the rotation of a single node) drops DOF
// k: its column of L is zero and 1 / L_kk = 0 marks it, so the factorisation
// goes on as that of A_c without that DOF.  Otherwise column k is scaled by
// 1/sqrt(p) and written out (the diagonal holds 1/sqrt(p)), the next row of
// A_c (loaded one step ahead) enters the ring slot of the finished row
// k - 1, and the window takes the rank-1 update; the thread that updates
// S_{k+1,k+1} then forms the next pivot's 1/sqrt.  Two barriers per step.
__global__ void __launch_bounds__(CHOL_T) k_coarse_chol(CoarseArgs a) {
	extern __shared__ float2 sm2[];
	int const n = a.nc, bw = a.bw, B = bw + 1, M = bw + 2;
	float2* W = sm2;                    // entry (r, c) at W[(r % M) M + c % M]
	float2* col = W + M * M;            // scaled column k (rows k + 1 ..)
	float2* piv = col + M;              // 1/sqrt of the current pivot (0: dropped)
	float* thr = reinterpret_cast<float*>(piv + 2);   // drop thresholds, 1e-12 A_c,kk
	short2* pr = reinterpret_cast<short2*>(thr + n + 1);  // update pairs (ii, jj), jj <= ii < bw, by rows
	int const tx = threadIdx.x;
	for (int ii = tx; ii < bw; ii += blockDim.x)
		for (int jj = 0; jj <= ii; jj++) pr[ii * (ii + 1) / 2 + jj] = make_short2((short) ii, (short) jj);
	for (int k = tx; k < n; k += blockDim.x) thr[k] = (float) (1e-12 * a.diag0[k]);
	for (int e = tx; e < B * B; e += blockDim.x) {
		int const r = e / B, t = e % B;
		if (r < n && r - t >= 0) W[(r % M) * M + (r - t) % M] = a.band[(long) r * B + t];
	}
	__syncthreads();
	if (tx == 0) {
		dfl const q = pivot_rsqrt({W[0].x, W[0].y}, thr[0]);
		piv[0] = make_float2(q.hi, q.lo);
	}
	__syncthreads();
	// ring slots advance with k: s1 = (k + 1) % M, sk = k % M; the row entering
	// at step k (k + bw + 1) was loaded one step earlier
	float2 nv = (bw + 1 < n && tx < B) ? a.band[(long) (bw + 1) * B + tx] : make_float2(0.f, 0.f);
	int sk = 0;
	for (int k = 0; k < n; k++) {
		dfl const isq = {piv[0].x, piv[0].y};
		int const s1 = sk + 1 == M ? 0 : sk + 1;
		int const m = min(bw, n - 1 - k);  // rows k + 1 .. k + m below the pivot
		int const r = k + bw + 1;
		bool const ld = r < n && tx < B;
		float2 const nv2 = (r + 1 < n && tx < B) ? a.band[(long) (r + 1) * B + tx] : make_float2(0.f, 0.f);
		for (int ii = tx; ii < m; ii += blockDim.x) {
			int si = s1 + ii;
			si -= si >= M ? M : 0;
			float2 const w = W[si * M + sk];
			dfl const c = df_mul({w.x, w.y}, isq);
			col[ii] = make_float2(c.hi, c.lo);
			a.band[(long) (k + 1 + ii) * B + ii + 1] = make_float2(c.hi, c.lo);
		}
		if (tx == 0) a.band[(long) k * B] = make_float2(isq.hi, isq.lo);
		if (ld) {
			// row r's slot is that of row k - 1, i.e. sk - 1; entry (r, r - tx) at column slot (r - tx) % M
			int const sr = sk == 0 ? M - 1 : sk - 1;
			int sc = sr - tx;
			sc += sc < 0 ? M : 0;
			W[sr * M + sc] = nv;
		}
		nv = nv2;
		__syncthreads();
		int const nu = m * (m + 1) / 2;
		auto upd = [&](int e) {
			short2 const q = pr[e];
			int si = s1 + q.x, sj = s1 + q.y;
			si -= si >= M ? M : 0;
			sj -= sj >= M ? M : 0;
			float2 const ci = col[q.x], cj = col[q.y], w = W[si * M + sj];
			dfl const u = df_add({w.x, w.y}, df_neg(df_mul({ci.x, ci.y}, {cj.x, cj.y})));
			W[si * M + sj] = make_float2(u.hi, u.lo);
		};
		// pair 0 is S_{k+1,k+1}: the block's last thread updates it first and
		// forms the next pivot at once, and the other pairs go round-robin
		// from thread 0, so the pivot's dependent chain runs in a warp with
		// one pair fewer than the busiest ones instead of after thread 0's
		if (tx == blockDim.x - 1 && m > 0) {
			upd(0);
			float2 const p = W[s1 * M + s1];
			dfl const q = pivot_rsqrt({p.x, p.y}, thr[k + 1]);
			piv[0] = make_float2(q.hi, q.lo);
		}
		for (int e = 1 + tx; e < nu; e += blockDim.x) upd(e);
		sk = s1;
		__syncthreads();
	}
}

// X = L^-1 by columns, in double-float arithmetic: each warp takes LINV_C
// consecutive columns j0 .., LINV_L lanes per column (lane h of a column takes
// the band entries t = 1 + h, 1 + h + LINV_L, ..), a shuffle sum over them,
// forward substitution down the band from row j0 (rows above a column's own
// j come out zero).  The rows of L are staged in shared memory (the next one
// loaded while this one is used), each column's last bw values in a shared
// ring.  A dropped DOF (1 / L_ii = 0) gets a zero row, and a zero column.  X
// is written, rounded to FP32, by rows to xl and transposed to xu.
__global__ void __launch_bounds__(32 * LINV_W) k_coarse_linv(CoarseArgs a) {
	extern __shared__ float2 lsm2[];
	constexpr int NL = (COARSE_MAX_BW + 1 + 31) / 32;  // row entries per lane when staging
	int const n = a.nc, bw = a.bw, B = bw + 1, M = bw + 2;
	int const w = threadIdx.x >> 5, lane = threadIdx.x & 31, c = lane / LINV_L, h = lane % LINV_L;
	int const j0 = (blockIdx.x * LINV_W + w) * LINV_C;
	if (j0 >= n) return;
	float2* ring = lsm2 + (size_t) w * (LINV_C * M + 2 * B);
	float2* Lr = ring + LINV_C * M;
	int const j = j0 + c;
	for (int t = lane; t < LINV_C * M; t += 32) ring[t] = make_float2(0.f, 0.f);
	for (int t = lane; t < B; t += 32) Lr[t] = a.band[(long) j0 * B + t];
	__syncwarp();
	float2* R = ring + c * M;
	int si = j0 % M;  // ring slot of row i
	for (int i = j0; i < n; i++) {
		const float2* cur = Lr + ((i - j0) & 1) * B;
		float2* nxt = Lr + ((i - j0 + 1) & 1) * B;
		float2 nv[NL];
#pragma unroll
		for (int u = 0; u < NL; u++) {
			int const t = lane + 32 * u;
			nv[u] = (i + 1 < n && t < B) ? a.band[(long) (i + 1) * B + t] : make_float2(0.f, 0.f);
		}
		int const tmax = min(bw, i - j0);
		dfl s0 = {0.f, 0.f}, s1 = {0.f, 0.f};
		// ring slot of row i - t, stepped down by LINV_L per term (M >= 10 and
		// LINV_L <= 16: two wraps at most)
		int sl = si - 1 - h;
		while (sl < 0) sl += M;
		for (int t = 1 + h; t <= tmax; t += 2 * LINV_L) {
			float2 const l0 = cur[t], x0 = R[sl];
			s0 = df_add(s0, df_mul({l0.x, l0.y}, {x0.x, x0.y}));
			sl -= LINV_L;
			while (sl < 0) sl += M;
			if (t + LINV_L <= tmax) {
				float2 const l1 = cur[t + LINV_L], x1 = R[sl];
				s1 = df_add(s1, df_mul({l1.x, l1.y}, {x1.x, x1.y}));
			}
			sl -= LINV_L;
			while (sl < 0) sl += M;
		}
		dfl s = df_add(s0, s1);
#pragma unroll
		for (int o = 1; o < LINV_L; o <<= 1)
			s = df_add(s, {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
		float2 const d = cur[0];
		dfl const x = df_mul(df_add({i == j ? 1.f : 0.f, 0.f}, df_neg(s)), {d.x, d.y});
		__syncwarp();
		if (h == 0 && j < n) {
			R[si] = make_float2(x.hi, x.lo);
			if (i >= j) {
				a.xl[xrow(i) + j] = x.hi;
				a.xu[xrow(n - 1 - j) + (i - j)] = x.hi;
			}
		}
#pragma unroll
		for (int u = 0; u < NL; u++) {
			int const t = lane + 32 * u;
			if (t < B) nxt[t] = nv[u];
		}
		si = si + 1 == M ? 0 : si + 1;
		__syncwarp();
	}
}

// X = L^-1 by block rows (block size b >= bw, so L is block bidiagonal:
// block row k holds its diagonal block L_kk and the block L_k,k-1).  Row i of
// X follows x_i = d_i (e_i - sum_{i' < i} L_ii' x_i') with d_i = 1 / L_ii (0
// for a dropped DOF: a zero row and column, as the column-wise form).  Within
// block row k that forward substitution is linear in what block row k-1
// feeds it, so X_kk is the substitution of the unit vectors and, for every
// column of an earlier block, X_kj = M_k X_k-1,j with M_k = -X_kk L_k,k-1.
// k_linv_diag forms X_kk and M_k for every k at once (a block each); then
// k_linv_step, one launch per block row, forms X_kj for all j < k from the
// previous block row: the sequential chain is nc / b launches instead of nc
// dependent steps per column.  Double-float throughout; X and X^T written
// rounded to FP32 in the layout of k_coarse_linv.
constexpr int LB_T = 256;  // threads of the blocked-inversion kernels

__host__ __device__ constexpr size_t linv_diag_smem(int b) { return sizeof(float2) * 2 * (size_t) b * b; }

__global__ void __launch_bounds__(LB_T) k_linv_diag(CoarseArgs a, int b, float2* __restrict__ M, float2* __restrict__ Xd) {
	extern __shared__ float2 lbs[];
	int const n = a.nc, bw = a.bw, B = bw + 1;
	int const k = blockIdx.x, r0 = k * b, rows = min(b, n - r0);
	float2* Lk = lbs;          // [b][b]: L(r0 + i, r0 + i') for i' < i, 1 / L_ii on the diagonal
	float2* Xk = lbs + b * b;  // [b][b]: X(r0 + i, r0 + j)
	for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
		int const i = e / b, ip = e % b;
		float2 v = make_float2(0.f, 0.f);
		if (i < rows && ip <= i && i - ip <= bw) v = a.band[(long) (r0 + i) * B + (i - ip)];
		Lk[e] = v;
		Xk[e] = make_float2(0.f, 0.f);
	}
	__syncthreads();
	for (int j = threadIdx.x; j < rows; j += blockDim.x)
		for (int i = j; i < rows; i++) {
			dfl s = {i == j ? 1.f : 0.f, 0.f};
			for (int ip = max(j, i - bw); ip < i; ip++) {
				float2 const l = Lk[i * b + ip], x = Xk[ip * b + j];
				s = df_add(s, df_neg(df_mul({l.x, l.y}, {x.x, x.y})));
			}
			float2 const d = Lk[i * b + i];
			dfl const x = df_mul(s, {d.x, d.y});
			Xk[i * b + j] = make_float2(x.hi, x.lo);
		}
	__syncthreads();
	for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
		int const i = e / b, j = e % b;
		float2 const x = Xk[e];
		Xd[(long) k * b * b + e] = x;
		if (i < rows && j <= i) {
			a.xl[xrow(r0 + i) + r0 + j] = x.x;
			a.xu[xrow(n - 1 - (r0 + j)) + (i - j)] = x.x;
		}
	}
	if (k == 0) return;
	// M_k = -X_kk L_k,k-1: L(r0 + m, r0 - b + c) is in the band when m + b - c <= bw
	for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
		int const i = e / b, c = e % b;
		dfl s = {0.f, 0.f};
		if (i < rows)
			for (int m = 0; m <= i; m++) {
				int const t = m + b - c;
				if (t > bw) continue;
				float2 const x = Xk[i * b + m], l = a.band[(long) (r0 + m) * B + t];
				s = df_add(s, df_mul({x.x, x.y}, {l.x, l.y}));
			}
		M[(long) k * b * b + e] = make_float2(-s.hi, -s.lo);
	}
}

// block row k of X for the columns of the earlier blocks (0 .. r0 - 1):
// X(r0 + i, col) = sum_c M_k(i, c) X(r0 - b + c, col), the previous block row
// read from Xw_prev (its columns before r0 - b) and Xd (its diagonal block)
__global__ void __launch_bounds__(LB_T) k_linv_step(CoarseArgs a, int b, int k, const float2* __restrict__ M,
                                                     const float2* __restrict__ Xd, const float2* __restrict__ Xw_prev,
                                                     float2* __restrict__ Xw_cur) {
	int const n = a.nc, r0 = k * b, rows = min(b, n - r0);
	long const t = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (t >= (long) rows * r0) return;
	int const i = (int) (t / r0), col = (int) (t % r0);
	int const pb = r0 - b;  // first column of the previous diagonal block
	const float2* Mi = M + ((long) k * b + i) * b;
	dfl s = {0.f, 0.f};
	for (int c = 0; c < b; c++) {
		float2 const m = Mi[c];
		float2 const x = col < pb ? Xw_prev[(long) c * n + col] : Xd[((long) (k - 1) * b + c) * b + (col - pb)];
		s = df_add(s, df_mul({m.x, m.y}, {x.x, x.y}));
	}
	Xw_cur[(long) i * n + col] = make_float2(s.hi, s.lo);
	a.xl[xrow(r0 + i) + col] = s.hi;
	a.xu[xrow(n - 1 - col) + (r0 + i - col)] = s.hi;
}

// The block rows of X in one cooperative launch: a grid barrier between block
// rows instead of a launch each (bounded waits: a timeout sets *a.berr and the
// blocks stop).  The recurrence X_kj = M_k X_k-1,j runs in FP32 on the
// double-float M_k and diagonal blocks' leading parts: X is stored in FP32, and
// its rounding already perturbs X^T X by about u_fp32 cond(A_c), the order of
// what the FP32 recurrence adds (forward substitution is backward stable)
__global__ void __launch_bounds__(LB_T) k_linv_all(CoarseArgs a, int b, const float2* __restrict__ M,
                                                    const float2* __restrict__ Xd, float2* __restrict__ Xw) {
	grid_barrier_init(a.bar);
	int const n = a.nc, nb = (n + b - 1) / b;
	long const stride = (long) gridDim.x * blockDim.x;
	for (int k = 1; k < nb; k++) {
		int const r0 = k * b, rows = min(b, n - r0), pb = r0 - b;
		const float2* prev = Xw + (long) ((k + 1) & 1) * b * n;
		float2* cur = Xw + (long) (k & 1) * b * n;
		for (long t = blockIdx.x * (long) blockDim.x + threadIdx.x; t < (long) rows * r0; t += stride) {
			int const i = (int) (t / r0), col = (int) (t % r0);
			const float2* Mi = M + ((long) k * b + i) * b;
			float s = 0.f;
			for (int c = 0; c < b; c++) {
				float const m = Mi[c].x;
				float const x = col < pb ? __ldcg(prev + (long) c * n + col).x : Xd[((long) (k - 1) * b + c) * b + (col - pb)].x;
				s = __fmaf_rn(m, x, s);
			}
			__stcg(cur + (long) i * n + col, make_float2(s, 0.f));
			a.xl[xrow(r0 + i) + col] = s;
			a.xu[xrow(n - 1 - col) + (r0 + i - col)] = s;
		}
		if (k + 1 < nb && !grid_barrier(a.bar, a.berr, a.polls)) return;
	}
}

// kernels of one SpMV shape (lanes per row), for the graph builder and the autotuner
struct CgKernels {
	void* hs64s;   // split-form K1 (with k_hs64_dir before it)
	void* hsdfs;   // split-form K1 (with k_hsdf_dir before it)
	void* spmv64;
	void* spmvmx;
	void* replace;
	void* res64;
	void* resmx;
	void* hs64;
	void* hs64repl;
	void* hsdf;
	void* hsdfrepl;
};

template <int LPR, int NB = 1>
CgKernels kernels_for() {
	return {(void*) k_hs64_spmv_s<LPR, NB>, (void*) k_hsdf_spmv_s<LPR, NB>,
	        (void*) k_cg64_spmv<LPR>, (void*) k_mx_spmv<LPR, NB>, (void*) k_mx_replace<LPR>,
	        (void*) k_true_residual<LPR, double>, (void*) k_true_residual<LPR, float>, (void*) k_hs64_spmv<LPR, NB>,
	        (void*) k_hs64_replace<LPR>, (void*) k_hsdf_spmv<LPR, NB>, (void*) k_hsdf_replace<LPR>};
}

// SpMV shape code: lanes per row + 100 x entries batched per lane (1:
// unbatched), + 1000 for the split form (direction kernel + p'-only SpMV;
// FP64 and double-float paths)
constexpr int SHAPES[] = {1, 2, 4, 8, 16, 401, 801, 402, 204, 1001, 1002, 1004, 1401, 1402, 1801};
constexpr int shape_lanes(int code) { return code % 100; }
constexpr bool shape_split(int code) { return code >= 1000; }

CgKernels kernels_lpr(int code) {
	switch (code % 1000) {
	case 1: return kernels_for<1>();
	case 2: return kernels_for<2>();
	case 4: return kernels_for<4>();
	case 16: return kernels_for<16>();
	case 401: return kernels_for<1, 4>();
	case 801: return kernels_for<1, 8>();
	case 402: return kernels_for<2, 4>();
	case 204: return kernels_for<4, 2>();
	default: return kernels_for<8>();
	}
}

}  // namespace
