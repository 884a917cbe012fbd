// Krylov kernels of the GB300 libbfm solver: grid reductions, the FP64 and
// mixed-precision PCG iterations and residual checks.  Included by every
// translation unit that launches them (internal linkage: each gets its own
// instantiations).
#pragma once

#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>

#include <bfm/gpu.h>

namespace {

#ifndef BFM_TPB
#define BFM_TPB 256
#endif
constexpr int TPB_K = BFM_TPB;

// ------------------------------------------------------------------ reductions

// Sum NV values over the whole grid: every block writes its partial sums,
// the last block to arrive (atomic ticket) adds them in block order and
// returns true with the totals in `out`.  The result does not depend on which
// block arrives last.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* __restrict__ partials, unsigned* ticket,
                                         double (&out)[NV]) {
	__shared__ double sm[TPB_K / 32][NV];
	__shared__ bool is_last;
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
	for (int i = 0; i < NV; i++)
		for (int o = 16; o; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
	if (lane == 0)
		for (int i = 0; i < NV; i++) sm[wid][i] = v[i];
	__syncthreads();
	if (wid == 0) {
#pragma unroll
		for (int i = 0; i < NV; i++) {
			double t = lane < nw ? sm[lane][i] : 0.0;
			for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
			if (lane == 0) partials[blockIdx.x * NV + i] = t;
		}
	}
	if (threadIdx.x == 0) {
		__threadfence();
		unsigned const tk = atomicAdd(ticket, 1u);
		is_last = tk == gridDim.x - 1;
	}
	__syncthreads();
	if (!is_last) return false;
	__threadfence();
	double w[NV];
#pragma unroll
	for (int i = 0; i < NV; i++) w[i] = 0.0;
	for (int blk = threadIdx.x; blk < gridDim.x; blk += blockDim.x)
#pragma unroll
		for (int i = 0; i < NV; i++) w[i] += __ldcg(&partials[blk * NV + i]);
#pragma unroll
	for (int i = 0; i < NV; i++)
		for (int o = 16; o; o >>= 1) w[i] += __shfl_down_sync(0xffffffffu, w[i], o);
	__syncthreads();
	if (lane == 0)
		for (int i = 0; i < NV; i++) sm[wid][i] = w[i];
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int i = 0; i < NV; i++) {
			double t = 0.0;
			for (int k = 0; k < nw; k++) t += sm[k][i];
			out[i] = t;
		}
		*ticket = 0u;
	}
	__syncthreads();
	return true;
}

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
	int iter, max_iters;
	int done, status;
	int replacements;
};

struct CgOpts {
	double rtol;
	double drop2;  // mixed: replace when (r,r) has dropped by this factor since the last replacement
	int max_iters;
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
	const float* corr;      // mixed: per-node 2x2 row-sum correction of the FP32 operator
	int block_pc;
	const double* b;
	double* x;
	V* r;
	V* u;   // FP64 path: u = M r (materialized); mixed path: dx, the grouped solution update
	V* p;   // FP64 path: direction; mixed path: direction read this iteration
	V* pn;  // mixed path: direction written this iteration (ping-pong with p)
	V* s;   // FP64 path: s = A p by recurrence
	V* w;   // FP64 path: w = A u; mixed path: q = A p
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgOpts opts;
	cudaGraphConditionalHandle cond;       // while-node: keep iterating
	cudaGraphConditionalHandle cond_repl;  // if-node: replace the residual this iteration
	int use_cond;  // launched inside the solve graph: drive its conditional nodes
	int timing;    // measurement launches: ignore the stop flag, never set it
};

template <typename V> struct Vec2;
template <> struct Vec2<double> { using T = double2; };
template <> struct Vec2<float> { using T = float2; };

template <typename V>
__device__ __forceinline__ typename Vec2<V>::T ld2(const V* p, int i) {
	return reinterpret_cast<const typename Vec2<V>::T*>(p)[i];
}
template <typename V>
__device__ __forceinline__ void st2(V* p, int i, V a, V b) {
	typename Vec2<V>::T t;
	t.x = a;
	t.y = b;
	reinterpret_cast<typename Vec2<V>::T*>(p)[i] = t;
}

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
		V u0, u1;
		precond_apply(a.dinv, a.block_pc, i, r0, r1, u0, u1);
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
		st->status = BFM_GPU_OK;
		st->done = out[0] == 0.0;  // b = 0: x = 0 is exact
		st->gamma_old = 0; st->alpha_old = 0;
		st->alpha = 0; st->beta = 0;
		st->rho = out[0];
		st->rho_ref = out[0];
		st->true_res2 = out[0];
		if (a.use_cond) cudaGraphSetConditional(a.cond, st->done ? 0u : 1u);
	}
}

// ---------------------------------------------------------------- FP64 path
// Chronopoulos-Gear PCG: one reduction per iteration and only the SpMV's
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
//   - the FP32 operator keeps the FP64 matrix's block row sums through a
//     per-node 2x2 correction block, so rounding does not break the rigid
//     translation modes (without it the FP32 operator loses definiteness on
//     ill-conditioned meshes and CG diverges).
//   K1: p' = M r + beta p; q = (A32 + C) p'; alpha = gamma / (p', q)
//   K2: dx += alpha p'; r -= alpha q; gamma' = (r, M r), rho = (r, r); beta
//   on request (IF node): x += dx, dx = 0; r = b - A64 x in FP64; gamma = (r, M r)

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

template <int LPR>
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
	int const bpc = a.block_pc;
	auto gather = [=](int c, float& g0, float& g1) {
		float2 const rc = ld2(r, c), pc = ld2(p, c);
		float z0, z1;
		precond_apply(dinv, bpc, c, rc.x, rc.y, z0, z1);
		g0 = z0 + beta * pc.x;
		g1 = z1 + beta * pc.y;
	};
	DF pq = {0.f, 0.f};
	FOR_ROWS(LPR) {
		bool const ok = row_ < a.N;
		int const ks = ok ? a.row_ptr[row_] : 0, ke = ok ? a.row_ptr[row_ + 1] : 0;
		float y0, y1;
		row_product<LPR, float>(a.cols, a.vals, ks, ke, sub_, gather, y0, y1);
		if (ok && sub_ == 0) {
			float g0, g1;
			gather(row_, g0, g1);
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
		float z0, z1;
		precond_apply(a.dinv, a.block_pc, i, r0, r1, z0, z1);
		df_add_prod(g, r0, z0);
		df_add_prod(g, r1, z1);
		df_add_prod(rr, r0, r0);
		df_add_prod(rr, r1, r1);
	}
	double v[2] = {df_value(g), df_value(rr)};
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
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
	double y0, y1;
	if (a.vals64) row_product<LPR, double>(a.cols, a.vals64, ks, ke, sub, gather, y0, y1);
	else row_product<LPR, double>(a.cols, a.vals, ks, ke, sub, gather, y0, y1);
	e0 = e1 = 0.0;
	if (ok) {
		if (!a.vals64 && a.corr) {
			float4 const cc = reinterpret_cast<const float4*>(a.corr)[row];
			double2 const xi = ld2(x, row);
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
			float z0, z1;
			precond_apply(a.dinv, a.block_pc, row_, r0, r1, z0, z1);
			v[0] += e0 * e0 + e1 * e1;
			v[1] += (double) r0 * (double) z0 + (double) r1 * (double) z1;
		}
	}
	double out[2];
	if (grid_sum<2>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		st->replacements += 1;
		st->rho_ref = out[0];
		st->true_res2 = out[0];
		st->gamma = out[1];
		if (out[0] <= st->rtol * st->rtol * st->bnorm2) {
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

// kernels of one SpMV shape (lanes per row), for the graph builder and the autotuner
struct CgKernels {
	void* spmv64;
	void* spmvmx;
	void* replace;
	void* res64;
	void* resmx;
};

template <int LPR>
CgKernels kernels_for() {
	return {(void*) k_cg64_spmv<LPR>, (void*) k_mx_spmv<LPR>, (void*) k_mx_replace<LPR>,
	        (void*) k_true_residual<LPR, double>, (void*) k_true_residual<LPR, float>};
}

CgKernels kernels_lpr(int lpr) {
	switch (lpr) {
	case 1: return kernels_for<1>();
	case 2: return kernels_for<2>();
	case 4: return kernels_for<4>();
	case 16: return kernels_for<16>();
	default: return kernels_for<8>();
	}
}


}  // namespace
