// Batched uneven solves of the GB300 libbfm: many independent meshes,
// assembled as one block-diagonal problem and solved by ONE persistent
// cooperative kernel in which every mesh ("part") runs its own mixed-precision
// PCG (its own alpha, beta, stopping test and FP64 residual replacements).
//
// Reference counterpart: the sequential instance loop of run_elasticity
// (libbfm/src/sim.c:103-135), one direct solve per instance.
//
// Work layout: the rows of every part are cut into tiles (part, first row,
// end row); block b owns tiles b, b+G, b+2G, ... for the whole solve.  Per
// iteration:
//   phase 1  tiles: p' = M r + beta_k p, q = A32 p' in difference form, partial (p', q)
//   barrier; every block sums each part's tile partials in tile order
//            (deterministic, identical in all blocks): alpha_k
//   phase 2  tiles: dx += alpha_k p', r -= alpha_k q, partials (r, M r), (r, r)
//   barrier; every block: beta_k, stopping and replacement decisions
//   [only when some part asks: flush dx into x, barrier, FP64 residual of
//    those parts, barrier, their new gamma and stopping test]
// Every block keeps a replica of all parts' scalars in shared memory, so no
// block ever waits for another to publish them.  Grid barriers spin with an
// iteration limit: on timeout the kernel records an error and every block
// leaves the loop.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <bfm/gpu.h>

#include "cg_kernels.cuh"
#include "internal.h"
#include "trace.h"

namespace {

constexpr int BT = 256;          // threads per block
constexpr int MAX_PARTS = 512;   // parts per batch (shared-memory replica)
constexpr long SPIN_LIMIT = 1l << 25;  // default polls per barrier (each an L2 round trip: seconds in all)

enum : int { BERR_BARRIER_TIMEOUT = 1 };

struct PartState {
	double bnorm2, gamma, alpha, beta, rho, rho_ref, true_res2;
	int iter, done, status, replacements;
};

struct BatchArgs {
	int N, n_parts, n_tiles;
	const int* tile_part;
	const int* tile_begin;   // first row (node) of the tile
	const int* tile_end;
	const int* part_tile;    // tiles of part k: [part_tile[k], part_tile[k+1])
	const int* row_ptr;
	const int* cols;
	const float* vals;
	const float* corr;       // row-sum block S of the FP32 operator (difference form)
	const float* dinv;
	const double* vals64;    // FP64 residual operator (nullptr: the FP32 one in difference form)
	const double* b;
	double* x;
	float* r;
	float* p0;
	float* p1;
	float* q;
	float* dx;
	double* partials;        // [n_tiles][2]
	PartState* ps;           // written by block 0 (statistics)
	unsigned* bar_count;
	unsigned* bar_gen;
	int* err;
	double rtol, drop2;
	int max_iters;
	int timing_iters;        // > 0: run exactly this many iterations (autotuner)
	long polls;              // polls per grid barrier before it gives up
};

struct Shared {
	double gamma[MAX_PARTS], alpha[MAX_PARTS], beta[MAX_PARTS], rho_ref[MAX_PARTS], bnorm2[MAX_PARTS];
	int done[MAX_PARTS], repl[MAX_PARTS], iter[MAX_PARTS], status[MAX_PARTS], nrepl[MAX_PARTS];
	int active, any_repl, bar_ok;
	unsigned gen;
};

// grid-wide barrier with a bounded wait; returns false (and flags the
// error word) if the other blocks did not arrive in time.  Thread 0 arrives
// with one acquire-release atomic (the block's writes, ordered before it by
// __syncthreads, are released with it); the last to arrive resets the count
// and publishes the next generation with a release store (count and
// generation sit on separate 128-byte lines); the others poll it with
// acquire loads, checking the error word every 1024 polls.
__device__ bool grid_barrier(const BatchArgs& a, Shared& sh) {
	__syncthreads();
	if (threadIdx.x == 0) {
		unsigned const target = sh.gen + 1u;
		int ok = 1;
		unsigned arrived;
		asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(arrived) : "l"(a.bar_count) : "memory");
		if (arrived == gridDim.x - 1) {
			asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(a.bar_count) : "memory");
			asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.bar_gen), "r"(target) : "memory");
		}
		else {
			long spins = 0;
			unsigned cur;
			while (true) {
				asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(a.bar_gen) : "memory");
				if (cur == target) break;
				++spins;
				if (spins > a.polls || ((spins & 1023) == 0 && *(volatile int*) a.err != 0)) {
					atomicOr(a.err, BERR_BARRIER_TIMEOUT);
					ok = 0;
					break;
				}
			}
		}
		sh.gen = target;
		sh.bar_ok = ok && *(volatile int*) a.err == 0;
	}
	__syncthreads();
	return sh.bar_ok;
}

// sum of column `c` of the partials of part k's tiles, in tile order
__device__ __forceinline__ double part_sum(const BatchArgs& a, int k, int c) {
	double s = 0.0;
	for (int t = a.part_tile[k]; t < a.part_tile[k + 1]; t++) s += __ldcg(&a.partials[2 * t + c]);
	return s;
}

// block-wide sum of two doubles (all threads call; result valid in thread 0)
__device__ __forceinline__ void block_sum2(double& v0, double& v1) {
	__shared__ double red[BT / 32][2];
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int o = 16; o; o >>= 1) {
		v0 += __shfl_down_sync(0xffffffffu, v0, o);
		v1 += __shfl_down_sync(0xffffffffu, v1, o);
	}
	__syncthreads();
	if (lane == 0) {
		red[wid][0] = v0;
		red[wid][1] = v1;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		v0 = v1 = 0.0;
		for (int w = 0; w < BT / 32; w++) {
			v0 += red[w][0];
			v1 += red[w][1];
		}
	}
}

template <int LPR>
__global__ void __launch_bounds__(BT) k_batch_pcg(BatchArgs a) {
	extern __shared__ unsigned char smem_raw[];
	Shared& sh = *reinterpret_cast<Shared*>(smem_raw);
	int const sub = threadIdx.x % LPR;
	int const rows_per_pass = BT / LPR;
	if (threadIdx.x == 0) asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(sh.gen) : "l"(a.bar_gen) : "memory");
	__syncthreads();

	// ---- init: x = dx = p = 0, r = b; partials (b,b), (r, M r)
	for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
		double v0 = 0.0, v1 = 0.0;
		for (int i = a.tile_begin[t] + threadIdx.x; i < a.tile_end[t]; i += BT) {
			double2 const bb = ld2(a.b, i);
			float const r0 = (float) bb.x, r1 = (float) bb.y;
			float z0, z1;
			precond_apply(a.dinv, 0, i, r0, r1, z0, z1);
			st2(a.x, i, 0.0, 0.0);
			st2(a.dx, i, 0.f, 0.f);
			st2(a.r, i, r0, r1);
			st2(a.p0, i, 0.f, 0.f);
			v0 += bb.x * bb.x + bb.y * bb.y;
			v1 += (double) r0 * (double) z0 + (double) r1 * (double) z1;
		}
		block_sum2(v0, v1);
		if (threadIdx.x == 0) {
			a.partials[2 * t] = v0;
			a.partials[2 * t + 1] = v1;
		}
	}
	if (!grid_barrier(a, sh)) return;
	for (int k = threadIdx.x; k < a.n_parts; k += BT) {
		double const bn = part_sum(a, k, 0), g = part_sum(a, k, 1);
		sh.bnorm2[k] = bn;
		sh.gamma[k] = g;
		sh.beta[k] = 0.0;
		sh.alpha[k] = 0.0;
		sh.rho_ref[k] = bn;
		sh.done[k] = a.timing_iters > 0 ? 0 : bn == 0.0;
		sh.repl[k] = 0;
		sh.iter[k] = 0;
		sh.status[k] = BFM_GPU_OK;
		sh.nrepl[k] = 0;
	}
	__syncthreads();

	float* pc = a.p0;  // direction read this iteration
	float* pn = a.p1;  // direction written this iteration
	for (int it = 0;; it++) {
		if (threadIdx.x == 0) {
			int act = 0;
			for (int k = 0; k < a.n_parts; k++) act += !sh.done[k];
			sh.active = act;
		}
		__syncthreads();
		if (sh.active == 0 || (a.timing_iters > 0 && it >= a.timing_iters)) break;

		// ---- phase 1: q = A32 p' (difference form), p' = M r + beta p
		for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
			int const k = a.tile_part[t];
			if (sh.done[k]) continue;
			float const beta = (float) sh.beta[k];
			const float* __restrict__ r = a.r;
			const float* __restrict__ pp = pc;
			const float* __restrict__ dinv = a.dinv;
			auto gather = [=](int c, float& g0, float& g1) {
				float2 const rc = ld2(r, c), pv = ld2(pp, c);
				float z0, z1;
				precond_apply(dinv, 0, c, rc.x, rc.y, z0, z1);
				g0 = z0 + beta * pv.x;
				g1 = z1 + beta * pv.y;
			};
			DF pq = {0.f, 0.f};
			int const t0 = a.tile_begin[t], t1 = a.tile_end[t];
			for (int base = t0; base < t1; base += rows_per_pass) {
				int const row = base + threadIdx.x / LPR;
				bool const ok = row < t1;
				int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
				// difference form: q_r = S_r g_r + sum_c A_rc (g_c - g_r)
				float g0 = 0.f, g1 = 0.f;
				if (ok) gather(row, g0, g1);
				auto dgather = [=](int c, float& d0, float& d1) {
					gather(c, d0, d1);
					d0 -= g0;
					d1 -= g1;
				};
				float y0, y1;
				row_product<LPR, float>(a.cols, a.vals, ks, ke, sub, dgather, y0, y1);
				if (ok && sub == 0) {
					float4 const cc = reinterpret_cast<const float4*>(a.corr)[row];
					y0 += cc.x * g0 + cc.y * g1;
					y1 += cc.z * g0 + cc.w * g1;
					st2(pn, row, g0, g1);
					st2(a.q, row, y0, y1);
					df_add_prod(pq, g0, y0);
					df_add_prod(pq, g1, y1);
				}
			}
			double v0 = df_value(pq), v1 = 0.0;
			block_sum2(v0, v1);
			if (threadIdx.x == 0) a.partials[2 * t] = v0;
		}
		if (!grid_barrier(a, sh)) return;
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			if (sh.done[k]) continue;
			double const d = part_sum(a, k, 0);
			if (!(d > 0.0)) {
				sh.done[k] = a.timing_iters > 0 ? 0 : 1;
				sh.status[k] = BFM_GPU_BREAKDOWN;
				sh.alpha[k] = 0.0;
			}
			else {
				sh.alpha[k] = sh.gamma[k] / d;
			}
		}
		__syncthreads();

		// ---- phase 2: dx += alpha p', r -= alpha q; (r, M r), (r, r)
		for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
			int const k = a.tile_part[t];
			if (sh.done[k]) continue;
			float const alpha = (float) sh.alpha[k];
			DF g = {0.f, 0.f}, rr = {0.f, 0.f};
			for (int i = a.tile_begin[t] + threadIdx.x; i < a.tile_end[t]; i += BT) {
				float2 const pv = ld2(pn, i), qv = ld2(a.q, i), rv = ld2(a.r, i), d = ld2(a.dx, i);
				st2(a.dx, i, d.x + alpha * pv.x, d.y + alpha * pv.y);
				float const r0 = rv.x - alpha * qv.x, r1 = rv.y - alpha * qv.y;
				st2(a.r, i, r0, r1);
				float z0, z1;
				precond_apply(a.dinv, 0, i, r0, r1, z0, z1);
				df_add_prod(g, r0, z0);
				df_add_prod(g, r1, z1);
				df_add_prod(rr, r0, r0);
				df_add_prod(rr, r1, r1);
			}
			double v0 = df_value(g), v1 = df_value(rr);
			block_sum2(v0, v1);
			if (threadIdx.x == 0) {
				a.partials[2 * t] = v0;
				a.partials[2 * t + 1] = v1;
			}
		}
		if (!grid_barrier(a, sh)) return;
		if (threadIdx.x == 0) sh.any_repl = 0;
		__syncthreads();
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			sh.repl[k] = 0;
			if (sh.done[k]) continue;
			double const gamma = part_sum(a, k, 0), rho = part_sum(a, k, 1);
			double const tol2 = a.rtol * a.rtol * sh.bnorm2[k];
			sh.iter[k] += 1;
			sh.beta[k] = gamma / sh.gamma[k];
			sh.gamma[k] = gamma;
			if (a.timing_iters > 0) continue;
			if (sh.iter[k] >= a.max_iters) {
				sh.done[k] = 1;
				sh.status[k] = BFM_GPU_NOT_CONVERGED;
			}
			else if (!(gamma > 0.0) && gamma != 0.0) {
				sh.done[k] = 1;
				sh.status[k] = BFM_GPU_BREAKDOWN;
			}
			else if (gamma == 0.0 || rho <= a.drop2 * sh.rho_ref[k] || rho <= tol2) {
				sh.repl[k] = 1;
				atomicOr(&sh.any_repl, 1);
			}
		}
		__syncthreads();
		float* const tmp = pc;
		pc = pn;
		pn = tmp;
		if (!sh.any_repl) continue;

		// ---- FP64 residual replacement of the parts that asked for it
		for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
			int const k = a.tile_part[t];
			if (!sh.repl[k]) continue;
			for (int i = a.tile_begin[t] + threadIdx.x; i < a.tile_end[t]; i += BT) {
				float2 const d = ld2(a.dx, i);
				double2 const xv = ld2(a.x, i);
				st2(a.x, i, xv.x + (double) d.x, xv.y + (double) d.y);
				st2(a.dx, i, 0.f, 0.f);
			}
		}
		if (!grid_barrier(a, sh)) return;
		for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
			int const k = a.tile_part[t];
			if (!sh.repl[k]) continue;
			double v0 = 0.0, v1 = 0.0;
			int const t0 = a.tile_begin[t], t1 = a.tile_end[t];
			const double* __restrict__ xx = a.x;
			for (int base = t0; base < t1; base += rows_per_pass) {
				int const row = base + threadIdx.x / LPR;
				bool const ok = row < t1;
				int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
				double2 const xi = ok ? ld2(xx, row) : make_double2(0.0, 0.0);
				// FP64 operator as stored; the FP32 one in difference form
				double2 const x0 = a.vals64 ? make_double2(0.0, 0.0) : xi;
				auto gx = [xx, x0](int c, double& g0, double& g1) {
					double2 const v = ld2(xx, c);
					g0 = v.x - x0.x;
					g1 = v.y - x0.y;
				};
				double y0, y1;
				if (a.vals64) row_product<LPR, double>(a.cols, a.vals64, ks, ke, sub, gx, y0, y1);
				else row_product<LPR, double>(a.cols, a.vals, ks, ke, sub, gx, y0, y1);
				if (ok && sub == 0) {
					if (!a.vals64) {
						float4 const cc = reinterpret_cast<const float4*>(a.corr)[row];
						y0 += (double) cc.x * xi.x + (double) cc.y * xi.y;
						y1 += (double) cc.z * xi.x + (double) cc.w * xi.y;
					}
					double2 const bb = ld2(a.b, row);
					double const e0 = bb.x - y0, e1 = bb.y - y1;
					float const r0 = (float) e0, r1 = (float) e1;
					st2(a.r, row, r0, r1);
					float z0, z1;
					precond_apply(a.dinv, 0, row, r0, r1, z0, z1);
					v0 += e0 * e0 + e1 * e1;
					v1 += (double) r0 * (double) z0 + (double) r1 * (double) z1;
				}
			}
			block_sum2(v0, v1);
			if (threadIdx.x == 0) {
				a.partials[2 * t] = v0;
				a.partials[2 * t + 1] = v1;
			}
		}
		if (!grid_barrier(a, sh)) return;
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			if (!sh.repl[k]) continue;
			double const rr = part_sum(a, k, 0);
			sh.nrepl[k] += 1;
			sh.rho_ref[k] = rr;
			sh.gamma[k] = part_sum(a, k, 1);
			if (rr <= a.rtol * a.rtol * sh.bnorm2[k]) sh.done[k] = 1;
		}
		__syncthreads();
	}

	// ---- flush the grouped updates and record per-part statistics
	for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x)
		for (int i = a.tile_begin[t] + threadIdx.x; i < a.tile_end[t]; i += BT) {
			float2 const d = ld2(a.dx, i);
			double2 const xv = ld2(a.x, i);
			st2(a.x, i, xv.x + (double) d.x, xv.y + (double) d.y);
			st2(a.dx, i, 0.f, 0.f);
		}
	if (blockIdx.x == 0)
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			PartState& s = a.ps[k];
			s.bnorm2 = sh.bnorm2[k];
			s.gamma = sh.gamma[k];
			s.iter = sh.iter[k];
			s.status = sh.status[k];
			s.replacements = sh.nrepl[k];
			s.done = sh.done[k];
		}
}

// ||b - A x||^2 per part (FP64 operator), after the persistent solve
__global__ void __launch_bounds__(BT) k_batch_residual(BatchArgs a) {
	for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
		double v0 = 0.0, v1 = 0.0;
		for (int row = a.tile_begin[t] + threadIdx.x; row < a.tile_end[t]; row += BT) {
			double y0 = 0, y1 = 0;
			double2 const xi = ld2(a.x, row);
			double2 const x0 = a.vals64 ? make_double2(0.0, 0.0) : xi;  // difference form of the FP32 operator
			for (int k = a.row_ptr[row]; k < a.row_ptr[row + 1]; k++) {
				int const c = a.cols[k];
				double2 xc = ld2(a.x, c);
				xc.x -= x0.x;
				xc.y -= x0.y;
				double m0, m1, m2, m3;
				if (a.vals64) ld_block(a.vals64, k, m0, m1, m2, m3);
				else {
					float n0, n1, n2, n3;
					ld_block(a.vals, k, n0, n1, n2, n3);
					m0 = n0; m1 = n1; m2 = n2; m3 = n3;
				}
				y0 += m0 * xc.x + m1 * xc.y;
				y1 += m2 * xc.x + m3 * xc.y;
			}
			if (!a.vals64) {
				float4 const cc = reinterpret_cast<const float4*>(a.corr)[row];
				y0 += (double) cc.x * xi.x + (double) cc.y * xi.y;
				y1 += (double) cc.z * xi.x + (double) cc.w * xi.y;
			}
			double2 const bb = ld2(a.b, row);
			v0 += (bb.x - y0) * (bb.x - y0) + (bb.y - y1) * (bb.y - y1);
		}
		block_sum2(v0, v1);
		if (threadIdx.x == 0) a.partials[2 * t] = v0;
	}
}

__global__ void k_batch_part_residual(BatchArgs a) {
	int const k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.n_parts) return;
	a.ps[k].true_res2 = part_sum(a, k, 0);
}

}  // namespace

// ====================================================================== host side

namespace {

thread_local char g_berr[512];

int bfail(const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_berr, sizeof g_berr, fmt, ap);
	va_end(ap);
	bfm_gpu_set_last_error(g_berr);
	return -1;
}

#define BCK(call)                                                                                      \
	do {                                                                                               \
		cudaError_t const e_ = (call);                                                                 \
		if (e_ != cudaSuccess) return bfail("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
	} while (0)

struct BatchState {
	int n_parts;
	int* node_off_h;       // host copy of the part offsets
	int rows_per_tile, lpr, tuned;
	int n_tiles, grid;
	int *tile_part, *tile_begin, *tile_end, *part_tile;
	double* partials;
	PartState* ps;
	unsigned* bar;         // count (word 0), gen (word 32)
	int* err;
	cudaGraphExec_t graph;
	double g_rtol, g_drop;
	int g_iters, g_rpt, g_lpr;
	int64_t g_polls;
	float last_ms;
	int direct;            // 1: launched without a graph (capture unsupported)
	cudaEvent_t ev[2];
	// bfm_gpu_problem_step_parts: assembly + solve captured as one graph
	cudaGraphExec_t step_graph;
	int step_direct;       // capture unsupported here: the same work launched directly
	int s_precision, s_rpt, s_lpr;
	unsigned s_gen;
	bfm_gpu_opts_t s_opts;
};

void batch_free(void* p) {
	BatchState* B = (BatchState*) p;
	if (!B) return;
	void* d[] = {B->tile_part, B->tile_begin, B->tile_end, B->part_tile, B->partials, B->ps, B->bar, B->err};
	for (void* q : d)
		if (q) cudaFree(q);
	if (B->graph) cudaGraphExecDestroy(B->graph);
	if (B->step_graph) cudaGraphExecDestroy(B->step_graph);
	for (auto& e : B->ev)
		if (e) cudaEventDestroy(e);
	free(B->node_off_h);
	free(B);
}

BatchState* state_of(bfm_gpu_problem_t* P) { return (BatchState*) *bfmi_ext_slot(P, nullptr); }

// cut every part into tiles of at most `rpt` rows; upload the tile lists
int build_tiles(BatchState* B, int rpt) {
	int n = 0;
	for (int k = 0; k < B->n_parts; k++) {
		int const len = B->node_off_h[k + 1] - B->node_off_h[k];
		n += len > 0 ? (len + rpt - 1) / rpt : 0;
	}
	int* tp = (int*) malloc(sizeof(int) * (n + 1));
	int* tb = (int*) malloc(sizeof(int) * (n + 1));
	int* te = (int*) malloc(sizeof(int) * (n + 1));
	int* pt = (int*) malloc(sizeof(int) * (B->n_parts + 1));
	if (!tp || !tb || !te || !pt) {
		free(tp); free(tb); free(te); free(pt);
		return bfail("out of host memory");
	}
	int t = 0;
	for (int k = 0; k < B->n_parts; k++) {
		pt[k] = t;
		for (int r = B->node_off_h[k]; r < B->node_off_h[k + 1]; r += rpt) {
			tp[t] = k;
			tb[t] = r;
			te[t] = r + rpt < B->node_off_h[k + 1] ? r + rpt : B->node_off_h[k + 1];
			t++;
		}
	}
	pt[B->n_parts] = t;
	int rc = 0;
	if (n > B->n_tiles || !B->tile_part) {
		void* d[] = {B->tile_part, B->tile_begin, B->tile_end, B->partials};
		for (void* q : d)
			if (q) cudaFree(q);
		if (cudaMalloc(&B->tile_part, sizeof(int) * (n + 1)) != cudaSuccess ||
		    cudaMalloc(&B->tile_begin, sizeof(int) * (n + 1)) != cudaSuccess ||
		    cudaMalloc(&B->tile_end, sizeof(int) * (n + 1)) != cudaSuccess ||
		    cudaMalloc(&B->partials, sizeof(double) * 2 * (n + 1)) != cudaSuccess)
			rc = bfail("cudaMalloc failed for the tile lists");
	}
	if (!rc) {
		B->n_tiles = n;
		B->rows_per_tile = rpt;
		if (cudaMemcpy(B->tile_part, tp, sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
		    cudaMemcpy(B->tile_begin, tb, sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
		    cudaMemcpy(B->tile_end, te, sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
		    cudaMemcpy(B->part_tile, pt, sizeof(int) * (B->n_parts + 1), cudaMemcpyHostToDevice) != cudaSuccess)
			rc = bfail("cudaMemcpy failed for the tile lists");
	}
	free(tp); free(tb); free(te); free(pt);
	return rc;
}

void* kernel_of(int lpr) {
	switch (lpr) {
	case 1: return (void*) k_batch_pcg<1>;
	case 2: return (void*) k_batch_pcg<2>;
	default: return (void*) k_batch_pcg<4>;
	}
}

BatchArgs batch_args(bfm_gpu_problem_t* P, BatchState* B, const bfm_gpu_opts_t* o) {
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	BatchArgs a;
	memset(&a, 0, sizeof a);
	a.N = bf.N;
	a.n_parts = B->n_parts;
	a.n_tiles = B->n_tiles;
	a.tile_part = B->tile_part;
	a.tile_begin = B->tile_begin;
	a.tile_end = B->tile_end;
	a.part_tile = B->part_tile;
	a.row_ptr = bf.row_ptr;
	a.cols = bf.cols;
	a.vals = bf.vals32;
	a.corr = bf.corr32;
	a.dinv = bf.dinv32;
	a.vals64 = bf.vals64;
	a.b = bf.b;
	a.x = bf.x;
	a.r = (float*) bf.vec[0];
	a.dx = (float*) bf.vec[1];
	a.p0 = (float*) bf.vec[2];
	a.p1 = (float*) bf.vec[3];
	a.q = (float*) bf.vec[4];
	a.partials = B->partials;
	a.ps = B->ps;
	a.bar_count = B->bar;
	a.bar_gen = B->bar + 32;
	a.err = B->err;
	a.polls = SPIN_LIMIT;
	if (o) {
		a.rtol = o->rtol;
		a.drop2 = o->replace_drop * o->replace_drop;
		a.max_iters = o->max_iters;
		if (o->barrier_polls > 0) a.polls = (long) o->barrier_polls;
	}
	return a;
}

// blocks of the persistent kernel that fit on the GPU at once (cooperative launch)
int coop_grid(int lpr, int* grid) {
	int dev = 0, sms = 0, nb = 0;
	BCK(cudaGetDevice(&dev));
	BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	BCK(cudaFuncSetAttribute(kernel_of(lpr), cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(Shared)));
	BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel_of(lpr), BT, sizeof(Shared)));
	if (nb < 1) return bfail("the batch kernel does not fit on an SM");
	*grid = sms * nb;
	return 0;
}

int launch(BatchState* B, BatchArgs* a, int lpr, int grid, cudaStream_t st) {
	BCK(cudaMemsetAsync(B->bar, 0, 64 * sizeof(unsigned), st));
	BCK(cudaMemsetAsync(B->err, 0, sizeof(int), st));
	void* params[1] = {a};
	BCK(cudaLaunchCooperativeKernel(kernel_of(lpr), dim3(grid), dim3(BT), params, sizeof(Shared), st));
	k_batch_residual<<<grid, BT, 0, st>>>(*a);
	k_batch_part_residual<<<(B->n_parts + 127) / 128, 128, 0, st>>>(*a);
	BCK(cudaGetLastError());
	return 0;
}

// Project autotuner for the batch: rows per tile x lanes per row, each
// candidate timed over 10 iterations of the persistent kernel on the
// assembled batch (timing mode: no stopping test), fastest kept.
int autotune(bfm_gpu_problem_t* P, BatchState* B, const bfm_gpu_opts_t* o, cudaStream_t st) {
	int const rpts[] = {128, 256, 512, 1024};
	int const lprs[] = {1, 2, 4};
	float best = 1e30f;
	int best_rpt = 256, best_lpr = 2;
	for (int rpt : rpts) {
		if (build_tiles(B, rpt)) return -1;
		for (int lpr : lprs) {
			int grid = 0;
			if (coop_grid(lpr, &grid)) return -1;
			BatchArgs a = batch_args(P, B, o);
			a.timing_iters = 10;
			BCK(cudaEventRecord(B->ev[0], st));
			if (launch(B, &a, lpr, grid, st)) return -1;
			BCK(cudaEventRecord(B->ev[1], st));
			BCK(cudaStreamSynchronize(st));
			float ms = 0;
			BCK(cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]));
			int err = 0;
			BCK(cudaMemcpy(&err, B->err, sizeof err, cudaMemcpyDeviceToHost));
			if (err) return bfail("batch kernel barrier timed out during autotuning");
			if (ms < best) {
				best = ms;
				best_rpt = rpt;
				best_lpr = lpr;
			}
		}
	}
	if (build_tiles(B, best_rpt)) return -1;
	B->lpr = best_lpr;
	B->tuned = 1;
	return 0;
}

}  // namespace

extern "C" {

int bfm_gpu_problem_set_parts(bfm_gpu_problem_t* P, int n_parts, const int32_t* node_offsets) {
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	if (n_parts < 1 || n_parts > MAX_PARTS) return bfail("a batch holds 1 to %d parts, got %d", MAX_PARTS, n_parts);
	if (node_offsets[0] != 0 || node_offsets[n_parts] != bf.N) return bfail("part offsets must run from 0 to n_nodes");
	for (int k = 0; k < n_parts; k++)
		if (node_offsets[k + 1] < node_offsets[k]) return bfail("part offsets must be non-decreasing");
	void (*fn)(void*) = batch_free;
	void** slot = bfmi_ext_slot(P, &fn);
	if (*slot) batch_free(*slot);
	*slot = nullptr;
	BatchState* B = (BatchState*) calloc(1, sizeof(BatchState));
	if (!B) return bfail("out of host memory");
	*slot = B;
	B->n_parts = n_parts;
	B->node_off_h = (int*) malloc(sizeof(int) * (n_parts + 1));
	if (!B->node_off_h) return bfail("out of host memory");
	memcpy(B->node_off_h, node_offsets, sizeof(int) * (n_parts + 1));
	BCK(cudaMalloc(&B->part_tile, sizeof(int) * (n_parts + 1)));
	BCK(cudaMalloc(&B->ps, sizeof(PartState) * n_parts));
	BCK(cudaMalloc(&B->bar, 64 * sizeof(unsigned)));
	BCK(cudaMalloc(&B->err, sizeof(int)));
	BCK(cudaEventCreate(&B->ev[0]));
	BCK(cudaEventCreate(&B->ev[1]));
	B->lpr = 2;
	return build_tiles(B, 256);
}

int bfm_gpu_problem_solve_parts(bfm_gpu_problem_t* P, const bfm_gpu_opts_t* opts) {
	BFM_RANGE("bfm_gpu_problem_solve_parts");
	g_berr[0] = 0;
	BatchState* B = state_of(P);
	if (!B) return bfail("set the parts first (bfm_gpu_problem_set_parts)");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	if (!bf.assembled) return bfail("assemble before solving");
	if (bf.precision != BFM_GPU_MIXED && bf.precision != BFM_GPU_MIXED_EXACT)
		return bfail("the batched solver runs the mixed-precision iteration: assemble with BFM_GPU_MIXED or BFM_GPU_MIXED_EXACT");
	if (bf.precond != BFM_GPU_PC_JACOBI) return bfail("the batched solver uses the Jacobi preconditioner");
	bfm_gpu_opts_t o;
	if (opts) o = *opts;
	else bfm_gpu_default_opts(&o);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	if (o.autotune && !B->tuned) {
		if (autotune(P, B, &o, st)) return -1;
		if (B->graph) cudaGraphExecDestroy(B->graph);
		B->graph = nullptr;
	}
	bool const same = (B->graph || B->direct) && B->g_rtol == o.rtol && B->g_drop == o.replace_drop && B->g_iters == o.max_iters &&
	                  B->g_rpt == B->rows_per_tile && B->g_lpr == B->lpr && B->g_polls == o.barrier_polls;
	if (!same) {
		// one graph: reset of the barrier words, the persistent cooperative
		// kernel, the per-part FP64 residuals
		int grid = 0;
		if (coop_grid(B->lpr, &grid)) return -1;
		B->grid = grid;
		BatchArgs a = batch_args(P, B, &o);
		cudaStream_t cs;
		BCK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
		cudaGraph_t g = nullptr;
		int rc = 0;
		if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = bfail("stream capture failed");
		if (!rc) rc = launch(B, &a, B->lpr, grid, cs);
		cudaError_t const ec = cudaStreamEndCapture(cs, &g);
		cudaStreamDestroy(cs);
		if (!rc && ec != cudaSuccess) rc = bfail("stream capture failed: %s", cudaGetErrorString(ec));
		if (B->graph) cudaGraphExecDestroy(B->graph);
		B->graph = nullptr;
		if (!rc) {
			cudaError_t const ei = cudaGraphInstantiate(&B->graph, g, 0);
			if (ei != cudaSuccess) rc = bfail("graph instantiation failed: %s", cudaGetErrorString(ei));
		}
		if (g) cudaGraphDestroy(g);
		cudaGetLastError();
		if (rc) {
			// a driver that cannot capture cooperative launches: same work, launched directly
			B->graph = nullptr;
			B->direct = 1;
			g_berr[0] = 0;
			bfm_gpu_set_last_error("");
		}
		B->g_rtol = o.rtol;
		B->g_drop = o.replace_drop;
		B->g_iters = o.max_iters;
		B->g_rpt = B->rows_per_tile;
		B->g_lpr = B->lpr;
		B->g_polls = o.barrier_polls;
	}
	BCK(cudaEventRecord(B->ev[0], st));
	if (B->graph) {
		BCK(cudaGraphLaunch(B->graph, st));
	}
	else {
		BatchArgs a = batch_args(P, B, &o);
		if (launch(B, &a, B->lpr, B->grid, st)) return -1;
	}
	BCK(cudaEventRecord(B->ev[1], st));
	return 0;
}

int bfm_gpu_problem_step_parts(bfm_gpu_problem_t* P, int precision, const bfm_gpu_opts_t* opts) {
	BFM_RANGE("bfm_gpu_problem_step_parts");
	g_berr[0] = 0;
	BatchState* B = state_of(P);
	if (!B) return bfail("set the parts first (bfm_gpu_problem_set_parts)");
	if (precision != BFM_GPU_MIXED && precision != BFM_GPU_MIXED_EXACT)
		return bfail("the batched solver runs the mixed-precision iteration: BFM_GPU_MIXED or BFM_GPU_MIXED_EXACT");
	bfm_gpu_opts_t o;
	if (opts) o = *opts;
	else bfm_gpu_default_opts(&o);
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	bool const same = (B->step_graph || B->step_direct) && B->s_precision == precision && B->s_gen == bf.inputs_gen &&
	                  B->s_rpt == B->rows_per_tile && B->s_lpr == B->lpr && B->s_opts.rtol == o.rtol &&
	                  B->s_opts.max_iters == o.max_iters && B->s_opts.replace_drop == o.replace_drop &&
	                  B->s_opts.barrier_polls == o.barrier_polls && B->s_opts.autotune == o.autotune;
	if (!same) {
		// one step launched directly first: it sizes every buffer, tunes the
		// tile shape and leaves nothing for the capture to allocate
		if (bfm_gpu_problem_assemble(P, precision)) return -1;
		if (bfm_gpu_problem_solve_parts(P, &o)) return -1;
		BCK(cudaStreamSynchronize(st));
		if (B->step_graph) cudaGraphExecDestroy(B->step_graph);
		B->step_graph = nullptr;
		B->step_direct = 0;
		int grid = 0;
		if (coop_grid(B->lpr, &grid)) return -1;
		B->grid = grid;
		BatchArgs a = batch_args(P, B, &o);
		cudaGraph_t g = nullptr;
		int rc = 0;
		if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = bfail("stream capture failed");
		if (!rc) rc = bfm_gpu_problem_assemble(P, precision);
		if (!rc) {
			BatchArgs a2 = batch_args(P, B, &o);  // the assembly's buffers, unchanged
			a = a2;
			rc = launch(B, &a, B->lpr, grid, st);
		}
		cudaError_t const ec = cudaStreamEndCapture(st, &g);
		if (!rc && ec != cudaSuccess) rc = bfail("stream capture failed: %s", cudaGetErrorString(ec));
		if (!rc) {
			cudaError_t const ei = cudaGraphInstantiate(&B->step_graph, g, 0);
			if (ei != cudaSuccess) rc = bfail("graph instantiation failed: %s", cudaGetErrorString(ei));
		}
		if (g) cudaGraphDestroy(g);
		cudaGetLastError();
		if (rc) {
			// no capture of this work here: the same two calls, launched directly
			B->step_graph = nullptr;
			B->step_direct = 1;
			g_berr[0] = 0;
			bfm_gpu_set_last_error("");
		}
		B->s_precision = precision;
		B->s_gen = bf.inputs_gen;
		B->s_rpt = B->rows_per_tile;
		B->s_lpr = B->lpr;
		B->s_opts = o;
	}
	if (B->step_direct) {
		if (bfm_gpu_problem_assemble(P, precision)) return -1;
		return bfm_gpu_problem_solve_parts(P, &o);
	}
	BCK(cudaEventRecord(B->ev[0], st));
	BCK(cudaGraphLaunch(B->step_graph, st));
	BCK(cudaEventRecord(B->ev[1], st));
	return 0;
}

int bfm_gpu_problem_part_stats(bfm_gpu_problem_t* P, int* iterations, int* status, int* replacements, double* rel_residual,
                               int* rows_per_tile, int* lanes_per_row, double* ms_solve) {
	g_berr[0] = 0;
	BatchState* B = state_of(P);
	if (!B) return bfail("no parts set");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	BCK(cudaStreamSynchronize((cudaStream_t) bf.stream));
	int err = 0;
	BCK(cudaMemcpy(&err, B->err, sizeof err, cudaMemcpyDeviceToHost));
	if (err) return bfail("batch kernel: a grid barrier timed out (error word %d)", err);
	PartState* h = (PartState*) malloc(sizeof(PartState) * B->n_parts);
	if (!h) return bfail("out of host memory");
	cudaError_t const e = cudaMemcpy(h, B->ps, sizeof(PartState) * B->n_parts, cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) {
		free(h);
		return bfail("CUDA error %s", cudaGetErrorString(e));
	}
	for (int k = 0; k < B->n_parts; k++) {
		if (iterations) iterations[k] = h[k].iter;
		if (status) status[k] = h[k].status;
		if (replacements) replacements[k] = h[k].replacements;
		if (rel_residual) rel_residual[k] = h[k].bnorm2 > 0 ? sqrt(h[k].true_res2 / h[k].bnorm2) : 0.0;
	}
	free(h);
	if (rows_per_tile) *rows_per_tile = B->rows_per_tile;
	if (lanes_per_row) *lanes_per_row = B->lpr;
	if (ms_solve) {
		float ms = 0;
		cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]);
		*ms_solve = ms;
	}
	return 0;
}

}  // extern "C"
