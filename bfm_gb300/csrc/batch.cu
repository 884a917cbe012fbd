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
//
// Two-level block Jacobi (BFM_GPU_PC_TWO_LEVEL_JACOBI): M^-1 = D^-1 + P A_c^-1
// P^T per part, D the 2x2 diagonal blocks, P the rigid-body modes of the
// cells of a grid over the part's bounding box.  A_c = P^T A P (FP64 sums of
// the FP32 operator in difference form) and A_c^-1 (FP32 Cholesky of the
// diagonally scaled A_c, X = L^-1, X^T X) are formed per step by three
// set-up kernels; per iteration, after phase 2 and after a replacement:
//   stage R  one warp per cell: r_c = P^T r;                                barrier
//   stage Y  one block per chunk of a part's cells: their rows of
//            y_c = A_c^-1 r_c, P y_c at their nodes, a partial (r_c, y_c);   barrier
// and z = D^-1 r + P y_c is formed where phase 1 gathers it.
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
constexpr int BC_MAX_CELLS = 64;       // two-level: coarse cells per part
constexpr int BC_MAX_N = 3 * BC_MAX_CELLS;  // coarse DOFs per part
constexpr int BC_INV_T = 1024;         // threads of the coarse inverse kernel
constexpr int BC_CHUNK = 10;           // cells per work item of stage Y (30 rows of A_c^-1)

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
	int block_pc;            // dinv holds each node's inverse 2x2 diagonal block
	// two-level correction (k_batch_pcg<LPR, true>)
	int n_cells;
	const int* part_cell;    // cells of part k: [part_cell[k], part_cell[k+1])
	const int* cell_part;
	const int* cell_ptr;     // nodes of cell c: cell_nodes[cell_ptr[c] .. cell_ptr[c+1])
	const int* cell_nodes;
	const int* node_cell;
	const float4* pnode;     // per node: offset (dx, dy) from its cell's centre over H, free flags
	const float* ainv;       // per part: A_c^-1, dense (3 cells)^2 FP32, from ainv_off[k]
	const long long* ainv_off;
	double* rc;              // r_c = P^T r, 3 per cell
	float2* zc;              // P y_c per node (y_c = A_c^-1 r_c, rounded to FP32)
	int n_chunks;            // stage Y's work items: BC_CHUNK consecutive cells of one part
	const int* chunk_part;
	const int* chunk_cell;   // first cell of the chunk
	const int* part_chunk;   // chunks of part k: [part_chunk[k], part_chunk[k+1])
	double* cdot;            // per chunk: its share of (r_c, y_c), the coarse part of (r, M r)
	// block-per-part kernel (k_batch_block)
	const int* node_off;     // nodes of part k: [node_off[k], node_off[k+1])
	const int* block_part;   // the part of each block (largest parts first)
	float* z;                // z = M r, materialized per node
};

struct Shared {
	double gamma[MAX_PARTS], alpha[MAX_PARTS], beta[MAX_PARTS], rho_ref[MAX_PARTS], bnorm2[MAX_PARTS];
	int done[MAX_PARTS], repl[MAX_PARTS], iter[MAX_PARTS], status[MAX_PARTS], nrepl[MAX_PARTS];
	double rcs[BC_MAX_N];                  // two-level: the part's r_c
	double ydot[3 * BC_CHUNK];             //   terms of (r_c, y_c) of a chunk's rows
	float ys[3 * BC_CHUNK];                //   the chunk's rows of y_c
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

// sum of column `c` of the partials of part k's tiles, in tile order (loads
// four at a time)
__device__ __forceinline__ double part_sum(const BatchArgs& a, int k, int c) {
	double s = 0.0;
	int t = a.part_tile[k];
	int const e = a.part_tile[k + 1];
	for (; t + 4 <= e; t += 4) {
		double const v0 = __ldcg(&a.partials[2 * t + c]), v1 = __ldcg(&a.partials[2 * t + 2 + c]);
		double const v2 = __ldcg(&a.partials[2 * t + 4 + c]), v3 = __ldcg(&a.partials[2 * t + 6 + c]);
		s += v0;
		s += v1;
		s += v2;
		s += v3;
	}
	for (; t < e; t++) s += __ldcg(&a.partials[2 * t + c]);
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

// Stage R: r_c = P^T r for every cell of a part still iterating.  One warp
// per cell, lanes over the cell's nodes, double sums in lane order and a
// fixed shuffle tree (deterministic).  P_i = [[f0, 0, -f0 dy], [0, f1, f1 dx]].
__device__ void coarse_restrict(const BatchArgs& a, const Shared& sh) {
	int const lane = threadIdx.x & 31;
	int const nw = gridDim.x * (BT / 32);
	for (int c = blockIdx.x * (BT / 32) + (threadIdx.x >> 5); c < a.n_cells; c += nw) {
		if (sh.done[a.cell_part[c]]) continue;
		double s0 = 0.0, s1 = 0.0, s2 = 0.0;
		int const end = a.cell_ptr[c + 1];
		for (int k0 = a.cell_ptr[c] + lane; k0 < end; k0 += 128) {
			// four nodes per lane in flight, summed in node-list order
			int id[4];
			float2 rv[4];
			float4 pq[4];
#pragma unroll
			for (int u = 0; u < 4; u++) id[u] = k0 + 32 * u < end ? a.cell_nodes[k0 + 32 * u] : -1;
#pragma unroll
			for (int u = 0; u < 4; u++) {
				rv[u] = id[u] >= 0 ? __ldcg(reinterpret_cast<const float2*>(a.r) + id[u]) : make_float2(0.f, 0.f);
				pq[u] = id[u] >= 0 ? a.pnode[id[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
			}
#pragma unroll
			for (int u = 0; u < 4; u++) {
				if (id[u] < 0) continue;
				double const x0 = pq[u].z != 0.f ? (double) rv[u].x : 0.0, x1 = pq[u].w != 0.f ? (double) rv[u].y : 0.0;
				s0 += x0;
				s1 += x1;
				s2 += (double) pq[u].x * x1 - (double) pq[u].y * x0;
			}
		}
		for (int o = 16; o; o >>= 1) {
			s0 += __shfl_xor_sync(0xffffffffu, s0, o);
			s1 += __shfl_xor_sync(0xffffffffu, s1, o);
			s2 += __shfl_xor_sync(0xffffffffu, s2, o);
		}
		if (lane == 0) {
			a.rc[3l * c] = s0;
			a.rc[3l * c + 1] = s1;
			a.rc[3l * c + 2] = s2;
		}
	}
}

// Stage Y, one block per work item (BC_CHUNK consecutive cells of one part
// still iterating): the part's r_c staged in shared memory; the chunk's rows
// of y_c = A_c^-1 r_c, one warp per row (lanes over columns, four loads in
// flight, fixed shuffle tree), rounded to FP32; P y_c written at the chunk's
// nodes (their lists are contiguous: cells are listed in order); and the
// chunk's share of (r_c, y_c) of the rounded values, in row order.
__device__ void coarse_solve(const BatchArgs& a, Shared& sh) {
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int q = blockIdx.x; q < a.n_chunks; q += gridDim.x) {
		int const k = a.chunk_part[q];
		if (sh.done[k]) continue;  // the same in every thread of the block
		int const c0 = a.part_cell[k], n = 3 * (a.part_cell[k + 1] - c0);
		int const cq = a.chunk_cell[q], ce = min(cq + BC_CHUNK, a.part_cell[k + 1]);
		int const row0 = 3 * (cq - c0), rows = 3 * (ce - cq);
		__syncthreads();  // the previous item's shared arrays are read
		for (int u = threadIdx.x; u < n; u += BT) sh.rcs[u] = __ldcg(a.rc + 3l * c0 + u);
		__syncthreads();
		const float* __restrict__ A = a.ainv + a.ainv_off[k];
		for (int i = warp; i < rows; i += BT / 32) {
			const float* __restrict__ Ar = A + (long) (row0 + i) * n;
			double s = 0.0;
			for (int j0 = lane; j0 < n; j0 += 128) {
				float v[4];
#pragma unroll
				for (int u = 0; u < 4; u++) v[u] = j0 + 32 * u < n ? __ldg(Ar + j0 + 32 * u) : 0.f;
#pragma unroll
				for (int u = 0; u < 4; u++)
					if (j0 + 32 * u < n) s += (double) v[u] * sh.rcs[j0 + 32 * u];
			}
			for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
			float const y = (float) s;
			if (lane == 0) {
				sh.ys[i] = y;
				sh.ydot[i] = (double) y * sh.rcs[row0 + i];
			}
		}
		__syncthreads();
		for (int t = a.cell_ptr[cq] + threadIdx.x; t < a.cell_ptr[ce]; t += BT) {
			int const i = a.cell_nodes[t];
			int const l = 3 * (a.node_cell[i] - cq);
			float4 const pq = a.pnode[i];
			float const y0 = sh.ys[l], y1 = sh.ys[l + 1], y2 = sh.ys[l + 2];
			a.zc[i] = make_float2(pq.z * (y0 - pq.y * y2), pq.w * (y1 + pq.x * y2));
		}
		if (warp == 0) {
			double d = lane < rows ? sh.ydot[lane] : 0.0;
			for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
			if (lane == 0) a.cdot[q] = d;
		}
	}
}

// the coarse share of (r, M r) of part k, its chunks in order (zero for
// one-level Jacobi)
template <bool TWO>
__device__ __forceinline__ double coarse_gamma(const BatchArgs& a, int k) {
	if (!TWO) return 0.0;
	double s = 0.0;
	for (int q = a.part_chunk[k]; q < a.part_chunk[k + 1]; q++) s += __ldcg(a.cdot + q);
	return s;
}

template <int LPR, bool TWO>
__global__ void __launch_bounds__(BT) k_batch_pcg(BatchArgs a) {
	extern __shared__ unsigned char smem_raw[];
	Shared& sh = *reinterpret_cast<Shared*>(smem_raw);
	int const sub = threadIdx.x % LPR;
	int const rows_per_pass = BT / LPR;
	if (threadIdx.x == 0) asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(sh.gen) : "l"(a.bar_gen) : "memory");
	for (int k = threadIdx.x; k < a.n_parts; k += BT) sh.done[k] = 0;  // the init's coarse stages run every part
	__syncthreads();

	// ---- init: x = dx = p = 0, r = b; partials (b,b), (r, M r)
	for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
		double v0 = 0.0, v1 = 0.0;
		for (int i = a.tile_begin[t] + threadIdx.x; i < a.tile_end[t]; i += BT) {
			double2 const bb = ld2(a.b, i);
			float const r0 = (float) bb.x, r1 = (float) bb.y;
			float z0, z1;
			precond_apply(a.dinv, a.block_pc, i, r0, r1, z0, z1);
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
	if (TWO) {
		coarse_restrict(a, sh);
		if (!grid_barrier(a, sh)) return;
		coarse_solve(a, sh);
		if (!grid_barrier(a, sh)) return;
	}
	for (int k = threadIdx.x; k < a.n_parts; k += BT) {
		double const bn = part_sum(a, k, 0), g = part_sum(a, k, 1) + coarse_gamma<TWO>(a, k);
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
			int const bpc = a.block_pc;
			const float2* zcv = a.zc;
			// z = D^-1 r (+ P y_c, two-level), then p' = z + beta p
			auto gather = [=](int c, float& g0, float& g1) {
				float2 const rc = ld2(r, c), pv = ld2(pp, c);
				float z0, z1;
				precond_apply(dinv, bpc, c, rc.x, rc.y, z0, z1);
				if (TWO) {
					float2 const zv = __ldcg(zcv + c);
					z0 += zv.x;
					z1 += zv.y;
				}
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
				precond_apply(a.dinv, a.block_pc, i, r0, r1, z0, z1);
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
		if (TWO) {
			coarse_restrict(a, sh);
			if (!grid_barrier(a, sh)) return;
			coarse_solve(a, sh);
			if (!grid_barrier(a, sh)) return;
		}
		if (threadIdx.x == 0) sh.any_repl = 0;
		__syncthreads();
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			sh.repl[k] = 0;
			if (sh.done[k]) continue;
			double const gamma = part_sum(a, k, 0) + coarse_gamma<TWO>(a, k), rho = part_sum(a, k, 1);
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
					precond_apply(a.dinv, a.block_pc, row, r0, r1, z0, z1);
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
		if (TWO) {
			coarse_restrict(a, sh);
			if (!grid_barrier(a, sh)) return;
			coarse_solve(a, sh);
			if (!grid_barrier(a, sh)) return;
		}
		for (int k = threadIdx.x; k < a.n_parts; k += BT) {
			if (!sh.repl[k]) continue;
			double const rr = part_sum(a, k, 0);
			sh.nrepl[k] += 1;
			sh.rho_ref[k] = rr;
			sh.gamma[k] = part_sum(a, k, 1) + coarse_gamma<TWO>(a, k);
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

// ====================================================================== block per part
//
// k_batch_block: one thread block runs one part's whole PCG -- the same
// mixed-precision iteration as k_batch_pcg (FP32 operator in difference form
// and FP32 vectors, FP64 inner products from double-float partial sums, FP64
// residual replacements, the same stopping rules) -- with block barriers only:
// no grid barrier, no spin wait, no cooperative launch.  Blocks take the
// parts largest first (block_part), so the longest solves start first.  With
// TWO, z = D^-1 r + P A_c^-1 P^T r is formed in three block-local stages:
// r_c = P^T r (a warp per cell, into shared memory), y_c = A_c^-1 r_c (a warp
// per row of A_c^-1, into shared memory), z at every node.  All sums are in a
// fixed order (lane strided, shuffle trees, warps in order): deterministic.

constexpr int BB_MAX_T = 1024;
constexpr int BB_MAX_NODES = 131072;  // larger parts go to the tiled persistent kernel

// block-wide sum of per-thread doubles (every thread calls, every thread gets
// the result), one barrier: each warp's shuffle sum goes to a slot of a
// double-buffered array (`ph` alternates with every call, the same in every
// thread), then every warp reduces the slots in the same fixed shuffle tree
// (deterministic).  A buffer is rewritten two calls later, after the next
// call's barrier, when every thread has read it.
__device__ __forceinline__ double bb_sum(double v, int& ph) {
	__shared__ double red[2][BB_MAX_T / 32];
	int const lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
	for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	if (lane == 0) red[ph][w] = v;
	__syncthreads();
	double t = lane < nw ? red[ph][lane] : 0.0;
	for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
	ph ^= 1;
	return t;
}

// z = M r over the part's nodes [n0, n1), returns (r, z) (block-wide).  The
// coarse stages sum in double-float on the FP32 pipe (GB300 issues FP64 at a
// small fraction of that rate): r_c = P^T r per cell, y_c = A_c^-1 r_c.
template <bool TWO>
__device__ double bb_apply_m(const BatchArgs& a, int k, int n0, int n1, float2* rcs, float* ys, int& ph) {
	int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	int c0 = 0;
	if (TWO) {
		c0 = a.part_cell[k];
		int const c1 = a.part_cell[k + 1], n = 3 * (c1 - c0);
		// r_c = P^T r, a warp per cell (four nodes per lane in flight, summed in list order)
		for (int c = c0 + warp; c < c1; c += nw) {
			dfl s0 = {0.f, 0.f}, s1 = {0.f, 0.f}, s2 = {0.f, 0.f};
			int const end = a.cell_ptr[c + 1];
			for (int k0 = a.cell_ptr[c] + lane; k0 < end; k0 += 128) {
				int id[4];
				float2 rv[4];
				float4 pq[4];
#pragma unroll
				for (int u = 0; u < 4; u++) id[u] = k0 + 32 * u < end ? a.cell_nodes[k0 + 32 * u] : -1;
#pragma unroll
				for (int u = 0; u < 4; u++) {
					rv[u] = id[u] >= 0 ? __ldcg(reinterpret_cast<const float2*>(a.r) + id[u]) : make_float2(0.f, 0.f);
					pq[u] = id[u] >= 0 ? a.pnode[id[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
				}
#pragma unroll
				for (int u = 0; u < 4; u++) {
					if (id[u] < 0) continue;
					float const x0 = pq[u].z != 0.f ? rv[u].x : 0.f, x1 = pq[u].w != 0.f ? rv[u].y : 0.f;
					s0 = df_add(s0, {x0, 0.f});
					s1 = df_add(s1, {x1, 0.f});
					s2 = df_add(s2, df_add(df_mul_f(pq[u].x, {x1, 0.f}), df_neg(df_mul_f(pq[u].y, {x0, 0.f}))));
				}
			}
			for (int o = 16; o; o >>= 1) {
				s0 = df_add(s0, {__shfl_xor_sync(0xffffffffu, s0.hi, o), __shfl_xor_sync(0xffffffffu, s0.lo, o)});
				s1 = df_add(s1, {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)});
				s2 = df_add(s2, {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)});
			}
			if (lane == 0) {
				rcs[3 * (c - c0)] = make_float2(s0.hi, s0.lo);
				rcs[3 * (c - c0) + 1] = make_float2(s1.hi, s1.lo);
				rcs[3 * (c - c0) + 2] = make_float2(s2.hi, s2.lo);
			}
		}
		__syncthreads();
		// y_c = A_c^-1 r_c, a warp per row, rounded to FP32
		const float* __restrict__ A = a.ainv + a.ainv_off[k];
		for (int i = warp; i < n; i += nw) {
			const float* __restrict__ Ar = A + (long) i * n;
			dfl s = {0.f, 0.f};
			for (int j0 = lane; j0 < n; j0 += 128) {
				float v[4];
#pragma unroll
				for (int u = 0; u < 4; u++) v[u] = j0 + 32 * u < n ? __ldg(Ar + j0 + 32 * u) : 0.f;
#pragma unroll
				for (int u = 0; u < 4; u++)
					if (j0 + 32 * u < n) {
						float2 const rj = rcs[j0 + 32 * u];
						s = df_add(s, df_mul_f(v[u], {rj.x, rj.y}));
					}
			}
			for (int o = 16; o; o >>= 1) s = df_add(s, {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
			if (lane == 0) ys[i] = s.hi + s.lo;
		}
		__syncthreads();
	}
	DF g = {0.f, 0.f};
	#pragma unroll 4
	for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
		float2 const rv = __ldcg(reinterpret_cast<const float2*>(a.r) + i);
		float z0, z1;
		precond_apply(a.dinv, a.block_pc, i, rv.x, rv.y, z0, z1);
		if (TWO) {
			int const l = 3 * (a.node_cell[i] - c0);
			float4 const pq = a.pnode[i];
			z0 += pq.z * (ys[l] - pq.y * ys[l + 2]);
			z1 += pq.w * (ys[l + 1] + pq.x * ys[l + 2]);
		}
		st2(a.z, i, z0, z1);
		df_add_prod(g, rv.x, z0);
		df_add_prod(g, rv.y, z1);
	}
	return bb_sum(df_value(g), ph);
}

template <int LPR, bool TWO>
__global__ void __launch_bounds__(BB_MAX_T) k_batch_block(BatchArgs a) {
	__shared__ float2 rcs[BC_MAX_N];  // r_c as double-float pairs
	__shared__ float ys[BC_MAX_N];
	int const k = a.block_part[blockIdx.x];
	int const n0 = a.node_off[k], n1 = a.node_off[k + 1];
	int const sub = threadIdx.x % LPR;
	int const rows_per_pass = blockDim.x / LPR;
	// ---- init: x = dx = p = 0, r = b, z = M r
	double bb = 0.0;
	for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
		double2 const bv = ld2(a.b, i);
		st2(a.x, i, 0.0, 0.0);
		st2(a.dx, i, 0.f, 0.f);
		st2(a.r, i, (float) bv.x, (float) bv.y);
		st2(a.p0, i, 0.f, 0.f);
		bb += bv.x * bv.x + bv.y * bv.y;
	}
	int ph = 0;  // bb_sum's buffer, the same in every thread
	double const bnorm2 = bb_sum(bb, ph);  // its barrier also orders the stores above
	double gamma = bb_apply_m<TWO>(a, k, n0, n1, rcs, ys, ph);
	double beta = 0.0, rho_ref = bnorm2;
	double const tol2 = a.rtol * a.rtol * bnorm2;
	int iter = 0, status = BFM_GPU_OK, nrepl = 0;
	bool done = a.timing_iters > 0 ? false : bnorm2 == 0.0;
	float* const p = a.p0;
	while (!done) {
		if (a.timing_iters > 0 && iter >= a.timing_iters) break;
		// p = z + beta p
		float const fb = (float) beta;
		#pragma unroll 4
		for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
			float2 const zv = ld2(a.z, i), pv = ld2(p, i);
			st2(p, i, zv.x + fb * pv.x, zv.y + fb * pv.y);
		}
		__syncthreads();
		// q = A32 p in difference form, (p, q); two rows per thread per pass
		// (independent gathers in flight), summed into (p, q) in row order
		DF pq = {0.f, 0.f};
		for (int base = n0; base < n1; base += 2 * rows_per_pass) {
			int rw[2], ks[2], ke[2];
			bool ok[2];
			float2 pr[2];
#pragma unroll
			for (int h = 0; h < 2; h++) {
				rw[h] = base + h * rows_per_pass + (int) threadIdx.x / LPR;
				ok[h] = rw[h] < n1;
				ks[h] = ok[h] ? a.row_ptr[rw[h]] : 0;
				ke[h] = ok[h] ? a.row_ptr[rw[h] + 1] : 0;
				pr[h] = ok[h] ? __ldcg(reinterpret_cast<const float2*>(p) + rw[h]) : make_float2(0.f, 0.f);
			}
			float y0[2], y1[2];
#pragma unroll
			for (int h = 0; h < 2; h++) {
				float2 const prh = pr[h];
				auto dg = [=](int c, float& d0, float& d1) {
					float2 const pc = __ldcg(reinterpret_cast<const float2*>(p) + c);
					d0 = pc.x - prh.x;
					d1 = pc.y - prh.y;
				};
				row_product_pf<LPR, 4, float>(a.cols, a.vals, ks[h], ke[h], sub, dg, y0[h], y1[h]);
			}
#pragma unroll
			for (int h = 0; h < 2; h++) {
				if (ok[h] && sub == 0) {
					float4 const cc = reinterpret_cast<const float4*>(a.corr)[rw[h]];
					float const q0 = y0[h] + cc.x * pr[h].x + cc.y * pr[h].y;
					float const q1 = y1[h] + cc.z * pr[h].x + cc.w * pr[h].y;
					st2(a.q, rw[h], q0, q1);
					df_add_prod(pq, pr[h].x, q0);
					df_add_prod(pq, pr[h].y, q1);
				}
			}
		}
		double const d = bb_sum(df_value(pq), ph);
		if (!(d > 0.0) && a.timing_iters == 0) {
			status = BFM_GPU_BREAKDOWN;
			break;
		}
		float const alpha = d > 0.0 ? (float) (gamma / d) : 0.f;
		// dx += alpha p, r -= alpha q, (r, r)
		DF rr = {0.f, 0.f};
		#pragma unroll 4
		for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
			float2 const pv = ld2(p, i), qv = ld2(a.q, i), rv = ld2(a.r, i), dv = ld2(a.dx, i);
			st2(a.dx, i, dv.x + alpha * pv.x, dv.y + alpha * pv.y);
			float const r0 = rv.x - alpha * qv.x, r1 = rv.y - alpha * qv.y;
			st2(a.r, i, r0, r1);
			df_add_prod(rr, r0, r0);
			df_add_prod(rr, r1, r1);
		}
		double const rho = bb_sum(df_value(rr), ph);
		iter++;
		double const gnew = bb_apply_m<TWO>(a, k, n0, n1, rcs, ys, ph);
		beta = gamma != 0.0 ? gnew / gamma : 0.0;
		gamma = gnew;
		if (a.timing_iters > 0) continue;
		if (iter >= a.max_iters) {
			status = BFM_GPU_NOT_CONVERGED;
			break;
		}
		if (!(gnew > 0.0) && gnew != 0.0) {
			status = BFM_GPU_BREAKDOWN;
			break;
		}
		if (gnew == 0.0 || rho <= a.drop2 * rho_ref || rho <= tol2) {
			// FP64 residual replacement: x += dx, r = b - A x in FP64
			for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
				float2 const dv = ld2(a.dx, i);
				double2 const xv = ld2(a.x, i);
				st2(a.x, i, xv.x + (double) dv.x, xv.y + (double) dv.y);
				st2(a.dx, i, 0.f, 0.f);
			}
			__syncthreads();
			double e2 = 0.0;
			const double* __restrict__ xx = a.x;
			for (int base = n0; base < n1; base += rows_per_pass) {
				int const row = base + (int) threadIdx.x / LPR;
				bool const ok = row < n1;
				int const ks = ok ? a.row_ptr[row] : 0, ke = ok ? a.row_ptr[row + 1] : 0;
				double2 const xi = ok ? __ldcg(reinterpret_cast<const double2*>(xx) + row) : make_double2(0.0, 0.0);
				double2 const x0 = a.vals64 ? make_double2(0.0, 0.0) : xi;
				auto gx = [xx, x0](int c, double& g0, double& g1) {
					double2 const v = __ldcg(reinterpret_cast<const double2*>(xx) + c);
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
					double2 const bv = ld2(a.b, row);
					double const e0 = bv.x - y0, e1 = bv.y - y1;
					st2(a.r, row, (float) e0, (float) e1);
					e2 += e0 * e0 + e1 * e1;
				}
			}
			double const r2 = bb_sum(e2, ph);
			nrepl++;
			rho_ref = r2;
			gamma = bb_apply_m<TWO>(a, k, n0, n1, rcs, ys, ph);
			if (r2 <= tol2) break;
		}
	}
	// flush the grouped update; statistics
	__syncthreads();
	for (int i = n0 + threadIdx.x; i < n1; i += blockDim.x) {
		float2 const dv = ld2(a.dx, i);
		double2 const xv = ld2(a.x, i);
		st2(a.x, i, xv.x + (double) dv.x, xv.y + (double) dv.y);
		st2(a.dx, i, 0.f, 0.f);
	}
	if (threadIdx.x == 0) {
		PartState& s = a.ps[k];
		s.bnorm2 = bnorm2;
		s.gamma = gamma;
		s.iter = iter;
		s.status = status;
		s.replacements = nrepl;
		s.done = 1;
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

// ---- two-level set-up, per step (after the assembly, inside the step's graph)

struct CoarseSetArgs {
	int N, n_cells;
	const int* part_cell;
	const int* cell_ptr;
	const int* cell_nodes;
	const int* node_cell;
	const int* cell_nbr;   // 9 per cell: the cell at grid offset (dx, dy) in slot 3 (dy + 1) + dx + 1, -1 outside
	const int2* cell_xy;   // per cell: its position in its part's grid
	const float2* dxdy;    // per node: offset from its cell's centre over H (FP32)
	const int* last_ci;    // per DOF: >= 0 when a Dirichlet condition eliminates it
	float4* pnode;
	const int* row_ptr;
	const int* cols;
	const float* vals;     // the FP32 iteration operator, applied in difference form:
	const float* corr;     //   (K g)_r = S_r g_r + sum_c K_rc (g_c - g_r)
	double* ac;            // 81 per cell: the 3x3 blocks A_c(I, J) of its 9 slots
	float* ainv;
	const long long* ainv_off;
};

// per node: (dx, dy, f0, f1), f = 0 for an eliminated DOF (its row of P is zero)
__global__ void k_bpnode(CoarseSetArgs a) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.N) return;
	float2 const d = a.dxdy[i];
	a.pnode[i] = make_float4(d.x, d.y, a.last_ci[2 * i] < 0 ? 1.f : 0.f, a.last_ci[2 * i + 1] < 0 ? 1.f : 0.f);
}

// A_c(I, J) = sum over the nodes r of cell I of P_r^T (K P^(J))_r, with the
// operator in difference form: (K P^(J))_r = S_r P^(J)_r + sum_{c != r}
// K_rc (P^(J)_c - P^(J)_r), P^(J)_c = P_c when c lies in cell J, else 0.
// One warp per (cell, slot), lanes over the cell's nodes, FP64 sums per lane
// then a fixed shuffle tree (deterministic).  Translations of interior nodes
// cancel exactly in the differences, so no large terms cancel in the sums.
__global__ void k_bcoarse_ac(CoarseSetArgs a) {
	long const t = ((long) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	int const lane = threadIdx.x & 31;
	if (t >= 9l * a.n_cells) return;
	int const I = (int) (t / 9), slot = (int) (t % 9);
	int const J = a.cell_nbr[9l * I + slot];
	double acc[9];
#pragma unroll
	for (int e = 0; e < 9; e++) acc[e] = 0.0;
	if (J >= 0) {
		bool const same = J == I;
		for (int k = a.cell_ptr[I] + lane; k < a.cell_ptr[I + 1]; k += 32) {
			int const r = a.cell_nodes[k];
			double pr[2][3], prj[2][3];
			p_block(a.pnode[r], true, pr);
			p_block(a.pnode[r], same, prj);
			if (same) {
				float4 const S = reinterpret_cast<const float4*>(a.corr)[r];
				acc_ptmd(acc, pr, S.x, S.y, S.z, S.w, prj);
			}
			for (int kb = a.row_ptr[r]; kb < a.row_ptr[r + 1]; kb++) {
				int const c = a.cols[kb];
				if (c == r) continue;
				bool const inJ = a.node_cell[c] == J;
				if (!inJ && !same) continue;  // P^(J) is zero at both ends
				double pc[2][3], d[2][3];
				p_block(a.pnode[c], inJ, pc);
#pragma unroll
				for (int u = 0; u < 2; u++)
#pragma unroll
					for (int b = 0; b < 3; b++) d[u][b] = pc[u][b] - prj[u][b];
				float4 const K = reinterpret_cast<const float4*>(a.vals)[kb];
				acc_ptmd(acc, pr, K.x, K.y, K.z, K.w, d);
			}
		}
	}
#pragma unroll
	for (int e = 0; e < 9; e++)
		for (int o = 16; o; o >>= 1) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], o);
	if (lane == 0) {
		double* o = a.ac + 81l * I + 9 * slot;
#pragma unroll
		for (int e = 0; e < 9; e++) o[e] = acc[e];
	}
}

// entry (i, j) of a part's A_c (cells from c0), 0 where the cells are not neighbours
__device__ __forceinline__ double ac_entry(const CoarseSetArgs& a, int c0, int i, int j) {
	int const I = c0 + i / 3, J = c0 + j / 3;
	int2 const pi = a.cell_xy[I], pj = a.cell_xy[J];
	int const dx = pj.x - pi.x, dy = pj.y - pi.y;
	if (dx < -1 || dx > 1 || dy < -1 || dy > 1) return 0.0;
	return a.ac[81l * I + 9 * (3 * (dy + 1) + dx + 1) + 3 * (i % 3) + j % 3];
}

// A_c^-1 of one part per block, in FP32 in shared memory: symmetric
// diagonal scaling s_i = A_ii^-1/2 (in FP64), Cholesky of the scaled matrix
// (a pivot below 1e-5 drops its coarse DOF: a cell without free nodes, or a
// mode the cell's nodes do not carry), X = L^-1 in place, then
// A_c^-1 = S X^T X S written in full (both triangles, the same value):
// symmetric positive semi-definite by construction, whatever the rounding.
__global__ void __launch_bounds__(BC_INV_T) k_bcoarse_inv(CoarseSetArgs a) {
	extern __shared__ float Sm[];  // n x n, row-major, lower triangle used
	__shared__ double sc[BC_MAX_N];
	__shared__ float tmp[BC_MAX_N];
	__shared__ int keep[BC_MAX_N];
	int const k = blockIdx.x;
	int const c0 = a.part_cell[k], n = 3 * (a.part_cell[k + 1] - c0);
	int const tid = threadIdx.x;
	if (n == 0) return;
	for (int i = tid; i < n; i += BC_INV_T) {
		double const d = ac_entry(a, c0, i, i);
		sc[i] = d > 0.0 ? 1.0 / sqrt(d) : 0.0;
	}
	__syncthreads();
	for (int e = tid; e < n * n; e += BC_INV_T) {
		int const i = e / n, j = e % n;
		if (j > i) continue;
		double const v = 0.5 * (ac_entry(a, c0, i, j) + ac_entry(a, c0, j, i));
		Sm[e] = (float) (v * sc[i] * sc[j]);
	}
	__syncthreads();
	// right-looking Cholesky, column by column
	for (int kk = 0; kk < n; kk++) {
		if (tid == 0) {
			float const d = Sm[kk * n + kk];
			keep[kk] = d > 1e-5f;
			Sm[kk * n + kk] = keep[kk] ? sqrtf(d) : 0.f;
		}
		__syncthreads();
		float const l = Sm[kk * n + kk];
		for (int i = kk + 1 + tid; i < n; i += BC_INV_T) Sm[i * n + kk] = l > 0.f ? Sm[i * n + kk] / l : 0.f;
		__syncthreads();
		int const m = n - kk - 1;
		for (int e = tid; e < m * m; e += BC_INV_T) {
			int const ii = e / m, jj = e % m;
			if (jj > ii) continue;
			int const i = kk + 1 + ii, j = kk + 1 + jj;
			Sm[i * n + j] -= Sm[i * n + kk] * Sm[j * n + kk];
		}
		__syncthreads();
	}
	// X = L^-1 in place, columns from the last: X_jj = 1 / L_jj and, below,
	// X[i][j] = -X_jj sum_{m=j+1..i} X[i][m] L[m][j] (one warp per row);
	// dropped DOFs get a zero row and column
	int const lane = tid & 31, warp = tid >> 5;
	for (int j = n - 1; j >= 0; j--) {
		for (int i = j + 1 + tid; i < n; i += BC_INV_T) tmp[i] = Sm[i * n + j];
		__syncthreads();
		float const xjj = keep[j] && Sm[j * n + j] > 0.f ? 1.f / Sm[j * n + j] : 0.f;
		for (int i = j + 1 + warp; i < n; i += BC_INV_T / 32) {
			float s = 0.f;
			if (keep[i])
				for (int m = j + 1 + lane; m <= i; m += 32) s += Sm[i * n + m] * tmp[m];
			for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
			if (lane == 0) Sm[i * n + j] = keep[i] ? -xjj * s : 0.f;
		}
		__syncthreads();
		if (tid == 0) Sm[j * n + j] = xjj;
		__syncthreads();
	}
	// A_c^-1 = S X^T X S: entry (i, j), i >= j, = s_i s_j sum_{m >= i} X[m][i] X[m][j]
	float* out = a.ainv + a.ainv_off[k];
	for (int e = tid; e < n * n; e += BC_INV_T) {
		int const i = e / n, j = e % n;
		if (j > i) continue;
		float s = 0.f;
		for (int m = i; m < n; m++) s += Sm[m * n + i] * Sm[m * n + j];
		float const v = (float) (sc[i] * sc[j] * (double) s);
		out[(long) i * n + j] = v;
		out[(long) j * n + i] = v;
	}
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
	// block-per-part kernel: used when every part has at most BB_MAX_NODES nodes
	int use_block, bnt;    // bnt: threads per block (autotuned with lpr)
	int* node_off_d;
	int* block_part;       // parts by decreasing node count
	int g_bnt, s_bnt;
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
	int two;               // the last solve's preconditioner is two-level
	// two-level coarse space (host-built cell grids, device set-up per step)
	int cb_built, n_cells, nmax, n_chunks;
	unsigned cb_gen;       // inputs generation the cells were built for
	int *part_cell, *cell_part, *cell_ptr, *cell_nodes, *node_cell, *cell_nbr;
	int *chunk_part, *chunk_cell, *part_chunk;
	int2* cell_xy;
	float2 *dxdy, *zc;
	float4* pnode;
	double *ac, *rc, *cdot;
	float* ainv;
	long long* ainv_off;
};

void batch_free(void* p) {
	BatchState* B = (BatchState*) p;
	if (!B) return;
	void* d[] = {B->tile_part, B->tile_begin, B->tile_end, B->part_tile, B->partials, B->ps, B->bar, B->err,
	             B->part_cell, B->cell_part, B->cell_ptr, B->cell_nodes, B->node_cell, B->cell_nbr, B->cell_xy,
	             B->dxdy, B->pnode, B->ac, B->rc, B->cdot, B->ainv, B->zc, B->ainv_off, B->chunk_part, B->chunk_cell,
	             B->part_chunk, B->node_off_d, B->block_part};
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

void* kernel_of_block(int lpr, int two) {
	switch (lpr) {
	case 1: return two ? (void*) k_batch_block<1, true> : (void*) k_batch_block<1, false>;
	case 2: return two ? (void*) k_batch_block<2, true> : (void*) k_batch_block<2, false>;
	default: return two ? (void*) k_batch_block<4, true> : (void*) k_batch_block<4, false>;
	}
}

void* kernel_of(int lpr, int two) {
	switch (lpr) {
	case 1: return two ? (void*) k_batch_pcg<1, true> : (void*) k_batch_pcg<1, false>;
	case 2: return two ? (void*) k_batch_pcg<2, true> : (void*) k_batch_pcg<2, false>;
	default: return two ? (void*) k_batch_pcg<4, true> : (void*) k_batch_pcg<4, false>;
	}
}

// Cell grid of one part over its bounding box (w x h): about one cell per
// `per_cell` nodes, at most BC_MAX_CELLS, as square as the box allows.
void part_grid(int n, double w, double h, int per_cell, int* gx, int* gy) {
	int target = n / per_cell;
	target = target < 1 ? 1 : target > BC_MAX_CELLS ? BC_MAX_CELLS : target;
	int x = 1, y = 1;
	if (w > 0 && h > 0) {
		x = (int) lround(sqrt((double) target * w / h));
		x = x < 1 ? 1 : x > target ? target : x;
		y = (int) lround((double) target / x);
		y = y > target / x ? target / x : y;
		y = y < 1 ? 1 : y;
	}
	else if (w > 0) x = target;
	else if (h > 0) y = target;
	*gx = x;
	*gy = y;
}

int coarse_nodes_per_cell() {
	char const* e = getenv("BFM_GPU_BATCH_COARSE_NODES");
	int const v = e ? atoi(e) : 0;
	return v >= 16 ? v : 48;
}

// The two-level coarse space of every part: its cell grid, the cell of each
// node and its offset from the cell's centre over H = max(cell width,
// height), the node lists per cell (a counting sort, ascending node index)
// and the neighbour table.  Host work from the coordinates, redone when an
// input changes; the device set-up (P's free flags, A_c, A_c^-1) runs per
// step.
int coarse_build(bfm_gpu_problem_t* P, BatchState* B, cudaStream_t st) {
	bfmi_mesh_t m;
	bfmi_mesh(P, &m);
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	int const N = bf.N, np = B->n_parts;
	int const per_cell = coarse_nodes_per_cell();
	double* xy = (double*) malloc(sizeof(double) * 2 * (N + 1));
	int* pgx = (int*) malloc(sizeof(int) * np);
	int* pgy = (int*) malloc(sizeof(int) * np);
	int* part_cell = (int*) malloc(sizeof(int) * (np + 1));
	long long* aoff = (long long*) malloc(sizeof(long long) * (np + 1));
	if (!xy || !pgx || !pgy || !part_cell || !aoff) {
		free(xy); free(pgx); free(pgy); free(part_cell); free(aoff);
		return bfail("out of host memory");
	}
	int rc = 0;
	if (cudaMemcpyAsync(xy, m.coords, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	    cudaStreamSynchronize(st) != cudaSuccess)
		rc = bfail("coordinate copy failed");
	// per part: box and grid
	double* box = (double*) malloc(sizeof(double) * 4 * np);
	if (!rc && !box) rc = bfail("out of host memory");
	int nc = 0, nmax = 0;
	long long na = 0;
	for (int k = 0; !rc && k < np; k++) {
		int const i0 = B->node_off_h[k], i1 = B->node_off_h[k + 1];
		double x0 = 0, y0 = 0, x1 = 0, y1 = 0;
		for (int i = i0; i < i1; i++) {
			double const x = xy[2 * i], y = xy[2 * i + 1];
			if (i == i0 || x < x0) x0 = x;
			if (i == i0 || x > x1) x1 = x;
			if (i == i0 || y < y0) y0 = y;
			if (i == i0 || y > y1) y1 = y;
		}
		box[4 * k] = x0;
		box[4 * k + 1] = y0;
		box[4 * k + 2] = x1 - x0;
		box[4 * k + 3] = y1 - y0;
		if (i1 > i0) part_grid(i1 - i0, x1 - x0, y1 - y0, per_cell, &pgx[k], &pgy[k]);
		else pgx[k] = pgy[k] = 0;
		part_cell[k] = nc;
		aoff[k] = na;
		int const n = 3 * pgx[k] * pgy[k];
		nc += pgx[k] * pgy[k];
		na += (long long) n * n;
		nmax = n > nmax ? n : nmax;
	}
	part_cell[np] = nc;
	aoff[np] = na;
	int* node_cell = (int*) malloc(sizeof(int) * (N + 1));
	float* dxdy = (float*) malloc(sizeof(float) * 2 * (N + 1));
	int* cell_ptr = (int*) calloc(nc + 1, sizeof(int));
	int* cell_nodes = (int*) malloc(sizeof(int) * (N + 1));
	int* cell_part = (int*) malloc(sizeof(int) * (nc + 1));
	int* cell_nbr = (int*) malloc(sizeof(int) * 9 * (nc + 1));
	int* cell_xy = (int*) malloc(sizeof(int) * 2 * (nc + 1));
	if (!rc && (!node_cell || !dxdy || !cell_ptr || !cell_nodes || !cell_part || !cell_nbr || !cell_xy))
		rc = bfail("out of host memory");
	for (int k = 0; !rc && k < np; k++) {
		int const gx = pgx[k], gy = pgy[k], c0 = part_cell[k];
		double const x0 = box[4 * k], y0 = box[4 * k + 1], w = box[4 * k + 2], h = box[4 * k + 3];
		double const cw = w > 0 ? w * (1.0 + 1e-12) / gx : 1.0, ch = h > 0 ? h * (1.0 + 1e-12) / gy : 1.0;
		double const H = cw > ch ? cw : ch;
		for (int i = B->node_off_h[k]; i < B->node_off_h[k + 1]; i++) {
			int cx = (int) ((xy[2 * i] - x0) / cw), cy = (int) ((xy[2 * i + 1] - y0) / ch);
			cx = cx < 0 ? 0 : cx >= gx ? gx - 1 : cx;
			cy = cy < 0 ? 0 : cy >= gy ? gy - 1 : cy;
			node_cell[i] = c0 + cx + gx * cy;
			dxdy[2 * i] = (float) ((xy[2 * i] - (x0 + (cx + 0.5) * cw)) / H);
			dxdy[2 * i + 1] = (float) ((xy[2 * i + 1] - (y0 + (cy + 0.5) * ch)) / H);
			cell_ptr[node_cell[i] + 1]++;
		}
		for (int cy = 0; cy < gy; cy++)
			for (int cx = 0; cx < gx; cx++) {
				int const c = c0 + cx + gx * cy;
				cell_part[c] = k;
				cell_xy[2 * c] = cx;
				cell_xy[2 * c + 1] = cy;
				for (int dy = -1; dy <= 1; dy++)
					for (int dx = -1; dx <= 1; dx++) {
						int const ux = cx + dx, uy = cy + dy;
						cell_nbr[9 * c + 3 * (dy + 1) + dx + 1] = ux >= 0 && ux < gx && uy >= 0 && uy < gy ? c0 + ux + gx * uy : -1;
					}
			}
	}
	// stage Y's work items: BC_CHUNK consecutive cells of one part
	int nq = 0;
	for (int k = 0; !rc && k < np; k++) nq += (part_cell[k + 1] - part_cell[k] + BC_CHUNK - 1) / BC_CHUNK;
	int* chunk_part = (int*) malloc(sizeof(int) * (nq + 1));
	int* chunk_cell = (int*) malloc(sizeof(int) * (nq + 1));
	int* part_chunk = (int*) malloc(sizeof(int) * (np + 1));
	if (!rc && (!chunk_part || !chunk_cell || !part_chunk)) rc = bfail("out of host memory");
	if (!rc) {
		int q = 0;
		for (int k = 0; k < np; k++) {
			part_chunk[k] = q;
			for (int c = part_cell[k]; c < part_cell[k + 1]; c += BC_CHUNK) {
				chunk_part[q] = k;
				chunk_cell[q] = c;
				q++;
			}
		}
		part_chunk[np] = q;
	}
	if (!rc) {
		for (int c = 0; c < nc; c++) cell_ptr[c + 1] += cell_ptr[c];
		int* fill = (int*) malloc(sizeof(int) * (nc + 1));
		if (!fill) rc = bfail("out of host memory");
		else {
			memcpy(fill, cell_ptr, sizeof(int) * (nc + 1));
			for (int i = 0; i < N; i++) cell_nodes[fill[node_cell[i]]++] = i;
			free(fill);
		}
	}
	if (!rc) {
		// device buffers, (re)sized for this batch
		void* old[] = {B->part_cell, B->cell_part, B->cell_ptr, B->cell_nodes, B->node_cell, B->cell_nbr, B->cell_xy,
		               B->dxdy, B->pnode, B->ac, B->rc, B->cdot, B->ainv, B->zc, B->ainv_off, B->chunk_part,
		               B->chunk_cell, B->part_chunk};
		for (void* q : old)
			if (q) cudaFree(q);
		B->part_cell = B->cell_part = B->cell_ptr = B->cell_nodes = B->node_cell = B->cell_nbr = nullptr;
		B->chunk_part = B->chunk_cell = B->part_chunk = nullptr;
		B->cell_xy = nullptr;
		B->dxdy = B->zc = nullptr;
		B->pnode = nullptr;
		B->ac = B->rc = B->cdot = nullptr;
		B->ainv = nullptr;
		B->ainv_off = nullptr;
		int const c1 = nc + 1;
		if (cudaMalloc(&B->part_cell, sizeof(int) * (np + 1)) != cudaSuccess ||
		    cudaMalloc(&B->cell_part, sizeof(int) * c1) != cudaSuccess ||
		    cudaMalloc(&B->cell_ptr, sizeof(int) * c1) != cudaSuccess ||
		    cudaMalloc(&B->cell_nodes, sizeof(int) * (N + 1)) != cudaSuccess ||
		    cudaMalloc(&B->node_cell, sizeof(int) * (N + 1)) != cudaSuccess ||
		    cudaMalloc(&B->cell_nbr, sizeof(int) * 9 * c1) != cudaSuccess ||
		    cudaMalloc(&B->cell_xy, sizeof(int2) * c1) != cudaSuccess ||
		    cudaMalloc(&B->dxdy, sizeof(float2) * (N + 1)) != cudaSuccess ||
		    cudaMalloc(&B->pnode, sizeof(float4) * (N + 1)) != cudaSuccess ||
		    cudaMalloc(&B->ac, sizeof(double) * 81 * c1) != cudaSuccess ||
		    cudaMalloc(&B->rc, sizeof(double) * 3 * c1) != cudaSuccess ||
		    cudaMalloc(&B->cdot, sizeof(double) * (nq + 1)) != cudaSuccess ||
		    cudaMalloc(&B->ainv, sizeof(float) * (na + 1)) != cudaSuccess ||
		    cudaMalloc(&B->zc, sizeof(float2) * (N + 1)) != cudaSuccess ||
		    cudaMalloc(&B->ainv_off, sizeof(long long) * (np + 1)) != cudaSuccess ||
		    cudaMalloc(&B->chunk_part, sizeof(int) * (nq + 1)) != cudaSuccess ||
		    cudaMalloc(&B->chunk_cell, sizeof(int) * (nq + 1)) != cudaSuccess ||
		    cudaMalloc(&B->part_chunk, sizeof(int) * (np + 1)) != cudaSuccess)
			rc = bfail("cudaMalloc failed for the two-level coarse space");
	}
	if (!rc && (cudaMemcpy(B->part_cell, part_cell, sizeof(int) * (np + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->cell_part, cell_part, sizeof(int) * nc, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->cell_ptr, cell_ptr, sizeof(int) * (nc + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->cell_nodes, cell_nodes, sizeof(int) * N, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->node_cell, node_cell, sizeof(int) * N, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->cell_nbr, cell_nbr, sizeof(int) * 9 * nc, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->cell_xy, cell_xy, sizeof(int) * 2 * nc, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->dxdy, dxdy, sizeof(float) * 2 * N, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->ainv_off, aoff, sizeof(long long) * (np + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->chunk_part, chunk_part, sizeof(int) * nq, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->chunk_cell, chunk_cell, sizeof(int) * nq, cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemcpy(B->part_chunk, part_chunk, sizeof(int) * (np + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
	            cudaMemset(B->zc, 0, sizeof(float2) * (N + 1)) != cudaSuccess))
		rc = bfail("cudaMemcpy failed for the two-level coarse space");
	if (!rc && cudaFuncSetAttribute(k_bcoarse_inv, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                (int) (nmax * nmax * sizeof(float))) != cudaSuccess)
		rc = bfail("the coarse inverse kernel cannot have %d bytes of shared memory", (int) (nmax * nmax * sizeof(float)));
	if (!rc) {
		B->n_cells = nc;
		B->n_chunks = nq;
		B->nmax = nmax;
		B->cb_built = 1;
		B->cb_gen = bf.inputs_gen;
	}
	free(xy); free(pgx); free(pgy); free(part_cell); free(aoff); free(box);
	free(node_cell); free(dxdy); free(cell_ptr); free(cell_nodes); free(cell_part); free(cell_nbr); free(cell_xy);
	free(chunk_part); free(chunk_cell); free(part_chunk);
	return rc;
}

CoarseSetArgs coarse_set_args(bfm_gpu_problem_t* P, BatchState* B) {
	bfmi_mesh_t m;
	bfmi_mesh(P, &m);
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	CoarseSetArgs c;
	memset(&c, 0, sizeof c);
	c.N = bf.N;
	c.n_cells = B->n_cells;
	c.part_cell = B->part_cell;
	c.cell_ptr = B->cell_ptr;
	c.cell_nodes = B->cell_nodes;
	c.node_cell = B->node_cell;
	c.cell_nbr = B->cell_nbr;
	c.cell_xy = B->cell_xy;
	c.dxdy = B->dxdy;
	c.last_ci = m.last_ci;
	c.pnode = B->pnode;
	c.row_ptr = bf.row_ptr;
	c.cols = bf.cols;
	c.vals = bf.vals32;
	c.corr = bf.corr32;
	c.ac = B->ac;
	c.ainv = B->ainv;
	c.ainv_off = B->ainv_off;
	return c;
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
	a.block_pc = bf.precond != BFM_GPU_PC_JACOBI;
	a.node_off = B->node_off_d;
	a.block_part = B->block_part;
	a.z = (float*) bf.vec[3];
	if (B->two) {
		a.n_cells = B->n_cells;
		a.part_cell = B->part_cell;
		a.cell_part = B->cell_part;
		a.cell_ptr = B->cell_ptr;
		a.cell_nodes = B->cell_nodes;
		a.node_cell = B->node_cell;
		a.pnode = B->pnode;
		a.ainv = B->ainv;
		a.ainv_off = B->ainv_off;
		a.rc = B->rc;
		a.zc = B->zc;
		a.cdot = B->cdot;
		a.n_chunks = B->n_chunks;
		a.chunk_part = B->chunk_part;
		a.chunk_cell = B->chunk_cell;
		a.part_chunk = B->part_chunk;
	}
	if (o) {
		a.rtol = o->rtol;
		a.drop2 = o->replace_drop * o->replace_drop;
		a.max_iters = o->max_iters;
		if (o->barrier_polls > 0) a.polls = (long) o->barrier_polls;
	}
	return a;
}

// blocks of the persistent kernel that fit on the GPU at once (cooperative launch)
int coop_grid(int lpr, int two, int* grid) {
	int dev = 0, sms = 0, nb = 0;
	BCK(cudaGetDevice(&dev));
	BCK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	BCK(cudaFuncSetAttribute(kernel_of(lpr, two), cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(Shared)));
	BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel_of(lpr, two), BT, sizeof(Shared)));
	if (nb < 1) return bfail("the batch kernel does not fit on an SM");
	*grid = sms * nb;
	return 0;
}

int launch(bfm_gpu_problem_t* P, BatchState* B, BatchArgs* a, int lpr, int grid, cudaStream_t st) {
	BCK(cudaMemsetAsync(B->bar, 0, 64 * sizeof(unsigned), st));
	BCK(cudaMemsetAsync(B->err, 0, sizeof(int), st));
	if (B->two) {
		// the coarse space of this assembly: P's free flags, A_c, A_c^-1
		// (k_bcoarse_inv's shared-memory size is set by coarse_build, outside any capture)
		CoarseSetArgs c = coarse_set_args(P, B);
		int const smem = B->nmax * B->nmax * (int) sizeof(float);
		if (c.N > 0) k_bpnode<<<(c.N + 255) / 256, 256, 0, st>>>(c);
		if (c.n_cells > 0) {
			k_bcoarse_ac<<<(int) ((9l * 32 * c.n_cells + 127) / 128), 128, 0, st>>>(c);
			k_bcoarse_inv<<<B->n_parts, BC_INV_T, smem, st>>>(c);
		}
		BCK(cudaGetLastError());
	}
	if (B->use_block) {
		// one block per part, largest parts first; block barriers only
		void* params[1] = {a};
		BCK(cudaLaunchKernel(kernel_of_block(lpr, B->two), dim3(B->n_parts), dim3(B->bnt), params, 0, st));
	}
	else {
		void* params[1] = {a};
		BCK(cudaLaunchCooperativeKernel(kernel_of(lpr, B->two), dim3(grid), dim3(BT), params, sizeof(Shared), st));
	}
	k_batch_residual<<<grid, BT, 0, st>>>(*a);
	k_batch_part_residual<<<(B->n_parts + 127) / 128, 128, 0, st>>>(*a);
	BCK(cudaGetLastError());
	return 0;
}

// Project autotuner for the batch: rows per tile x lanes per row, each
// candidate timed over 10 iterations of the persistent kernel on the
// assembled batch (timing mode: no stopping test), fastest kept.
// one timed launch of 10 iterations of the current shape (timing mode: no stopping test)
int time_shape(bfm_gpu_problem_t* P, BatchState* B, const bfm_gpu_opts_t* o, cudaStream_t st, int lpr, int grid, float* ms) {
	BatchArgs a = batch_args(P, B, o);
	a.timing_iters = 10;
	BCK(cudaEventRecord(B->ev[0], st));
	if (launch(P, B, &a, lpr, grid, st)) return -1;
	BCK(cudaEventRecord(B->ev[1], st));
	BCK(cudaStreamSynchronize(st));
	BCK(cudaEventElapsedTime(ms, B->ev[0], B->ev[1]));
	int err = 0;
	BCK(cudaMemcpy(&err, B->err, sizeof err, cudaMemcpyDeviceToHost));
	if (err) return bfail("batch kernel barrier timed out during autotuning");
	return 0;
}

int autotune(bfm_gpu_problem_t* P, BatchState* B, const bfm_gpu_opts_t* o, cudaStream_t st) {
	if (B->use_block) {
		// threads per block x lanes per row of the block-per-part kernel
		int const nts[] = {256, 512, 1024};
		int const lprs[] = {1, 2, 4};
		int grid = 0;
		if (coop_grid(2, B->two, &grid)) return -1;
		float best = 1e30f;
		int best_nt = 512, best_lpr = 2;
		for (int nt : nts)
			for (int lpr : lprs) {
				B->bnt = nt;
				float ms = 0;
				if (time_shape(P, B, o, st, lpr, grid, &ms)) return -1;
				if (ms < best) {
					best = ms;
					best_nt = nt;
					best_lpr = lpr;
				}
			}
		B->bnt = best_nt;
		B->lpr = best_lpr;
		B->tuned = 1;
		return 0;
	}
	int const rpts[] = {128, 256, 512, 1024};
	int const lprs[] = {1, 2, 4};
	float best = 1e30f;
	int best_rpt = 256, best_lpr = 2;
	for (int rpt : rpts) {
		if (build_tiles(B, rpt)) return -1;
		for (int lpr : lprs) {
			int grid = 0;
			if (coop_grid(lpr, B->two, &grid)) return -1;
			BatchArgs a = batch_args(P, B, o);
			a.timing_iters = 10;
			BCK(cudaEventRecord(B->ev[0], st));
			if (launch(P, B, &a, lpr, grid, st)) return -1;
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
	// the block-per-part kernel unless a part is too large for one block
	// (BFM_GPU_BATCH_KERNEL=tiled asks for the tiled persistent kernel)
	int maxn = 0;
	for (int k = 0; k < n_parts; k++)
		maxn = node_offsets[k + 1] - node_offsets[k] > maxn ? node_offsets[k + 1] - node_offsets[k] : maxn;
	char const* kern = getenv("BFM_GPU_BATCH_KERNEL");
	B->use_block = maxn <= BB_MAX_NODES && !(kern && strcmp(kern, "tiled") == 0);
	B->bnt = 512;
	int* order = (int*) malloc(sizeof(int) * n_parts);
	if (!order) return bfail("out of host memory");
	for (int k = 0; k < n_parts; k++) order[k] = k;
	// largest first, ties in part order (insertion sort: n_parts <= 512)
	for (int k = 1; k < n_parts; k++) {
		int const v = order[k], nv = node_offsets[v + 1] - node_offsets[v];
		int j = k - 1;
		while (j >= 0 && node_offsets[order[j] + 1] - node_offsets[order[j]] < nv) {
			order[j + 1] = order[j];
			j--;
		}
		order[j + 1] = v;
	}
	cudaError_t e = cudaMalloc(&B->block_part, sizeof(int) * n_parts);
	if (e == cudaSuccess) e = cudaMalloc(&B->node_off_d, sizeof(int) * (n_parts + 1));
	if (e == cudaSuccess) e = cudaMemcpy(B->block_part, order, sizeof(int) * n_parts, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(B->node_off_d, node_offsets, sizeof(int) * (n_parts + 1), cudaMemcpyHostToDevice);
	free(order);
	if (e != cudaSuccess) return bfail("CUDA error %s", cudaGetErrorString(e));
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
	bfm_gpu_opts_t o;
	if (opts) o = *opts;
	else bfm_gpu_default_opts(&o);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	if (o.precond != BFM_GPU_PC_JACOBI && o.precond != BFM_GPU_PC_BLOCK_JACOBI && o.precond != BFM_GPU_PC_TWO_LEVEL_JACOBI)
		return bfail("the batched solver takes the Jacobi, block Jacobi or two-level block Jacobi preconditioner, got %d",
		             o.precond);
	// the smoother's layout is formed by the assembly: assemble again if it differs
	int const want_pc = o.precond == BFM_GPU_PC_JACOBI ? BFM_GPU_PC_JACOBI : BFM_GPU_PC_BLOCK_JACOBI;
	if (bf.precond != want_pc) {
		if (bfmi_set_precond(P, want_pc) || bfm_gpu_problem_assemble(P, bf.precision)) return -1;
		bfmi_buffers(P, &bf);
	}
	int const two = o.precond == BFM_GPU_PC_TWO_LEVEL_JACOBI;
	if (two && (!B->cb_built || B->cb_gen != bf.inputs_gen) && coarse_build(P, B, st)) return -1;
	if (two != B->two) {
		B->two = two;
		B->tuned = 0;  // the tile shapes are tuned per kernel
		if (B->graph) cudaGraphExecDestroy(B->graph);
		B->graph = nullptr;
		B->direct = 0;
	}
	if (o.autotune && !B->tuned) {
		if (autotune(P, B, &o, st)) return -1;
		if (B->graph) cudaGraphExecDestroy(B->graph);
		B->graph = nullptr;
	}
	bool const same = (B->graph || B->direct) && B->g_rtol == o.rtol && B->g_drop == o.replace_drop && B->g_iters == o.max_iters &&
	                  B->g_rpt == B->rows_per_tile && B->g_lpr == B->lpr && B->g_polls == o.barrier_polls &&
	                  B->g_bnt == B->bnt;
	if (!same) {
		// one graph: reset of the barrier words, the persistent cooperative
		// kernel, the per-part FP64 residuals
		int grid = 0;
		if (coop_grid(B->lpr, B->two, &grid)) return -1;
		B->grid = grid;
		BatchArgs a = batch_args(P, B, &o);
		cudaStream_t cs;
		BCK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
		cudaGraph_t g = nullptr;
		int rc = 0;
		if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = bfail("stream capture failed");
		if (!rc) rc = launch(P, B, &a, B->lpr, grid, cs);
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
		B->g_bnt = B->bnt;
	}
	BCK(cudaEventRecord(B->ev[0], st));
	if (B->graph) {
		BCK(cudaGraphLaunch(B->graph, st));
	}
	else {
		BatchArgs a = batch_args(P, B, &o);
		if (launch(P, B, &a, B->lpr, B->grid, st)) return -1;
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
	if (o.precond != BFM_GPU_PC_JACOBI && o.precond != BFM_GPU_PC_BLOCK_JACOBI && o.precond != BFM_GPU_PC_TWO_LEVEL_JACOBI)
		return bfail("the batched solver takes the Jacobi, block Jacobi or two-level block Jacobi preconditioner, got %d",
		             o.precond);
	// the smoother's layout of the assemblies below
	if (bfmi_set_precond(P, o.precond == BFM_GPU_PC_JACOBI ? BFM_GPU_PC_JACOBI : BFM_GPU_PC_BLOCK_JACOBI)) return -1;
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	bool const same = (B->step_graph || B->step_direct) && B->s_precision == precision && B->s_gen == bf.inputs_gen &&
	                  B->s_rpt == B->rows_per_tile && B->s_lpr == B->lpr && B->s_bnt == B->bnt && B->s_opts.rtol == o.rtol &&
	                  B->s_opts.max_iters == o.max_iters && B->s_opts.replace_drop == o.replace_drop &&
	                  B->s_opts.barrier_polls == o.barrier_polls && B->s_opts.autotune == o.autotune &&
	                  B->s_opts.precond == o.precond;
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
		if (coop_grid(B->lpr, B->two, &grid)) return -1;
		B->grid = grid;
		BatchArgs a = batch_args(P, B, &o);
		cudaGraph_t g = nullptr;
		int rc = 0;
		if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = bfail("stream capture failed");
		if (!rc) rc = bfm_gpu_problem_assemble(P, precision);
		if (!rc) {
			BatchArgs a2 = batch_args(P, B, &o);  // the assembly's buffers, unchanged
			a = a2;
			rc = launch(P, B, &a, B->lpr, grid, st);
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
		B->s_bnt = B->bnt;
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

int bfm_gpu_problem_parts_coarse(bfm_gpu_problem_t* P, int* n_coarse, int64_t* ainv_offsets, float* ainv) {
	g_berr[0] = 0;
	BatchState* B = state_of(P);
	if (!B) return bfail("no parts set");
	if (!B->two || !B->cb_built) return bfail("no two-level solve of this batch yet");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	BCK(cudaStreamSynchronize((cudaStream_t) bf.stream));
	int const np = B->n_parts;
	int* pc = (int*) malloc(sizeof(int) * (np + 1));
	long long* off = (long long*) malloc(sizeof(long long) * (np + 1));
	if (!pc || !off) {
		free(pc);
		free(off);
		return bfail("out of host memory");
	}
	int rc = 0;
	if (cudaMemcpy(pc, B->part_cell, sizeof(int) * (np + 1), cudaMemcpyDeviceToHost) != cudaSuccess ||
	    cudaMemcpy(off, B->ainv_off, sizeof(long long) * (np + 1), cudaMemcpyDeviceToHost) != cudaSuccess)
		rc = bfail("cudaMemcpy failed");
	if (!rc) {
		for (int k = 0; k < np; k++) {
			if (n_coarse) n_coarse[k] = 3 * (pc[k + 1] - pc[k]);
			if (ainv_offsets) ainv_offsets[k] = off[k];
		}
		if (ainv_offsets) ainv_offsets[np] = off[np];
		if (ainv && off[np] > 0 &&
		    cudaMemcpy(ainv, B->ainv, sizeof(float) * (size_t) off[np], cudaMemcpyDeviceToHost) != cudaSuccess)
			rc = bfail("cudaMemcpy failed");
	}
	free(pc);
	free(off);
	return rc;
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
	if (rows_per_tile) *rows_per_tile = B->use_block ? B->bnt : B->rows_per_tile;
	if (lanes_per_row) *lanes_per_row = B->lpr;
	if (ms_solve) {
		float ms = 0;
		cudaEventElapsedTime(&ms, B->ev[0], B->ev[1]);
		*ms_solve = ms;
	}
	return 0;
}

}  // extern "C"
