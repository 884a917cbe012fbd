// GB300 (sm_103a) FEM hot path of libbfm: sparsity pattern, element loop,
// Dirichlet elimination, Neumann loads and preconditioned CG.
//
// Reference path replaced (libbfm, CPU, dense): system.c:427-529 create_planar
// (element loop system.c:109-227, constraints 358-386, Neumann 477-498),
// system.c:44-81 renumber + matrix.c:253-404 band LU, driven by
// sim.c:103-135 run_elasticity.
//
// Layout in HBM (one problem):
//   coords   f64[2N]        interleaved x,y
//   elems    i32[kind*E]
//   inc_ptr  i32[N+1], inc i32[kind*E]   node -> incident elements, ascending
//   row_ptr  i32[N+1], cols i32[nb]      node-block CSR (2x2 blocks), ascending
//   vals     f64[4*nb] or f32[4*nb]      block entries uu uv vu vv
//   b, x, r, p, s, w, dinv               f64 (or f32 for the mixed inner loop)
//
// Exactness: in FP64 mode each stiffness entry is accumulated in the
// reference's order (element ascending, then Gauss point) from terms computed
// with the reference's operation order and no fused multiply-add (the __d*_rn
// intrinsics are never contracted), so K is bit-identical to libbfm's dense
// K and the integer work derived from its exact zeros (RCM) matches exactly.
#include <cuda_runtime.h>

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <bfm/condition.h>
#include <bfm/gpu.h>

#include <stdarg.h>
#include <type_traits>

namespace {

constexpr int MAXV = 32;  // incident elements (or edges) per node
constexpr int MAXR = 32;  // node blocks per row
constexpr int MAXQ = 16;  // integration points
constexpr int MAXF = 8;   // body forces
constexpr int MAXC = 16;  // conditions handled by the fused kernels
constexpr int TPB = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = TPB * SCAN_ITEMS;

enum : int { ERR_VALENCE = 1, ERR_ROW = 2, ERR_EDGE_VALENCE = 4 };

struct Rule {
	int nq;
	double w[MAXQ];
	double phi[MAXQ][4];
	double dxi[MAXQ][4];
	double deta[MAXQ][4];
};

struct Forces {
	int nf;
	double f[MAXF][2];
	const double* field[MAXF];  // per-node field (device) or nullptr
};

// ------------------------------------------------------------------ exact FP64 arithmetic

__device__ __forceinline__ double xm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xd(double a, double b) { return __ddiv_rn(a, b); }

// material constants, reference system.c:454-458 (same operation order)
__device__ __forceinline__ void material_abc(double E, double nu, int stress, double& a, double& b, double& c) {
	if (!stress) {
		double const den = xs(1.0, xm(2.0, nu));
		a = xd(xd(xm(E, xs(1.0, nu)), xa(1.0, nu)), den);
		b = xd(xd(xm(E, nu), xa(1.0, nu)), den);
	}
	else {
		double const den = xs(1.0, xm(nu, nu));
		a = xd(E, den);
		b = xd(xm(E, nu), den);
	}
	c = xd(E, xm(2.0, xa(1.0, nu)));
}

// ------------------------------------------------------------------ scans

// inclusive scan of one value across the block; returns the block total in *total
__device__ __forceinline__ int block_incl_scan(int v, int* total) {
	__shared__ int warp_tot[TPB / 32];
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	for (int o = 1; o < 32; o <<= 1) {
		int const t = __shfl_up_sync(0xffffffffu, v, o);
		if (lane >= o) v += t;
	}
	if (lane == 31) warp_tot[wid] = v;
	__syncthreads();
	if (wid == 0) {
		int t = lane < TPB / 32 ? warp_tot[lane] : 0;
		for (int o = 1; o < 32; o <<= 1) {
			int const u = __shfl_up_sync(0xffffffffu, t, o);
			if (lane >= o) t += u;
		}
		if (lane < TPB / 32) warp_tot[lane] = t;
	}
	__syncthreads();
	if (wid > 0) v += warp_tot[wid - 1];
	*total = warp_tot[TPB / 32 - 1];
	__syncthreads();
	return v;
}

// per-tile exclusive scan; tile totals to sums[tile]
__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, int n, int* __restrict__ sums) {
	int const base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
	int v[SCAN_ITEMS];
	int loc = 0;
#pragma unroll
	for (int i = 0; i < SCAN_ITEMS; i++) {
		v[i] = base + i < n ? in[base + i] : 0;
		loc += v[i];
	}
	int total;
	int const incl = block_incl_scan(loc, &total);
	int run = incl - loc;
#pragma unroll
	for (int i = 0; i < SCAN_ITEMS; i++) {
		if (base + i < n) out[base + i] = run;
		run += v[i];
	}
	if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// exclusive scan of the tile totals in one block (serial over chunks of the block width)
__global__ void k_scan_spine(int* sums, int ntiles, int* grand_total) {
	int carry = 0;
	for (int base = 0; base < ntiles; base += TPB) {
		int const i = base + threadIdx.x;
		int const v = i < ntiles ? sums[i] : 0;
		int total;
		int const incl = block_incl_scan(v, &total);
		if (i < ntiles) sums[i] = carry + incl - v;
		carry += total;
	}
	if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ sums, const int* __restrict__ grand_total) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] += sums[i / SCAN_TILE];
	if (i == 0) out[n] = *grand_total;
}

// ------------------------------------------------------------------ incidence (node -> items)

__global__ void k_count(const int* __restrict__ items, long total, int* __restrict__ cnt) {
	for (long i = blockIdx.x * (long) blockDim.x + threadIdx.x; i < total; i += (long) gridDim.x * blockDim.x)
		atomicAdd(&cnt[items[i]], 1);
}

__global__ void k_fill(const int* __restrict__ items, long total, int arity, const int* __restrict__ ptr,
                       int* __restrict__ cursor, int* __restrict__ list) {
	for (long i = blockIdx.x * (long) blockDim.x + threadIdx.x; i < total; i += (long) gridDim.x * blockDim.x) {
		int const node = items[i];
		int const pos = ptr[node] + atomicAdd(&cursor[node], 1);
		list[pos] = (int) (i / arity);
	}
}

// ascending order of each node's list (insertion sort; lists are short)
__global__ void k_sort_lists(int n, const int* __restrict__ ptr, int* __restrict__ list, int maxlen, int* err, int code) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= n) return;
	int const s = ptr[r], len = ptr[r + 1] - s;
	if (len > maxlen) {
		atomicOr(err, code);
		return;
	}
	int* v = list + s;
	for (int i = 1; i < len; i++) {
		int const t = v[i];
		int j = i - 1;
		while (j >= 0 && v[j] > t) {
			v[j + 1] = v[j];
			j--;
		}
		v[j + 1] = t;
	}
}

// ------------------------------------------------------------------ node-block pattern

// Per node: the sorted distinct nodes of its incident elements (itself
// included), written at cand + kind*inc_ptr[r]; row_len[r] their count.
__global__ void k_rows_count(int N, int kind, const int* __restrict__ elems, const int* __restrict__ inc_ptr,
                             const int* __restrict__ inc, int* __restrict__ cand, int* __restrict__ row_len, int* err) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= N) return;
	int const s = inc_ptr[r], deg = inc_ptr[r + 1] - s;
	if (deg > MAXV) {
		// flagged; keep the row well formed (diagonal only) so later kernels stay in bounds
		atomicOr(err, ERR_VALENCE);
		cand[(long) kind * s] = r;
		row_len[r] = 1;
		return;
	}
	int c[MAXV * 4];
	int m = 0;
	for (int t = 0; t < deg; t++) {
		int const e = inc[s + t];
		for (int j = 0; j < kind; j++) c[m++] = elems[(long) e * kind + j];
	}
	for (int i = 1; i < m; i++) {
		int const t = c[i];
		int j = i - 1;
		while (j >= 0 && c[j] > t) {
			c[j + 1] = c[j];
			j--;
		}
		c[j + 1] = t;
	}
	int u = 0;
	for (int i = 0; i < m; i++)
		if (u == 0 || c[u - 1] != c[i]) c[u++] = c[i];
	if (u == 0) c[u++] = r;  // isolated node: diagonal block only
	if (u > MAXR) {
		atomicOr(err, ERR_ROW);
		u = MAXR;
	}
	int* out = cand + (long) kind * s;
	// an isolated node has no candidate slots of its own: it borrows row_len's
	// guarantee of one block and is written by k_rows_fill directly
	if (deg > 0)
		for (int i = 0; i < u; i++) out[i] = c[i];
	row_len[r] = u;
}

__global__ void k_rows_fill(int N, int kind, const int* __restrict__ inc_ptr, const int* __restrict__ cand,
                            const int* __restrict__ row_ptr, int* __restrict__ cols) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= N) return;
	int const s = inc_ptr[r], rs = row_ptr[r], len = row_ptr[r + 1] - rs;
	if (inc_ptr[r + 1] == s) {
		cols[rs] = r;
		return;
	}
	const int* in = cand + (long) kind * s;
	for (int i = 0; i < len; i++) cols[rs + i] = in[i];
}

// ------------------------------------------------------------------ Dirichlet bookkeeping

// Conditions are applied in order; per DOF we keep the first value (used to
// eliminate its column, system.c:358-366), the last value (the final b entry,
// system.c:373) and the index of the last condition touching it.
__global__ void k_dirichlet_mark(int N, int ci, int shift, double value, const uint8_t* __restrict__ mask,
                                 int* __restrict__ last_ci, double* __restrict__ first, double* __restrict__ last) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N || !mask[i]) return;
	int const d = 2 * i + shift;
	if (last_ci[d] < 0) first[d] = value;
	last[d] = value;
	last_ci[d] = ci;
}

// ------------------------------------------------------------------ assembly

struct AsmArgs {
	int N, kind, stress;
	const double* coords;
	const int* elems;
	const double* elemE;
	const double* elemNu;
	double E, nu, rho;
	Rule rule;
	Forces forces;
	const int* inc_ptr;
	const int* inc;
	const int* row_ptr;
	const int* cols;
	const int* last_ci;
	const double* first;
	const double* last;
	double* vals64;
	float* vals32;
	double* b;
	double* dinv64;  // jacobi: 2 per node; block-jacobi: 4 per node
	float* dinv32;
	int precond;
	int* err;
};

__device__ __forceinline__ void store_precond(const AsmArgs& a, int r, double k00, double k01, double k10, double k11) {
	if (a.precond == BFM_GPU_PC_BLOCK_JACOBI) {
		double const det = k00 * k11 - k01 * k10;
		double const id = det != 0.0 ? 1.0 / det : 0.0;
		double const m0 = k11 * id, m1 = -k01 * id, m2 = -k10 * id, m3 = k00 * id;
		if (a.dinv64) {
			a.dinv64[4 * r + 0] = m0; a.dinv64[4 * r + 1] = m1;
			a.dinv64[4 * r + 2] = m2; a.dinv64[4 * r + 3] = m3;
		}
		if (a.dinv32) {
			a.dinv32[4 * r + 0] = (float) m0; a.dinv32[4 * r + 1] = (float) m1;
			a.dinv32[4 * r + 2] = (float) m2; a.dinv32[4 * r + 3] = (float) m3;
		}
	}
	else {
		double const d0 = k00 != 0.0 ? 1.0 / k00 : 0.0;
		double const d1 = k11 != 0.0 ? 1.0 / k11 : 0.0;
		if (a.dinv64) { a.dinv64[2 * r] = d0; a.dinv64[2 * r + 1] = d1; }
		if (a.dinv32) { a.dinv32[2 * r] = (float) d0; a.dinv32[2 * r + 1] = (float) d1; }
	}
}

// One thread per node row (owner computes, no atomics): walk the node's
// incident elements in ascending order, evaluate each element at every
// integration point exactly as system.c:136-224 does and accumulate the terms
// that land in this row.  Epilogue: symmetric Dirichlet elimination of the
// row (system.c:358-374) and the preconditioner's diagonal.
//
// EXACT = true: FP64 with the reference's operation order (bit-identical K).
// EXACT = false: FP32 element integration from FP64 node offsets.
template <bool EXACT>
__global__ void __launch_bounds__(128) k_assemble(AsmArgs a) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= a.N) return;
	using T = typename std::conditional<EXACT, double, float>::type;
	int const kind = a.kind;
	int const rs = a.row_ptr[r], len = a.row_ptr[r + 1] - rs;
	if (len > MAXR) return;  // already flagged by the pattern kernels

	int col[MAXR];
	T acc[MAXR][4];
	for (int s = 0; s < len; s++) {
		col[s] = a.cols[rs + s];
		acc[s][0] = acc[s][1] = acc[s][2] = acc[s][3] = T(0);
	}
	double b0 = 0.0, b1 = 0.0;

	double ca = 0, cb = 0, cc = 0;
	if (!a.elemE && !a.elemNu) material_abc(a.E, a.nu, a.stress, ca, cb, cc);

	int const is = a.inc_ptr[r], ie = a.inc_ptr[r + 1];
	int prev_e = -1;
	for (int t = is; t < ie; t++) {
		int const e = a.inc[t];
		if (e == prev_e) continue;  // a node repeated inside one element: degenerate, det = 0
		prev_e = e;
		int map[4];
		double x[4], y[4];
		int jr = 0;
		for (int j = 0; j < kind; j++) {
			map[j] = a.elems[(long) e * kind + j];
			x[j] = a.coords[2l * map[j]];
			y[j] = a.coords[2l * map[j] + 1];
		}
		for (int j = kind - 1; j >= 0; j--)
			if (map[j] == r) jr = j;
		int slot[4];
		for (int k = 0; k < kind; k++) {
			int s = 0;
			while (s < len - 1 && col[s] != map[k]) s++;
			slot[k] = s;
		}
		double ea = ca, eb = cb, ec = cc;
		if (a.elemE || a.elemNu) {
			double const E = a.elemE ? a.elemE[e] : a.E;
			double const nu = a.elemNu ? a.elemNu[e] : a.nu;
			material_abc(E, nu, a.stress, ea, eb, ec);
		}
		if constexpr (EXACT) {
			for (int q = 0; q < a.rule.nq; q++) {
				double const w = a.rule.w[q];
				double dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0;
				for (int j = 0; j < kind; j++) {
					dx_dxsi = xa(dx_dxsi, xm(x[j], a.rule.dxi[q][j]));
					dx_deta = xa(dx_deta, xm(x[j], a.rule.deta[q][j]));
					dy_dxsi = xa(dy_dxsi, xm(y[j], a.rule.dxi[q][j]));
					dy_deta = xa(dy_deta, xm(y[j], a.rule.deta[q][j]));
				}
				double const det = fabs(xs(xm(dx_dxsi, dy_deta), xm(dx_deta, dy_dxsi)));
				double dx[4], dy[4];
				for (int j = 0; j < kind; j++) {
					dx[j] = xd(xs(xm(a.rule.dxi[q][j], dy_deta), xm(a.rule.deta[q][j], dy_dxsi)), det);
					dy[j] = xd(xs(xm(a.rule.deta[q][j], dx_dxsi), xm(a.rule.dxi[q][j], dx_deta)), det);
				}
				double const dw = xm(det, w);
				double const ph = a.rule.phi[q][jr];
				for (int f = 0; f < a.forces.nf; f++) {
					double fx = a.forces.f[f][0], fy = a.forces.f[f][1];
					if (a.forces.field[f]) {
						fx = a.forces.field[f][2l * r];
						fy = a.forces.field[f][2l * r + 1];
					}
					b0 = xa(b0, xm(xm(xm(dw, fx), a.rho), ph));
					b1 = xa(b1, xm(xm(xm(dw, fy), a.rho), ph));
				}
				double const xj = dx[jr], yj = dy[jr];
				for (int k = 0; k < kind; k++) {
					double const f11 = xa(xm(xm(ea, xj), dx[k]), xm(xm(ec, yj), dy[k]));
					double const f12 = xa(xm(xm(eb, xj), dy[k]), xm(xm(ec, yj), dx[k]));
					double const f21 = xa(xm(xm(eb, yj), dx[k]), xm(xm(ec, xj), dy[k]));
					double const f22 = xa(xm(xm(ea, yj), dy[k]), xm(xm(ec, xj), dx[k]));
					int const s = slot[k];
					acc[s][0] = xa(acc[s][0], xm(dw, f11));
					acc[s][1] = xa(acc[s][1], xm(dw, f12));
					acc[s][2] = xa(acc[s][2], xm(dw, f21));
					acc[s][3] = xa(acc[s][3], xm(dw, f22));
				}
			}
		}
		else {
			// FP32 integration on coordinates relative to the element's first
			// node (taken in FP64), which keeps the Jacobian accurate for
			// small elements far from the origin.
			float lx[4], ly[4];
			for (int j = 0; j < kind; j++) {
				lx[j] = (float) (x[j] - x[0]);
				ly[j] = (float) (y[j] - y[0]);
			}
			float const fa = (float) ea, fb = (float) eb, fc = (float) ec;
			for (int q = 0; q < a.rule.nq; q++) {
				float const w = (float) a.rule.w[q];
				float dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0;
				for (int j = 0; j < kind; j++) {
					float const gx = (float) a.rule.dxi[q][j], ge = (float) a.rule.deta[q][j];
					dx_dxsi += lx[j] * gx;
					dx_deta += lx[j] * ge;
					dy_dxsi += ly[j] * gx;
					dy_deta += ly[j] * ge;
				}
				float const det = fabsf(dx_dxsi * dy_deta - dx_deta * dy_dxsi);
				float const idet = 1.0f / det;
				float dx[4], dy[4];
				for (int j = 0; j < kind; j++) {
					float const gx = (float) a.rule.dxi[q][j], ge = (float) a.rule.deta[q][j];
					dx[j] = (gx * dy_deta - ge * dy_dxsi) * idet;
					dy[j] = (ge * dx_dxsi - gx * dx_deta) * idet;
				}
				float const dw = det * w;
				double const ph = a.rule.phi[q][jr];
				for (int f = 0; f < a.forces.nf; f++) {
					double fx = a.forces.f[f][0], fy = a.forces.f[f][1];
					if (a.forces.field[f]) {
						fx = a.forces.field[f][2l * r];
						fy = a.forces.field[f][2l * r + 1];
					}
					b0 += (double) dw * fx * a.rho * ph;
					b1 += (double) dw * fy * a.rho * ph;
				}
				float const xj = dx[jr], yj = dy[jr];
				for (int k = 0; k < kind; k++) {
					int const s = slot[k];
					acc[s][0] += dw * (fa * xj * dx[k] + fc * yj * dy[k]);
					acc[s][1] += dw * (fb * xj * dy[k] + fc * yj * dx[k]);
					acc[s][2] += dw * (fb * yj * dx[k] + fc * xj * dy[k]);
					acc[s][3] += dw * (fa * yj * dy[k] + fc * xj * dx[k]);
				}
			}
		}
	}

	// symmetric Dirichlet elimination of this row
	int const r0 = 2 * r, r1 = 2 * r + 1;
	bool const c0 = a.last_ci[r0] >= 0, c1 = a.last_ci[r1] >= 0;
	double k00 = 0, k01 = 0, k10 = 0, k11 = 0;
	for (int s = 0; s < len; s++) {
		int const c = col[s];
		int const d0 = 2 * c, d1 = 2 * c + 1;
		bool const e0 = a.last_ci[d0] >= 0, e1 = a.last_ci[d1] >= 0;
		if (e0 || e1) {
			double const f0 = e0 ? a.first[d0] : 0.0, f1 = e1 ? a.first[d1] : 0.0;
			if (!c0) {
				if (e0) b0 -= f0 * (double) acc[s][0];
				if (e1) b0 -= f1 * (double) acc[s][1];
			}
			if (!c1) {
				if (e0) b1 -= f0 * (double) acc[s][2];
				if (e1) b1 -= f1 * (double) acc[s][3];
			}
		}
		T v[4] = {acc[s][0], acc[s][1], acc[s][2], acc[s][3]};
		if (c0 || e0) v[0] = (r0 == d0) ? T(1) : T(0);
		if (c0 || e1) v[1] = T(0);
		if (c1 || e0) v[2] = T(0);
		if (c1 || e1) v[3] = (r1 == d1) ? T(1) : T(0);
		long const o = 4l * (rs + s);
		if (a.vals64) {
			a.vals64[o + 0] = (double) v[0]; a.vals64[o + 1] = (double) v[1];
			a.vals64[o + 2] = (double) v[2]; a.vals64[o + 3] = (double) v[3];
		}
		if (a.vals32) {
			a.vals32[o + 0] = (float) v[0]; a.vals32[o + 1] = (float) v[1];
			a.vals32[o + 2] = (float) v[2]; a.vals32[o + 3] = (float) v[3];
		}
		if (c == r) {
			k00 = (double) v[0]; k01 = (double) v[1];
			k10 = (double) v[2]; k11 = (double) v[3];
		}
	}
	if (c0) b0 = a.last[r0];
	if (c1) b1 = a.last[r1];
	a.b[r0] = b0;
	a.b[r1] = b1;
	store_precond(a, r, k00, k01, k10, k11);
}

// Neumann X/Y loads (system.c:477-498), gathered per node in condition order
// then edge order (deterministic, no atomics).  A load on a constrained DOF
// survives only when applied after that DOF's last Dirichlet condition.
struct NeuArgs {
	int N, n_conds;
	int kinds[MAXC];
	double values[MAXC];
	const uint8_t* masks;
	const int* edges;
	const int* eptr;
	const int* elist;
	const double* coords;
	const int* last_ci;
	double* b;
};

__global__ void k_neumann(NeuArgs a) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= a.N) return;
	int const s = a.eptr[r], t = a.eptr[r + 1];
	if (s == t) return;
	double add0 = 0, add1 = 0;
	for (int ci = 0; ci < a.n_conds; ci++) {
		int const kd = a.kinds[ci];
		if (kd != BFM_CONDITION_KIND_NEUMANN_X && kd != BFM_CONDITION_KIND_NEUMANN_Y) continue;
		const uint8_t* m = a.masks + (long) ci * a.N;
		if (!m[r]) continue;
		int const shift = kd == BFM_CONDITION_KIND_NEUMANN_X ? 0 : 1;
		int const lc = a.last_ci[2 * r + shift];
		if (lc > ci) continue;
		for (int k = s; k < t; k++) {
			int const ed = a.elist[k];
			int const n1 = a.edges[2 * ed], n2 = a.edges[2 * ed + 1];
			if (!m[n1] || !m[n2]) continue;
			double const dx = a.coords[2l * n1] - a.coords[2l * n2];
			double const dy = a.coords[2l * n1 + 1] - a.coords[2l * n2 + 1];
			double const jac = sqrt(dx * dx + dy * dy) / 2;
			// an edge whose two ends are the same node adds twice, as in the reference
			int const mult = (n1 == r) + (n2 == r);
			for (int u = 0; u < mult; u++) {
				if (shift == 0) add0 += jac * a.values[ci];
				else add1 += jac * a.values[ci];
			}
		}
	}
	a.b[2 * r] += add0;
	a.b[2 * r + 1] += add1;
}

// ------------------------------------------------------------------ reductions

// Sum NV values over the whole grid: every block writes its partial sums,
// the last block to arrive (atomic ticket) adds them in block order and
// returns true with the totals in `out`.  The result does not depend on which
// block arrives last.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* __restrict__ partials, unsigned* ticket,
                                         double (&out)[NV]) {
	__shared__ double sm[TPB / 32][NV];
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

template <typename V>
struct CgArgs {
	int N;
	const int* row_ptr;
	const int* cols;
	const V* vals;          // iteration operator
	const double* vals64;   // FP64 operator for true residuals (nullptr: `vals` widened)
	const V* dinv;
	int block_pc;
	const double* b;
	double* x;
	V* r;
	V* p;
	V* s;
	V* w;
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgOpts opts;
	cudaGraphConditionalHandle cond;       // while-node: keep iterating
	cudaGraphConditionalHandle cond_repl;  // if-node: replace the residual this iteration
	int use_cond;  // launched inside the solve graph: drive its conditional nodes
	int timing;    // measurement launches: ignore the stop flag, never set it
	int mixed;     // FP32 recurrence with FP64 residual replacement
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

// 2x2 block k of the matrix: m0 m1 / m2 m3
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
__device__ __forceinline__ void precond_apply(const CgArgs<V>& a, int c, V r0, V r1, V& u0, V& u1) {
	if (a.block_pc) {
		V m0, m1, m2, m3;
		ld_block(a.dinv, c, m0, m1, m2, m3);
		u0 = m0 * r0 + m1 * r1;
		u1 = m2 * r0 + m3 * r1;
	}
	else {
		auto const d = ld2(a.dinv, c);
		u0 = d.x * r0;
		u1 = d.y * r1;
	}
}

// y = A_res x in FP64 for row i (the residual operator)
template <typename V>
__device__ __forceinline__ void spmv64_row(const CgArgs<V>& a, int i, double& y0, double& y1) {
	y0 = 0.0;
	y1 = 0.0;
	for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; k++) {
		int const c = a.cols[k];
		double2 const xc = ld2(a.x, c);
		double m0, m1, m2, m3;
		if (a.vals64) ld_block(a.vals64, k, m0, m1, m2, m3);
		else {
			V n0, n1, n2, n3;
			ld_block(a.vals, k, n0, n1, n2, n3);
			m0 = n0; m1 = n1; m2 = n2; m3 = n3;
		}
		y0 += m0 * xc.x + m1 * xc.y;
		y1 += m2 * xc.x + m3 * xc.y;
	}
}

template <typename V>
__global__ void __launch_bounds__(TPB) k_cg_init(CgArgs<V> a) {
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double2 const bb = ld2(a.b, i);
		st2(a.x, i, 0.0, 0.0);
		st2(a.r, i, (V) bb.x, (V) bb.y);
		st2(a.p, i, (V) 0, (V) 0);
		st2(a.s, i, (V) 0, (V) 0);
		v[0] += bb.x * bb.x + bb.y * bb.y;
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		CgState* st = a.st;
		st->bnorm2 = out[0];
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

// w = A u with u = M r formed on the fly; gamma = (r,u), delta = (w,u), rho = (r,r)
template <typename V>
__global__ void __launch_bounds__(TPB) k_cg_spmv_dots(CgArgs<V> a) {
	CgState* st = a.st;
	// The loop continues only if this launch's finisher says so: block 0
	// clears the conditions first, the last block sets them after the
	// stopping test.  A launch whose finisher did not run ends the loop.
	if (a.use_cond && blockIdx.x == 0 && threadIdx.x == 0) {
		cudaGraphSetConditional(a.cond, 0u);
		if (a.mixed) cudaGraphSetConditional(a.cond_repl, 0u);
	}
	if (st->done && !a.timing) return;
	double v[3] = {0.0, 0.0, 0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		int const ks = a.row_ptr[i], ke = a.row_ptr[i + 1];
		V y0 = 0, y1 = 0;
		for (int k = ks; k < ke; k++) {
			int const c = a.cols[k];
			auto const rc = ld2(a.r, c);
			V u0, u1;
			precond_apply(a, c, rc.x, rc.y, u0, u1);
			V m0, m1, m2, m3;
			ld_block(a.vals, k, m0, m1, m2, m3);
			y0 += m0 * u0 + m1 * u1;
			y1 += m2 * u0 + m3 * u1;
		}
		st2(a.w, i, y0, y1);
		auto const ri = ld2(a.r, i);
		V u0, u1;
		precond_apply(a, i, ri.x, ri.y, u0, u1);
		v[0] += (double) ri.x * (double) u0 + (double) ri.y * (double) u1;
		v[1] += (double) y0 * (double) u0 + (double) y1 * (double) u1;
		v[2] += (double) ri.x * (double) ri.x + (double) ri.y * (double) ri.y;
	}
	double out[3];
	if (grid_sum<3>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		double const gamma = out[0], delta = out[1], rho = out[2];
		double const tol2 = st->rtol * st->rtol * st->bnorm2;
		st->rho = rho;
		int stop = 0, repl = 0;
		if (!a.mixed && rho <= tol2) {
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
				// mixed: the FP32 recurrence has lost `drop` since the last
				// FP64 residual, or claims convergence -> refresh from FP64
				if (a.mixed) repl = rho <= st->drop2 * st->rho_ref || rho <= tol2;
			}
		}
		if (a.timing) return;
		st->done = stop;
		if (a.use_cond && !stop) {
			cudaGraphSetConditional(a.cond, 1u);
			if (repl) cudaGraphSetConditional(a.cond_repl, 1u);
		}
	}
}

template <typename V>
__global__ void __launch_bounds__(TPB) k_cg_update(CgArgs<V> a) {
	CgState const* st = a.st;
	if (st->done && !a.timing) return;
	V const alpha = (V) st->alpha, beta = (V) st->beta;
	double const alpha64 = st->alpha;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		auto const r = ld2(a.r, i);
		V u0, u1;
		precond_apply(a, i, r.x, r.y, u0, u1);
		auto const p = ld2(a.p, i);
		auto const s = ld2(a.s, i);
		auto const w = ld2(a.w, i);
		V const p0 = u0 + beta * p.x, p1 = u1 + beta * p.y;
		V const s0 = w.x + beta * s.x, s1 = w.y + beta * s.y;
		st2(a.p, i, p0, p1);
		st2(a.s, i, s0, s1);
		double2 const x = ld2(a.x, i);
		st2(a.x, i, x.x + alpha64 * (double) p0, x.y + alpha64 * (double) p1);
		st2(a.r, i, r.x - alpha * s0, r.y - alpha * s1);
	}
}

// Mixed precision, run only when requested (IF node): r = b - A_res x in
// FP64 (rounded to the iteration precision), s = A p afresh, and the FP64
// stopping test on the true residual.
template <typename V>
__global__ void __launch_bounds__(TPB) k_cg_replace(CgArgs<V> a) {
	CgState* st = a.st;
	if (st->done) return;
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double y0, y1;
		spmv64_row(a, i, y0, y1);
		double2 const bb = ld2(a.b, i);
		double const e0 = bb.x - y0, e1 = bb.y - y1;
		st2(a.r, i, (V) e0, (V) e1);
		v[0] += e0 * e0 + e1 * e1;
		V s0 = 0, s1 = 0;
		for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; k++) {
			int const c = a.cols[k];
			auto const pc = ld2(a.p, c);
			V m0, m1, m2, m3;
			ld_block(a.vals, k, m0, m1, m2, m3);
			s0 += m0 * pc.x + m1 * pc.y;
			s1 += m2 * pc.x + m3 * pc.y;
		}
		st2(a.s, i, s0, s1);
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		st->replacements += 1;
		st->rho_ref = out[0];
		st->true_res2 = out[0];
		if (out[0] <= st->rtol * st->rtol * st->bnorm2) {
			st->done = 1;
			if (a.use_cond) cudaGraphSetConditional(a.cond, 0u);
		}
	}
}

// ||b - A_res x||^2 in FP64
template <typename V>
__global__ void __launch_bounds__(TPB) k_true_residual(CgArgs<V> a) {
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double y0, y1;
		spmv64_row(a, i, y0, y1);
		double2 const bb = ld2(a.b, i);
		double const e0 = bb.x - y0, e1 = bb.y - y1;
		v[0] += e0 * e0 + e1 * e1;
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) a.st->true_res2 = out[0];
}

int g_num_sms = 0;

int num_sms() {
	if (!g_num_sms) {
		int dev = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
		if (g_num_sms <= 0) g_num_sms = 1;
	}
	return g_num_sms;
}

}  // namespace

// ====================================================================== host side

struct bfm_gpu_problem {
	int kind, N, NE, max_edges, max_conds;
	cudaStream_t stream;
	bool own_stream;
	int grid;  // persistent-style grid for the CG kernels (multiple of the SM count)

	// inputs
	double* coords;
	int* elems;
	double* elemE;
	double* elemNu;
	bool has_elemE, has_elemNu;
	double E, nu, rho;
	int stress;
	Rule rule;
	Forces forces;
	double* force_fields[MAXF];
	int n_conds;
	int kinds[MAXC];
	double values[MAXC];
	uint8_t* masks;
	int n_edges;
	int* edges;

	// pattern
	int *cnt, *inc_ptr, *inc, *cand, *row_len, *row_ptr, *cols;
	int *ecnt, *eptr, *elist;
	int* scan_sums;
	int* scan_total;
	long nb_cap;

	// system
	double* vals64;
	float* vals32;
	double* b;
	int* last_ci;
	double *first, *last;
	double* dinv64;
	float* dinv32;
	int precision, precond;

	// CG
	double* x;
	void *r, *p, *s, *w;  // double or float
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgState* st_host;  // pinned
	int* err;
	int* err_host;     // pinned

	cudaGraphExec_t graph;
	int graph_precision, graph_precond;
	bfm_gpu_opts_t graph_opts;

	cudaEvent_t ev[4];
	bool assembled, solved;
};

namespace {

thread_local char g_err[512];

int fail(const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof g_err, fmt, ap);
	va_end(ap);
	return -1;
}

#define CK(call)                                                                        \
	do {                                                                                \
		cudaError_t const e_ = (call);                                                  \
		if (e_ != cudaSuccess) {                                                        \
			snprintf(g_err, sizeof g_err, "CUDA error %s at %s:%d", cudaGetErrorString(e_), \
			         __FILE__, __LINE__);                                               \
			return -1;                                                                  \
		}                                                                               \
	} while (0)

template <typename T>
int dalloc(T** p, size_t n) {
	*p = nullptr;
	if (n == 0) n = 1;
	cudaError_t const e = cudaMalloc((void**) p, n * sizeof(T));
	if (e != cudaSuccess) {
		snprintf(g_err, sizeof g_err, "cudaMalloc of %zu bytes failed: %s", n * sizeof(T), cudaGetErrorString(e));
		return -1;
	}
	return 0;
}

inline int blocks_for(long n, int tpb = TPB) { return (int) ((n + tpb - 1) / tpb) > 0 ? (int) ((n + tpb - 1) / tpb) : 1; }

int scan(bfm_gpu_problem* P, const int* in, int* out, int n) {
	int const tiles = (n + SCAN_TILE - 1) / SCAN_TILE > 0 ? (n + SCAN_TILE - 1) / SCAN_TILE : 1;
	k_scan_tiles<<<tiles, TPB, 0, P->stream>>>(in, out, n, P->scan_sums);
	k_scan_spine<<<1, TPB, 0, P->stream>>>(P->scan_sums, tiles, P->scan_total);
	k_scan_add<<<blocks_for(n > 0 ? n : 1), TPB, 0, P->stream>>>(out, n, P->scan_sums, P->scan_total);
	CK(cudaGetLastError());
	return 0;
}

// node -> item incidence lists (ascending), items of `arity` nodes each
int incidence(bfm_gpu_problem* P, const int* items, int n_items, int arity, int* cnt, int* ptr, int* list, int maxlen, int code) {
	long const total = (long) n_items * arity;
	CK(cudaMemsetAsync(cnt, 0, (P->N + 1) * sizeof(int), P->stream));
	int const g = 4 * num_sms();
	if (total) k_count<<<g, TPB, 0, P->stream>>>(items, total, cnt);
	if (scan(P, cnt, ptr, P->N)) return -1;
	CK(cudaMemsetAsync(cnt, 0, (P->N + 1) * sizeof(int), P->stream));
	if (total) k_fill<<<g, TPB, 0, P->stream>>>(items, total, arity, ptr, cnt, list);
	k_sort_lists<<<blocks_for(P->N), TPB, 0, P->stream>>>(P->N, ptr, list, maxlen, P->err, code);
	CK(cudaGetLastError());
	return 0;
}

template <typename V>
CgArgs<V> cg_args(bfm_gpu_problem* P, const bfm_gpu_opts_t* o) {
	CgArgs<V> a;
	memset(&a, 0, sizeof a);
	a.N = P->N;
	a.row_ptr = P->row_ptr;
	a.cols = P->cols;
	if constexpr (sizeof(V) == 8) {
		a.vals = P->vals64;
		a.dinv = P->dinv64;
		a.vals64 = P->vals64;
	}
	else {
		a.vals = P->vals32;
		a.dinv = P->dinv32;
		a.vals64 = P->precision == BFM_GPU_MIXED_EXACT ? P->vals64 : nullptr;
		a.mixed = 1;
	}
	a.block_pc = P->precond == BFM_GPU_PC_BLOCK_JACOBI;
	a.b = P->b;
	a.x = P->x;
	a.r = (V*) P->r;
	a.p = (V*) P->p;
	a.s = (V*) P->s;
	a.w = (V*) P->w;
	a.partials = P->partials;
	a.ticket = P->ticket;
	a.st = P->st;
	if (o) {
		a.opts.rtol = o->rtol;
		a.opts.drop2 = o->replace_drop * o->replace_drop;
		a.opts.max_iters = o->max_iters;
	}
	return a;
}

template <typename V>
int add_kernel(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* deps, int ndeps, void* fn, int grid, CgArgs<V>* args) {
	cudaKernelNodeParams kp = {};
	void* params[1] = {args};
	kp.func = fn;
	kp.gridDim = dim3(grid);
	kp.blockDim = dim3(TPB);
	kp.sharedMemBytes = 0;
	kp.kernelParams = params;
	CK(cudaGraphAddKernelNode(node, g, deps, ndeps, &kp));
	return 0;
}

// init -> while(running){ spmv+dots ; update ; [mixed: if(replace){ FP64 residual }] } -> true residual
template <typename V>
int build_graph(bfm_gpu_problem* P, const bfm_gpu_opts_t* o) {
	cudaGraph_t g;
	CK(cudaGraphCreate(&g, 0));
	CgArgs<V> a = cg_args<V>(P, o);
	a.use_cond = 1;
	CK(cudaGraphConditionalHandleCreate(&a.cond, g, 1u, cudaGraphCondAssignDefault));
	cudaGraphNode_t n_init, n_cond, n_a, n_b, n_if, n_r, n_res;
	// the body's if-handle is created once the body graph exists; the
	// kernels of every node must carry it, so add the nodes afterwards
	cudaGraphNodeParams cp = {};
	cp.type = cudaGraphNodeTypeConditional;
	cp.conditional.handle = a.cond;
	cp.conditional.type = cudaGraphCondTypeWhile;
	cp.conditional.size = 1;
	// init first (no dependency), then the while node after it
	CgArgs<V> a0 = a;
	if (add_kernel<V>(g, &n_init, nullptr, 0, (void*) k_cg_init<V>, P->grid, &a0)) return -1;
	CK(cudaGraphAddNode(&n_cond, g, &n_init, nullptr, 1, &cp));
	cudaGraph_t body = cp.conditional.phGraph_out[0];
	cudaGraphNodeParams ip = {};
	if (a.mixed) {
		CK(cudaGraphConditionalHandleCreate(&a.cond_repl, body, 0u, cudaGraphCondAssignDefault));
		ip.type = cudaGraphNodeTypeConditional;
		ip.conditional.handle = a.cond_repl;
		ip.conditional.type = cudaGraphCondTypeIf;
		ip.conditional.size = 1;
	}
	if (add_kernel<V>(body, &n_a, nullptr, 0, (void*) k_cg_spmv_dots<V>, P->grid, &a)) return -1;
	if (add_kernel<V>(body, &n_b, &n_a, 1, (void*) k_cg_update<V>, P->grid, &a)) return -1;
	if (a.mixed) {
		CK(cudaGraphAddNode(&n_if, body, &n_b, nullptr, 1, &ip));
		if (add_kernel<V>(ip.conditional.phGraph_out[0], &n_r, nullptr, 0, (void*) k_cg_replace<V>, P->grid, &a)) return -1;
	}
	if (add_kernel<V>(g, &n_res, &n_cond, 1, (void*) k_true_residual<V>, P->grid, &a)) return -1;
	if (P->graph) cudaGraphExecDestroy(P->graph);
	P->graph = nullptr;
	CK(cudaGraphInstantiate(&P->graph, g, 0));
	cudaGraphDestroy(g);
	return 0;
}

}  // namespace

extern "C" {

const char* bfm_gpu_last_error(void) { return g_err; }

int bfm_gpu_device_count(void) {
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess) {
		cudaGetLastError();
		return 0;
	}
	return n;
}

void bfm_gpu_default_opts(bfm_gpu_opts_t* o) {
	o->precision = BFM_GPU_FP64;
	o->precond = BFM_GPU_PC_JACOBI;
	o->rtol = 1e-10;
	o->max_iters = 200000;
	o->replace_drop = 1e-2;
	o->deterministic = 1;
}

int bfm_gpu_problem_create(bfm_gpu_problem_t** out, int kind, int n_nodes, int n_elems, int n_edges, int n_conds, void* stream) {
	g_err[0] = 0;
	*out = nullptr;
	if (kind != 3 && kind != 4) return fail("element kind %d must be 3 (P1) or 4 (Q1)", kind);
	if (n_nodes < 0 || n_elems < 0 || n_edges < 0 || n_conds < 0) return fail("negative size");
	if (n_conds > MAXC) return fail("at most 16 conditions per instance are supported");
	if ((long) n_elems * kind * kind > 2000000000l) return fail("mesh too large for 32-bit block indices");
	if (bfm_gpu_device_count() <= 0) return fail("no CUDA device available (the GPU path has no CPU fallback)");
	bfm_gpu_problem* P = (bfm_gpu_problem*) calloc(1, sizeof *P);
	if (!P) return fail("out of host memory");
	P->kind = kind;
	P->N = n_nodes;
	P->NE = n_elems;
	P->max_edges = n_edges;
	P->max_conds = n_conds;
	P->precision = -1;
	P->graph_precision = -1;
	if (stream) {
		P->stream = (cudaStream_t) stream;
		P->own_stream = false;
	}
	else {
		if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess) {
			free(P);
			return fail("cudaStreamCreate failed");
		}
		P->own_stream = true;
	}
	int const sms = num_sms();
	P->grid = sms * 4;
	long const N = n_nodes, E = n_elems;
	long const inc_total = E * kind;
	P->nb_cap = inc_total * kind > N ? inc_total * kind : N;
	long const tiles = (N + SCAN_TILE) / SCAN_TILE + 1;
	*out = P;
	if (dalloc(&P->coords, 2 * N) || dalloc(&P->elems, inc_total) || dalloc(&P->masks, (long) (n_conds ? n_conds : 1) * N) ||
	    dalloc(&P->edges, 2l * n_edges) || dalloc(&P->cnt, N + 1) || dalloc(&P->inc_ptr, N + 1) || dalloc(&P->inc, inc_total) ||
	    dalloc(&P->cand, inc_total * kind) || dalloc(&P->row_len, N + 1) || dalloc(&P->row_ptr, N + 1) ||
	    dalloc(&P->cols, P->nb_cap) || dalloc(&P->ecnt, N + 1) || dalloc(&P->eptr, N + 1) || dalloc(&P->elist, 2l * n_edges) ||
	    dalloc(&P->scan_sums, tiles) || dalloc(&P->scan_total, 1) || dalloc(&P->b, 2 * N) || dalloc(&P->last_ci, 2 * N) ||
	    dalloc(&P->first, 2 * N) || dalloc(&P->last, 2 * N) || dalloc(&P->x, 2 * N) || dalloc(&P->partials, 4l * P->grid) ||
	    dalloc(&P->ticket, 1) || dalloc(&P->st, 1) || dalloc(&P->err, 1)) {
		bfm_gpu_problem_destroy(P);
		*out = nullptr;
		return -1;
	}
	if (cudaMallocHost((void**) &P->st_host, sizeof(CgState)) != cudaSuccess ||
	    cudaMallocHost((void**) &P->err_host, sizeof(int)) != cudaSuccess) {
		bfm_gpu_problem_destroy(P);
		*out = nullptr;
		return fail("cudaMallocHost failed");
	}
	for (int i = 0; i < 4; i++) cudaEventCreate(&P->ev[i]);
	cudaMemsetAsync(P->ticket, 0, sizeof(unsigned), P->stream);
	cudaMemsetAsync(P->err, 0, sizeof(int), P->stream);
	cudaMemsetAsync(P->st, 0, sizeof(CgState), P->stream);
	CK(cudaGetLastError());
	return 0;
}

int bfm_gpu_problem_destroy(bfm_gpu_problem_t* P) {
	if (!P) return 0;
	if (P->stream) cudaStreamSynchronize(P->stream);
	if (P->graph) cudaGraphExecDestroy(P->graph);
	void* bufs[] = {P->coords, P->elems, P->elemE, P->elemNu, P->masks, P->edges, P->cnt, P->inc_ptr, P->inc, P->cand,
	                P->row_len, P->row_ptr, P->cols, P->ecnt, P->eptr, P->elist, P->scan_sums, P->scan_total, P->vals64,
	                P->vals32, P->b, P->last_ci, P->first, P->last, P->dinv64, P->dinv32, P->x, P->r, P->p, P->s, P->w,
	                P->partials, P->ticket, P->st, P->err};
	for (void* p : bufs)
		if (p) cudaFree(p);
	for (int i = 0; i < MAXF; i++)
		if (P->force_fields[i]) cudaFree(P->force_fields[i]);
	if (P->st_host) cudaFreeHost(P->st_host);
	if (P->err_host) cudaFreeHost(P->err_host);
	for (int i = 0; i < 4; i++)
		if (P->ev[i]) cudaEventDestroy(P->ev[i]);
	if (P->own_stream && P->stream) cudaStreamDestroy(P->stream);
	free(P);
	return 0;
}

void* bfm_gpu_problem_stream(bfm_gpu_problem_t* P) { return (void*) P->stream; }

static cudaMemcpyKind kind_of(int where) { return where == BFM_GPU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }

int bfm_gpu_problem_set_geometry(bfm_gpu_problem_t* P, const double* coords, const int32_t* elems, int where) {
	g_err[0] = 0;
	CK(cudaMemcpyAsync(P->coords, coords, 2l * P->N * sizeof(double), kind_of(where), P->stream));
	CK(cudaMemcpyAsync(P->elems, elems, (long) P->NE * P->kind * sizeof(int), kind_of(where), P->stream));
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_material(bfm_gpu_problem_t* P, double E, double nu, double rho, int stress, const double* elem_E,
                                 const double* elem_nu, int where) {
	g_err[0] = 0;
	P->E = E;
	P->nu = nu;
	P->rho = rho;
	P->stress = stress;
	P->has_elemE = elem_E != nullptr;
	P->has_elemNu = elem_nu != nullptr;
	if (elem_E) {
		if (!P->elemE && dalloc(&P->elemE, P->NE)) return -1;
		CK(cudaMemcpyAsync(P->elemE, elem_E, (long) P->NE * sizeof(double), kind_of(where), P->stream));
	}
	if (elem_nu) {
		if (!P->elemNu && dalloc(&P->elemNu, P->NE)) return -1;
		CK(cudaMemcpyAsync(P->elemNu, elem_nu, (long) P->NE * sizeof(double), kind_of(where), P->stream));
	}
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_rule(bfm_gpu_problem_t* P, int n_points, const double* weights, const double* phi, const double* dxi,
                             const double* deta) {
	g_err[0] = 0;
	if (n_points < 0 || n_points > MAXQ) return fail("integration rules of at most 16 points are supported");
	P->rule.nq = n_points;
	for (int q = 0; q < n_points; q++) {
		P->rule.w[q] = weights[q];
		for (int j = 0; j < P->kind; j++) {
			P->rule.phi[q][j] = phi[q * P->kind + j];
			P->rule.dxi[q][j] = dxi[q * P->kind + j];
			P->rule.deta[q][j] = deta[q * P->kind + j];
		}
	}
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_forces(bfm_gpu_problem_t* P, int n_forces, const double* values, const double* const* node_values, int where) {
	g_err[0] = 0;
	if (n_forces < 0 || n_forces > MAXF) return fail("at most 8 body forces are supported");
	P->forces.nf = n_forces;
	for (int f = 0; f < n_forces; f++) {
		P->forces.f[f][0] = values ? values[2 * f] : 0.0;
		P->forces.f[f][1] = values ? values[2 * f + 1] : 0.0;
		P->forces.field[f] = nullptr;
		if (node_values && node_values[f]) {
			if (!P->force_fields[f] && dalloc(&P->force_fields[f], 2l * P->N)) return -1;
			CK(cudaMemcpyAsync(P->force_fields[f], node_values[f], 2l * P->N * sizeof(double), kind_of(where), P->stream));
			P->forces.field[f] = P->force_fields[f];
		}
	}
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_conditions(bfm_gpu_problem_t* P, int n_conds, const int* kinds, const double* values, const uint8_t* masks,
                                   int n_edges, const int32_t* edges, int where) {
	g_err[0] = 0;
	if (n_conds > P->max_conds || n_conds < 0) return fail("more conditions than the problem was created for");
	if (n_edges > P->max_edges || n_edges < 0) return fail("more edges than the problem was created for");
	for (int c = 0; c < n_conds; c++) {
		int const k = kinds[c];
		if (k != BFM_CONDITION_KIND_DIRICHLET_X && k != BFM_CONDITION_KIND_DIRICHLET_Y && k != BFM_CONDITION_KIND_NEUMANN_X &&
		    k != BFM_CONDITION_KIND_NEUMANN_Y)
			return fail("condition kind %d is not supported on the GPU path (X/Y Dirichlet and Neumann only)", k);
		P->kinds[c] = k;
		P->values[c] = values[c];
	}
	P->n_conds = n_conds;
	P->n_edges = n_edges;
	if (n_conds) CK(cudaMemcpyAsync(P->masks, masks, (long) n_conds * P->N, kind_of(where), P->stream));
	if (n_edges) CK(cudaMemcpyAsync(P->edges, edges, 2l * n_edges * sizeof(int), kind_of(where), P->stream));
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_assemble(bfm_gpu_problem_t* P, int precision) {
	g_err[0] = 0;
	if (precision != BFM_GPU_FP64 && precision != BFM_GPU_MIXED && precision != BFM_GPU_MIXED_EXACT)
		return fail("unknown precision %d", precision);
	bool const want64 = precision != BFM_GPU_MIXED;  // FP64 values: the operator, or the residual operator
	bool const want32 = precision != BFM_GPU_FP64;   // FP32 values: the mixed iteration operator
	cudaStream_t const st = P->stream;
	long const N = P->N;
	// value storage for this precision (allocated once, on first use)
	if (want64 && !P->vals64 && dalloc(&P->vals64, 4 * P->nb_cap)) return -1;
	if (want32 && !P->vals32 && dalloc(&P->vals32, 4 * P->nb_cap)) return -1;
	if (!want32 && !P->dinv64 && dalloc(&P->dinv64, 4 * N)) return -1;
	if (want32 && !P->dinv32 && dalloc(&P->dinv32, 4 * N)) return -1;
	size_t const vsz = precision == BFM_GPU_FP64 ? sizeof(double) : sizeof(float);
	if ((P->precision == BFM_GPU_FP64) != (precision == BFM_GPU_FP64) || !P->r) {
		void** vecs[] = {&P->r, &P->p, &P->s, &P->w};
		for (void** v : vecs) {
			if (*v) cudaFree(*v);
			*v = nullptr;
			CK(cudaMalloc(v, 2 * (N ? N : 1) * vsz));
		}
	}
	P->precision = precision;
	CK(cudaEventRecord(P->ev[0], st));
	CK(cudaMemsetAsync(P->err, 0, sizeof(int), st));
	// 1. node -> element incidence, ascending
	if (incidence(P, P->elems, P->NE, P->kind, P->cnt, P->inc_ptr, P->inc, MAXV, ERR_VALENCE)) return -1;
	// 2. node-block pattern
	k_rows_count<<<blocks_for(N), TPB, 0, st>>>(P->N, P->kind, P->elems, P->inc_ptr, P->inc, P->cand, P->row_len, P->err);
	if (scan(P, P->row_len, P->row_ptr, P->N)) return -1;
	k_rows_fill<<<blocks_for(N), TPB, 0, st>>>(P->N, P->kind, P->inc_ptr, P->cand, P->row_ptr, P->cols);
	// 3. Dirichlet bookkeeping, conditions in order
	CK(cudaMemsetAsync(P->last_ci, 0xff, 2 * N * sizeof(int), st));
	for (int c = 0; c < P->n_conds; c++) {
		int const k = P->kinds[c];
		if (k == BFM_CONDITION_KIND_DIRICHLET_X || k == BFM_CONDITION_KIND_DIRICHLET_Y)
			k_dirichlet_mark<<<blocks_for(N), TPB, 0, st>>>(P->N, c, k == BFM_CONDITION_KIND_DIRICHLET_X ? 0 : 1, P->values[c],
			                                                 P->masks + (long) c * N, P->last_ci, P->first, P->last);
	}
	// 4. element loop + elimination + preconditioner diagonal
	AsmArgs a;
	memset(&a, 0, sizeof a);
	a.N = P->N;
	a.kind = P->kind;
	a.stress = P->stress;
	a.coords = P->coords;
	a.elems = P->elems;
	a.elemE = P->has_elemE ? P->elemE : nullptr;
	a.elemNu = P->has_elemNu ? P->elemNu : nullptr;
	a.E = P->E;
	a.nu = P->nu;
	a.rho = P->rho;
	a.rule = P->rule;
	a.forces = P->forces;
	a.inc_ptr = P->inc_ptr;
	a.inc = P->inc;
	a.row_ptr = P->row_ptr;
	a.cols = P->cols;
	a.last_ci = P->last_ci;
	a.first = P->first;
	a.last = P->last;
	a.vals64 = want64 ? P->vals64 : nullptr;
	a.vals32 = want32 ? P->vals32 : nullptr;
	a.b = P->b;
	a.dinv64 = want32 ? nullptr : P->dinv64;
	a.dinv32 = want32 ? P->dinv32 : nullptr;
	a.precond = P->precond;
	a.err = P->err;
	if (precision != BFM_GPU_MIXED) k_assemble<true><<<blocks_for(N, 128), 128, 0, st>>>(a);
	else k_assemble<false><<<blocks_for(N, 128), 128, 0, st>>>(a);
	// 5. Neumann loads
	bool has_neu = false;
	for (int c = 0; c < P->n_conds; c++)
		has_neu |= P->kinds[c] == BFM_CONDITION_KIND_NEUMANN_X || P->kinds[c] == BFM_CONDITION_KIND_NEUMANN_Y;
	if (has_neu && P->n_edges) {
		if (incidence(P, P->edges, P->n_edges, 2, P->ecnt, P->eptr, P->elist, 2 * MAXV, ERR_EDGE_VALENCE)) return -1;
		NeuArgs na;
		memset(&na, 0, sizeof na);
		na.N = P->N;
		na.n_conds = P->n_conds;
		for (int c = 0; c < P->n_conds; c++) {
			na.kinds[c] = P->kinds[c];
			na.values[c] = P->values[c];
		}
		na.masks = P->masks;
		na.edges = P->edges;
		na.eptr = P->eptr;
		na.elist = P->elist;
		na.coords = P->coords;
		na.last_ci = P->last_ci;
		na.b = P->b;
		k_neumann<<<blocks_for(N), TPB, 0, st>>>(na);
	}
	CK(cudaGetLastError());
	CK(cudaEventRecord(P->ev[1], st));
	P->assembled = true;
	P->solved = false;
	return 0;
}

int bfm_gpu_problem_solve(bfm_gpu_problem_t* P, const bfm_gpu_opts_t* opts) {
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble before solving");
	bfm_gpu_opts_t o;
	if (opts) o = *opts;
	else bfm_gpu_default_opts(&o);
	if (!(o.rtol >= 0.0) || o.max_iters < 0) return fail("invalid solver options");
	if (o.precond == BFM_GPU_PC_LEARNED) return fail("learned preconditioner not available in this build");
	if (o.precond != P->precond) {
		// the preconditioner is formed by the assembly epilogue
		P->precond = o.precond;
		if (bfm_gpu_problem_assemble(P, P->precision)) return -1;
	}
	// options are baked into the graph's kernel parameters: rebuild only when they change
	bool const same = P->graph && P->graph_precision == P->precision && P->graph_precond == P->precond &&
	                  P->graph_opts.rtol == o.rtol && P->graph_opts.max_iters == o.max_iters &&
	                  P->graph_opts.replace_drop == o.replace_drop;
	if (!same) {
		int const rc = P->precision == BFM_GPU_FP64 ? build_graph<double>(P, &o) : build_graph<float>(P, &o);
		if (rc) return -1;
		P->graph_precision = P->precision;
		P->graph_precond = P->precond;
		P->graph_opts = o;
	}
	CK(cudaEventRecord(P->ev[2], P->stream));
	CK(cudaGraphLaunch(P->graph, P->stream));
	CK(cudaEventRecord(P->ev[3], P->stream));
	P->solved = true;
	return 0;
}

int bfm_gpu_problem_stats(bfm_gpu_problem_t* P, bfm_gpu_stats_t* s) {
	g_err[0] = 0;
	memset(s, 0, sizeof *s);
	CK(cudaMemcpyAsync(P->err_host, P->err, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
	CK(cudaMemcpyAsync(P->st_host, P->st, sizeof(CgState), cudaMemcpyDeviceToHost, P->stream));
	int nb = 0;
	CK(cudaMemcpyAsync(&nb, P->row_ptr + P->N, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
	CK(cudaStreamSynchronize(P->stream));
	s->n_blocks = P->assembled ? nb : 0;
	s->n_dof = 2l * P->N;
	float ms = 0;
	if (P->assembled && cudaEventElapsedTime(&ms, P->ev[0], P->ev[1]) == cudaSuccess) s->ms_assemble = ms;
	if (P->solved && cudaEventElapsedTime(&ms, P->ev[2], P->ev[3]) == cudaSuccess) s->ms_solve = ms;
	cudaGetLastError();
	if (*P->err_host) {
		s->status = BFM_GPU_BAD_MESH;
		snprintf(g_err, sizeof g_err,
		         "mesh exceeds the kernel caps (code %d): at most %d elements per node and %d neighbour nodes per node",
		         *P->err_host, MAXV, MAXR);
		return 0;
	}
	if (P->solved) {
		CgState const* h = P->st_host;
		s->status = h->status;
		s->iterations = h->iter;
		s->replacements = h->replacements;
		s->rel_residual = h->bnorm2 > 0 ? sqrt(h->true_res2 / h->bnorm2) : 0.0;
	}
	return 0;
}

int bfm_gpu_problem_solution(bfm_gpu_problem_t* P, double* out, int where) {
	g_err[0] = 0;
	CK(cudaMemcpyAsync(out, P->x, 2l * P->N * sizeof(double),
	                   where == BFM_GPU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
	if (where != BFM_GPU_DEVICE) CK(cudaStreamSynchronize(P->stream));
	return 0;
}

int bfm_gpu_problem_n_blocks(bfm_gpu_problem_t* P, int64_t* n_blocks) {
	g_err[0] = 0;
	int nb = 0;
	CK(cudaMemcpyAsync(&nb, P->row_ptr + P->N, sizeof(int), cudaMemcpyDeviceToHost, P->stream));
	CK(cudaStreamSynchronize(P->stream));
	*n_blocks = nb;
	return 0;
}

int bfm_gpu_problem_download(bfm_gpu_problem_t* P, int32_t* row_ptr, int32_t* cols, double* vals, double* b) {
	g_err[0] = 0;
	int64_t nb = 0;
	if (bfm_gpu_problem_n_blocks(P, &nb)) return -1;
	if (row_ptr) CK(cudaMemcpy(row_ptr, P->row_ptr, (P->N + 1) * sizeof(int), cudaMemcpyDeviceToHost));
	if (cols) CK(cudaMemcpy(cols, P->cols, nb * sizeof(int), cudaMemcpyDeviceToHost));
	if (vals) {
		if (P->precision == BFM_GPU_FP64) CK(cudaMemcpy(vals, P->vals64, 4 * nb * sizeof(double), cudaMemcpyDeviceToHost));
		else {
			float* tmp = (float*) malloc(4 * nb * sizeof(float) + 1);
			if (!tmp) return fail("out of host memory");
			cudaError_t const e = cudaMemcpy(tmp, P->vals32, 4 * nb * sizeof(float), cudaMemcpyDeviceToHost);
			for (int64_t i = 0; i < 4 * nb; i++) vals[i] = tmp[i];
			free(tmp);
			CK(e);
		}
	}
	if (b) CK(cudaMemcpy(b, P->b, 2l * P->N * sizeof(double), cudaMemcpyDeviceToHost));
	return 0;
}

// Launch the CG's two per-iteration kernels `reps` times each on the
// problem's stream (outside the graph, on a scratch copy of the solver state)
// and report their mean durations from CUDA events.  Overwrites the Krylov
// vectors: call after the solution has been read.
int bfm_gpu_problem_time_kernels(bfm_gpu_problem_t* P, int reps, double* ms_spmv, double* ms_update) {
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble first");
	CgState* scratch = nullptr;
	if (dalloc(&scratch, 1)) return -1;
	CgState h;
	memset(&h, 0, sizeof h);
	h.rtol = 0.0;
	h.max_iters = 1 << 30;
	h.bnorm2 = 1.0;
	CK(cudaMemcpyAsync(scratch, &h, sizeof h, cudaMemcpyHostToDevice, P->stream));
	cudaEvent_t e[3];
	for (auto& x : e) cudaEventCreate(&x);
	float t1 = 0, t2 = 0;
	if (P->precision == BFM_GPU_FP64) {
		CgArgs<double> a = cg_args<double>(P, nullptr);
		a.opts.rtol = 0.0;
		a.opts.max_iters = 1 << 30;
		a.st = scratch;
		a.timing = 1;
		k_cg_init<double><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaMemcpyAsync(scratch, &h, sizeof h, cudaMemcpyHostToDevice, P->stream);
		cudaEventRecord(e[0], P->stream);
		for (int i = 0; i < reps; i++) k_cg_spmv_dots<double><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaEventRecord(e[1], P->stream);
		for (int i = 0; i < reps; i++) k_cg_update<double><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaEventRecord(e[2], P->stream);
	}
	else {
		CgArgs<float> a = cg_args<float>(P, nullptr);
		a.opts.rtol = 0.0;
		a.opts.max_iters = 1 << 30;
		a.st = scratch;
		a.timing = 1;
		k_cg_init<float><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaMemcpyAsync(scratch, &h, sizeof h, cudaMemcpyHostToDevice, P->stream);
		cudaEventRecord(e[0], P->stream);
		for (int i = 0; i < reps; i++) k_cg_spmv_dots<float><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaEventRecord(e[1], P->stream);
		for (int i = 0; i < reps; i++) k_cg_update<float><<<P->grid, TPB, 0, P->stream>>>(a);
		cudaEventRecord(e[2], P->stream);
	}
	cudaError_t const err = cudaStreamSynchronize(P->stream);
	cudaEventElapsedTime(&t1, e[0], e[1]);
	cudaEventElapsedTime(&t2, e[1], e[2]);
	for (auto& x : e) cudaEventDestroy(x);
	cudaFree(scratch);
	CK(err);
	*ms_spmv = t1 / reps;
	*ms_update = t2 / reps;
	return 0;
}

}  // extern "C"
