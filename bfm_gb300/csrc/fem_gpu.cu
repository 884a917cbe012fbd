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

#include "internal.h"
#include "trace.h"

#include <pthread.h>
#include <stdarg.h>
#include <algorithm>
#include <type_traits>
#include <vector>

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

// material constants, reference system.c:454-458 (same operation order).
// stress 0 plane strain, 1 plane stress, 2 axisymmetric (the plane-strain
// constants), 3 axisymmetric with the constant a of system.c:241, which
// multiplies by (1 - 2 nu) where it should divide
__device__ __forceinline__ void material_abc(double E, double nu, int stress, double& a, double& b, double& c) {
	if (stress != 1) {
		double const den = xs(1.0, xm(2.0, nu));
		a = xd(xd(xm(E, xs(1.0, nu)), xa(1.0, nu)), den);
		if (stress == 3) a = xm(xd(xm(E, xs(1.0, nu)), xa(1.0, nu)), den);
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

// ------------------------------------------------------------------ multicolour node order
// The SSOR preconditioners sweep the nodes colour by colour (no two nodes of
// one colour share an element), so the problem is renumbered colour-major:
// then every block row lists its lower-colour neighbours, its diagonal block
// and its higher-colour neighbours in that order, and a colour is a
// contiguous range of rows.

// dst[i] = src[map[i]] for `width` consecutive elements per node
template <typename T>
__global__ void k_gather_nodes(long N, int width, const T* __restrict__ src, const int* __restrict__ map, T* __restrict__ dst) {
	long const t = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (t >= N * width) return;
	long const i = t / width;
	int const k = (int) (t - i * width);
	dst[t] = src[(long) map[i] * width + k];
}

// order-independent 64-bit fingerprint of the element array (each entry
// mixed with its position, XOR-combined): a colouring is reused while it matches
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
	x ^= x >> 33;
	x *= 0xff51afd7ed558ccdull;
	x ^= x >> 33;
	x *= 0xc4ceb9fe1a85ec53ull;
	x ^= x >> 33;
	return x;
}
// 64-bit node ids of the reference's element array (size_t) to the int32 ids
// the kernels use; an id at or beyond N records the lowest such position
__global__ void k_elems_from_u64(long n, int N, const unsigned long long* __restrict__ in, int* __restrict__ out,
                                 unsigned long long* __restrict__ bad) {
	long const i = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (i >= n) return;
	unsigned long long const v = in[i];
	if (v >= (unsigned long long) N) {
		atomicMin(bad, (unsigned long long) i);
		out[i] = 0;
	}
	else out[i] = (int) v;
}

__global__ void k_elems_hash(long n, const int* __restrict__ elems, unsigned long long* __restrict__ out) {
	unsigned long long h = 0;
	for (long t = blockIdx.x * (long) blockDim.x + threadIdx.x; t < n; t += (long) gridDim.x * blockDim.x)
		h ^= mix64(((unsigned long long) t << 32) ^ (unsigned) elems[t]);
	for (int o = 16; o; o >>= 1) h ^= __shfl_xor_sync(0xffffffffu, h, o);
	if ((threadIdx.x & 31) == 0 && h) atomicXor(out, h);
}

// node ids through a map (ids outside [0, N) stay: the pattern kernels report them)
__global__ void k_map_ids(long n, int N, int* __restrict__ ids, const int* __restrict__ map) {
	long const t = blockIdx.x * (long) blockDim.x + threadIdx.x;
	if (t >= n) return;
	int const v = ids[t];
	if (v >= 0 && v < N) ids[t] = map[v];
}

// first block of each row at or after the diagonal: the lower-colour
// neighbours are [row_ptr[i], dpos[i]), the higher-colour ones follow the
// diagonal block
// ------------------------------------------------------------------ sliced ELL of the SSOR sweeps

// slices of 32 consecutive rows of one colour: colour c's slices start at
// sbase[c] (sbase[ncol] = all slices)
struct SellMap {
	int ncol;
	int off[65];
	int sbase[65];
};

// row of slice s and lane (or -1 past the colour's last row), its colour in c
__device__ __forceinline__ int sell_row_of(const SellMap& m, int s, int lane, int& c) {
	c = 0;
	while (c + 1 < m.ncol && m.sbase[c + 1] <= s) c++;
	int const row = m.off[c] + ((s - m.sbase[c]) << 5) + lane;
	return row < m.off[c + 1] ? row : -1;
}

// per slice (one warp each): 32 x the most lower-colour and the most
// higher-colour blocks any of its rows has
__global__ void k_sell_width(int ns, SellMap m, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                             int* __restrict__ lw, int* __restrict__ uw) {
	int const s = (int) ((blockIdx.x * (long) blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
	if (s >= ns) return;  // whole warps
	int c;
	int const row = sell_row_of(m, s, lane, c);
	int nl = 0, nu = 0;
	if (row >= 0)
		for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
			int const j = cols[k];
			nl += j < m.off[c];
			nu += j >= m.off[c + 1];
		}
	nl = __reduce_max_sync(0xffffffffu, nl);
	nu = __reduce_max_sync(0xffffffffu, nu);
	if (lane == 0) {
		lw[s] = 32 * nl;
		uw[s] = 32 * nu;
	}
}

// the widest slice of colour blockIdx.x, lower- and higher-colour blocks (in blocks)
__global__ void k_sell_wmax(SellMap m, const int* __restrict__ lw, const int* __restrict__ uw, int* __restrict__ wm) {
	int const c = blockIdx.x;
	int l = 0, u = 0;
	for (int s = m.sbase[c] + threadIdx.x; s < m.sbase[c + 1]; s += blockDim.x) {
		l = max(l, lw[s]);
		u = max(u, uw[s]);
	}
	l = __reduce_max_sync(0xffffffffu, l);
	u = __reduce_max_sync(0xffffffffu, u);
	__shared__ int sl[32], su[32];
	if ((threadIdx.x & 31) == 0) {
		sl[threadIdx.x >> 5] = l;
		su[threadIdx.x >> 5] = u;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int w = 1; w < (int) (blockDim.x >> 5); w++) {
			l = max(l, sl[w]);
			u = max(u, su[w]);
		}
		wm[2 * c] = l / 32;
		wm[2 * c + 1] = u / 32;
	}
}

// copy each row's lower- and higher-colour blocks (ascending columns, as in
// the CSR rows) into its lane of the slice; pad with column -1
__global__ void k_sell_fill(int ns, SellMap m, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                            const float4* __restrict__ vals, const int* __restrict__ lp, const int* __restrict__ up,
                            float4* __restrict__ lv, int* __restrict__ lc, float4* __restrict__ uv, int* __restrict__ uc) {
	int const s = (int) ((blockIdx.x * (long) blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
	if (s >= ns) return;
	int c;
	int const row = sell_row_of(m, s, lane, c);
	int const el = lp[s] + lane, eu = up[s] + lane;
	int const wl = (lp[s + 1] - lp[s]) >> 5, wu = (up[s + 1] - up[s]) >> 5;
	int nl = 0, nu = 0;
	if (row >= 0)
		for (int k = row_ptr[row]; k < row_ptr[row + 1]; k++) {
			int const j = cols[k];
			if (j < m.off[c]) {
				lc[el + 32 * nl] = j;
				lv[el + 32 * nl] = vals[k];
				nl++;
			}
			else if (j >= m.off[c + 1]) {
				uc[eu + 32 * nu] = j;
				uv[eu + 32 * nu] = vals[k];
				nu++;
			}
		}
	for (; nl < wl; nl++) {
		lc[el + 32 * nl] = -1;
		lv[el + 32 * nl] = make_float4(0.f, 0.f, 0.f, 0.f);
	}
	for (; nu < wu; nu++) {
		uc[eu + 32 * nu] = -1;
		uv[eu + 32 * nu] = make_float4(0.f, 0.f, 0.f, 0.f);
	}
}

__global__ void k_diag_pos(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols, int* __restrict__ dpos) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	int k = row_ptr[i];
	int const e = row_ptr[i + 1];
	while (k < e && cols[k] < i) k++;
	dpos[i] = k;
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

// Dirichlet normal/tangent condition (system.c:388-425): for a flagged node,
// the half-sums over its boundary edges (one adjacent element) of the unit
// vector from the other end to the node, (tx, ty), in edge order; then both
// DOFs are constrained, to value * (tx, ty) (tangent) or value * (-ty, tx)
// (normal), with the same first/last bookkeeping as the X/Y conditions.
// The arithmetic is the reference's, correctly rounded.
__global__ void k_dirichlet_nt_mark(int N, int ci, int tangent, double value, const uint8_t* __restrict__ mask,
                                    const int* __restrict__ eptr, const int* __restrict__ elist, const int* __restrict__ edges,
                                    const uint8_t* __restrict__ eboundary, const double* __restrict__ coords,
                                    int* __restrict__ last_ci, double* __restrict__ first, double* __restrict__ last) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N || !mask[i]) return;
	double tx = 0.0, ty = 0.0;
	int prev = -1;
	int const k0 = eptr ? eptr[i] : 0, k1 = eptr ? eptr[i + 1] : 0;  // no edges: (tx, ty) = 0
	for (int k = k0; k < k1; k++) {
		int const e = elist[k];
		if (e == prev) continue;  // an edge from the node to itself is listed twice, counted once
		prev = e;
		if (!eboundary[e]) continue;
		int const n1 = edges[2 * e], n2 = edges[2 * e + 1];
		int const other = n1 == i ? n2 : n1;
		double const dx = xs(coords[2l * i], coords[2l * other]);
		double const dy = xs(coords[2l * i + 1], coords[2l * other + 1]);
		double const length = __dsqrt_rn(xa(xm(dx, dx), xm(dy, dy)));
		tx = xa(tx, xd(xd(dx, length), 2.0));
		ty = xa(ty, xd(xd(dy, length), 2.0));
	}
	double const v0 = xm(value, tangent ? tx : -ty), v1 = xm(value, tangent ? ty : tx);
	for (int c = 0; c < 2; c++) {
		int const d = 2 * i + c;
		double const v = c ? v1 : v0;
		if (last_ci[d] < 0) first[d] = v;
		last[d] = v;
		last_ci[d] = ci;
	}
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
	float* corr32;   // per node: the FP32 operator's 2x2 block row sum S (difference form)
	float* vals32lo; // double-float path: FP32 rounding of (FP64 value - FP32 value)
	float* srow_df;  // double-float path: per node the FP64 block row sum as a df pair (4 hi, 4 lo)
	double* b;
	const float4* coords32;  // FP32 integration: per node (x hi, y hi, x lo, y lo)
	int const_grad;          // FP32 integration: shape gradients equal at every Gauss point (P1)
	const float4* mat32;     // FP32 integration: per-element (a, b, c) material constants, or nullptr
	const double* egrad;     // exact P1 integration: per element dx[3], dy[3], det w, a, b, c (k_elem_grad), or nullptr
	int NE;
	double* dinv64;  // jacobi: 2 per node; block-jacobi: 4 per node
	float* dinv32;
	int precond;
	int skip_upto;  // rows of at most this many blocks are another kernel's
	int* err;
};

__device__ __forceinline__ void store_precond(const AsmArgs& a, int r, double k00, double k01, double k10, double k11) {
	if (a.precond != BFM_GPU_PC_JACOBI) {  // block Jacobi; also the starting blocks of the learned one
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


// s + x as an unevaluated float pair (TwoSum, no ordering assumption)
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
	float const t = __fadd_rn(hi, x);
	float const z = __fsub_rn(t, hi);
	float const err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(x, z));
	hi = t;
	lo = __fadd_rn(lo, err);
}

__global__ void k_split_coords(int N, const double* __restrict__ coords, float4* __restrict__ out) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double2 const c = reinterpret_cast<const double2*>(coords)[i];
	float const xh = (float) c.x, yh = (float) c.y;
	out[i] = make_float4(xh, yh, (float) (c.x - (double) xh), (float) (c.y - (double) yh));
}

// Exact FP64 integration of P1 elements under a rule whose shape gradients
// and weights are the same at every point: the Jacobian, the shape gradients
// and det w then come out the same at every point (the same operations on
// the same values), so they are formed once per element here -- in the
// operation order of k_assemble<true> below, at point 0 -- instead of once per
// owner row and point (three rows, three points).  Per element, 10 doubles:
// dx[3], dy[3], det w, and the material constants a, b, c.
__global__ void k_elem_grad(AsmArgs a, double* __restrict__ eg) {
	int const e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= a.NE) return;
	double x[3], y[3];
	for (int j = 0; j < 3; j++) {
		int const m = a.elems[3l * e + j];
		x[j] = a.coords[2l * m];
		y[j] = a.coords[2l * m + 1];
	}
	double dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0;
	for (int j = 0; j < 3; j++) {
		dx_dxsi = xa(dx_dxsi, xm(x[j], a.rule.dxi[0][j]));
		dx_deta = xa(dx_deta, xm(x[j], a.rule.deta[0][j]));
		dy_dxsi = xa(dy_dxsi, xm(y[j], a.rule.dxi[0][j]));
		dy_deta = xa(dy_deta, xm(y[j], a.rule.deta[0][j]));
	}
	double const det = fabs(xs(xm(dx_dxsi, dy_deta), xm(dx_deta, dy_dxsi)));
	double* o = eg + 10l * e;
	for (int j = 0; j < 3; j++) {
		o[j] = xd(xs(xm(a.rule.dxi[0][j], dy_deta), xm(a.rule.deta[0][j], dy_dxsi)), det);
		o[3 + j] = xd(xs(xm(a.rule.deta[0][j], dx_dxsi), xm(a.rule.dxi[0][j], dx_deta)), det);
	}
	o[6] = xm(det, a.rule.w[0]);
	double ea, eb, ec;
	material_abc(a.elemE ? a.elemE[e] : a.E, a.elemNu ? a.elemNu[e] : a.nu, a.stress, ea, eb, ec);
	o[7] = ea;
	o[8] = eb;
	o[9] = ec;
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
	if (len <= a.skip_upto) return;

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
			if (a.egrad) {
				// P1 with point-independent gradients (k_elem_grad): this row's
				// contributions formed once, then added once per point in the
				// order of the loop below, so the sums are the same bit for bit
				const double* g = a.egrad + 10l * e;
				double const dw = g[6];
				ea = g[7];
				eb = g[8];
				ec = g[9];
				for (int q = 0; q < a.rule.nq; q++) {
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
				}
				double const xj = g[jr], yj = g[3 + jr];
				double c[3][4];
				for (int k = 0; k < 3; k++) {
					double const dk = g[k], ek = g[3 + k];
					c[k][0] = xm(dw, xa(xm(xm(ea, xj), dk), xm(xm(ec, yj), ek)));
					c[k][1] = xm(dw, xa(xm(xm(eb, xj), ek), xm(xm(ec, yj), dk)));
					c[k][2] = xm(dw, xa(xm(xm(eb, yj), dk), xm(xm(ec, xj), ek)));
					c[k][3] = xm(dw, xa(xm(xm(ea, yj), ek), xm(xm(ec, xj), dk)));
				}
				for (int q = 0; q < a.rule.nq; q++)
					for (int k = 0; k < 3; k++) {
						int const s = slot[k];
						acc[s][0] = xa(acc[s][0], c[k][0]);
						acc[s][1] = xa(acc[s][1], c[k][1]);
						acc[s][2] = xa(acc[s][2], c[k][2]);
						acc[s][3] = xa(acc[s][3], c[k][3]);
					}
				continue;
			}
			bool const axi = a.stress >= 2;
			for (int q = 0; q < a.rule.nq; q++) {
				double const w = a.rule.w[q];
				double dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0, rad = 0;
				for (int j = 0; j < kind; j++) {
					dx_dxsi = xa(dx_dxsi, xm(x[j], a.rule.dxi[q][j]));
					dx_deta = xa(dx_deta, xm(x[j], a.rule.deta[q][j]));
					dy_dxsi = xa(dy_dxsi, xm(y[j], a.rule.dxi[q][j]));
					dy_deta = xa(dy_deta, xm(y[j], a.rule.deta[q][j]));
					rad = xa(rad, xm(x[j], a.rule.phi[q][j]));
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
					double bx = xm(xm(xm(dw, fx), a.rho), ph), by = xm(xm(xm(dw, fy), a.rho), ph);
					if (axi) {  // system.c:321-322: weighted by the radius of the Gauss point
						bx = xm(bx, rad);
						by = xm(by, rad);
					}
					b0 = xa(b0, bx);
					b1 = xa(b1, by);
				}
				double const xj = dx[jr], yj = dy[jr];
				if (axi) {
					// axisymmetric terms, system.c:334-337, the reference's
					// operation order; (r, z) = (x, y) and the hoop strain u/r.
					// The reference leaves the radius off the c dphi_dx dphi_dx
					// term of f_22; stress 2 puts it back, stress 3 keeps it off.
					double const pj = ph;
					for (int k = 0; k < kind; k++) {
						double const pk = a.rule.phi[q][k];
						double const f11 = xa(xa(xa(xm(xm(xm(ea, xj), dx[k]), rad), xm(xm(xm(ec, yj), dy[k]), rad)),
						                         xm(pj, xa(xm(eb, dx[k]), xd(xm(ea, pk), rad)))),
						                      xm(xm(xj, eb), pk));
						double const f12 = xa(xa(xm(xm(xm(eb, xj), dy[k]), rad), xm(xm(xm(ec, yj), dx[k]), rad)),
						                      xm(xm(pj, eb), dy[k]));
						double const f21 = xa(xa(xm(xm(xm(eb, yj), dx[k]), rad), xm(xm(xm(ec, xj), dy[k]), rad)),
						                      xm(xm(yj, eb), pk));
						double const cxx = xm(xm(ec, xj), dx[k]);
						double const f22 = xa(xm(xm(xm(ea, yj), dy[k]), rad), a.stress == 2 ? xm(cxx, rad) : cxx);
						int const s = slot[k];
						acc[s][0] = xa(acc[s][0], xm(dw, f11));
						acc[s][1] = xa(acc[s][1], xm(dw, f12));
						acc[s][2] = xa(acc[s][2], xm(dw, f21));
						acc[s][3] = xa(acc[s][3], xm(dw, f22));
					}
					continue;
				}
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
			// (the same offsets and FP32 materials as k_assemble32, so rows
			// shared with it stay exactly symmetric)
			float lx[4], ly[4];
			float4 const c0 = a.coords32[map[0]];
			for (int j = 0; j < kind; j++) {
				float4 const cj = a.coords32[map[j]];
				lx[j] = __fadd_rn(__fsub_rn(cj.x, c0.x), __fsub_rn(cj.z, c0.z));
				ly[j] = __fadd_rn(__fsub_rn(cj.y, c0.y), __fsub_rn(cj.w, c0.w));
			}
			float fa, fb, fc;
			if (a.mat32) {
				float4 const m = a.mat32[e];
				fa = m.x;
				fb = m.y;
				fc = m.z;
			}
			else {
				fa = (float) ea;
				fb = (float) eb;
				fc = (float) ec;
			}
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
					float const pxx = xj * dx[k], pyy = yj * dy[k], pxy = xj * dy[k], pyx = yj * dx[k];
					acc[s][0] += dw * (fa * pxx + fc * pyy);
					acc[s][1] += dw * (fb * pxy + fc * pyx);
					acc[s][2] += dw * (fb * pyx + fc * pxy);
					acc[s][3] += dw * (fa * pyy + fc * pxx);
				}
			}
		}
	}

	// FP32 integration: rebuild the diagonal block from the off-diagonal ones
	// (FP64 sum), so every block row sums to zero as it does exactly: FP32
	// rounding must not break the translation modes, or the FP32 operator
	// stops being positive definite on ill-conditioned meshes.
	int sd = -1;
	for (int s = 0; s < len; s++)
		if (col[s] == r) sd = s;
	double dfix[4] = {0, 0, 0, 0};
	if constexpr (!EXACT) {
		if (sd >= 0 && is < ie) {
			for (int s = 0; s < len; s++)
				if (s != sd)
					for (int k = 0; k < 4; k++) dfix[k] -= (double) acc[s][k];
			for (int k = 0; k < 4; k++) acc[sd][k] = (T) dfix[k];
		}
	}
	// symmetric Dirichlet elimination of this row
	int const r0 = 2 * r, r1 = 2 * r + 1;
	bool const c0 = a.last_ci[r0] >= 0, c1 = a.last_ci[r1] >= 0;
	double k00 = 0, k01 = 0, k10 = 0, k11 = 0;
	double rsum[4] = {0, 0, 0, 0};  // FP64 block row sum: the FP32 operator's S block (difference form)
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
		double v[4] = {(double) acc[s][0], (double) acc[s][1], (double) acc[s][2], (double) acc[s][3]};
		if (s == sd && !EXACT) {
			v[0] = dfix[0]; v[1] = dfix[1]; v[2] = dfix[2]; v[3] = dfix[3];
		}
		if (c0 || e0) v[0] = (r0 == d0) ? 1.0 : 0.0;
		if (c0 || e1) v[1] = 0.0;
		if (c1 || e0) v[2] = 0.0;
		if (c1 || e1) v[3] = (r1 == d1) ? 1.0 : 0.0;
		long const o = 4l * (rs + s);
		if (a.vals64) {
			a.vals64[o + 0] = v[0]; a.vals64[o + 1] = v[1];
			a.vals64[o + 2] = v[2]; a.vals64[o + 3] = v[3];
		}
		if (a.vals32) {
			// FP32 path: one value for both off-diagonal entries of the diagonal block (symmetric)
			float const sym = (float) (0.5 * (v[1] + v[2]));
			for (int k = 0; k < 4; k++) {
				float const f = (!EXACT && s == sd && (k == 1 || k == 2)) ? sym : (float) v[k];
				a.vals32[o + k] = f;
				rsum[k] += v[k];
				if (a.vals32lo) a.vals32lo[o + k] = (float) (v[k] - (double) f);
			}
		}
		if (c == r) {
			k00 = v[0]; k01 = v[1];
			k10 = v[2]; k11 = v[3];
		}
	}
	if (a.corr32 && !a.vals32lo) {
		a.corr32[4 * r + 0] = (float) rsum[0]; a.corr32[4 * r + 1] = (float) rsum[1];
		a.corr32[4 * r + 2] = (float) rsum[2]; a.corr32[4 * r + 3] = (float) rsum[3];
	}
	if (a.srow_df) {
		// the double-float SpMV's row-sum block, from the FP64 values
		float h[4], l[4];
		for (int k = 0; k < 4; k++) {
			h[k] = (float) rsum[k];
			l[k] = (float) (rsum[k] - (double) h[k]);
		}
		reinterpret_cast<float4*>(a.srow_df)[2 * r] = make_float4(h[0], h[1], h[2], h[3]);
		reinterpret_cast<float4*>(a.srow_df)[2 * r + 1] = make_float4(l[0], l[1], l[2], l[3]);
	}
	if (c0) b0 = a.last[r0];
	if (c1) b1 = a.last[r1];
	a.b[r0] = b0;
	a.b[r1] = b1;
	store_precond(a, r, k00, k01, k10, k11);
}

// Material constants (a, b, c) of every element for the FP32 integration,
// once per element rather than once per owner row (three or four times):
// computed in FP64 and rounded once, so they are the FP64 constants to FP32
// precision
// 1/x in FP64 from an FP32 estimate and two Newton steps (FMA form), for x
// in FP32 range: a few FP64 operations where a correctly rounded division
// takes many more on this GPU's FP64 pipe; within an ulp or two of 1/x
__device__ __forceinline__ double recip_nr(double x) {
	double r = (double) __frcp_rn((float) x);
	r = __fma_rn(r, __fma_rn(-x, r, 1.0), r);
	return __fma_rn(r, __fma_rn(-x, r, 1.0), r);
}

// material_abc's formulas with reciprocals in place of its correctly rounded
// divisions: the FP64 result is within a few ulps, so its rounding to FP32
// is the same but for values within a few FP64 ulps of an FP32 tie
__device__ __forceinline__ void material_abc_fast(double E, double nu, int stress, double& a, double& b, double& c) {
	double const r1 = recip_nr(1.0 + nu);
	if (stress != 1) {
		double const den = 1.0 - 2.0 * nu;
		double const ef = E * (1.0 - nu) * r1;
		a = stress == 3 ? ef * den : ef * recip_nr(den);
		b = E * nu * r1 * recip_nr(den);
	}
	else {
		double const rd = recip_nr(1.0 - nu * nu);
		a = E * rd;
		b = E * nu * rd;
	}
	c = E * 0.5 * r1;
}

__global__ void k_elem_mat32(int NE, const double* __restrict__ elemE, const double* __restrict__ elemNu, double E,
                             double nu, int stress, float4* __restrict__ mat) {
	int const e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= NE) return;
	double da, db, dc;
	material_abc_fast(elemE ? elemE[e] : E, elemNu ? elemNu[e] : nu, stress, da, db, dc);
	mat[e] = make_float4((float) da, (float) db, (float) dc, 0.f);
}


// FP32 element integration, fast form (BFM_GPU_MIXED): one thread per node
// row as above (owner computes, no atomics), with the per-element and per-row
// work on the FP32 pipe (GB300 issues FP64 at a small fraction of its FP32
// rate):
//  - node offsets within an element from a hi/lo float split of the FP64
//    coordinates (the hi difference of nearby nodes is exact, the lo
//    difference restores what the split dropped);
//  - material constants from the per-element table above; the Gauss rule
//    from shared memory; for rules whose shape gradients are the same at
//    every point (P1) one evaluation with the summed weights;
//  - the row's blocks accumulated in shared memory (slot found once per
//    element node), each element's contribution summed over the integration
//    points before it is added;
//  - gradient products formed first, so the owner of the transposed block
//    forms the same products and the FP32 operator is exactly symmetric;
//  - the diagonal block rebuilt as a double-float sum of the off-diagonal
//    blocks (exact zero row sums: the translation modes), and the row-sum
//    block S of the difference form that the solver applies,
//    (K g)_r = S_r g_r + sum_c K_rc (g_c - g_r), as a double-float sum of
//    the stored row (zero for an interior node);
//  - the block's output rows staged in shared memory and written with
//    coalesced 16-byte stores.
// Rows longer than RMAX are left to k_assemble<false>.
template <int RMAX>
__global__ void __launch_bounds__(128, 6) k_assemble32(AsmArgs a) {
	constexpr int BT = 128;
	// the rows' block accumulators, [slot * 4 + entry][thread]; once every thread
	// has read its column back (before the epilogue's barrier) the same memory
	// stages the block's output rows
	__shared__ __align__(16) float smem_rows[RMAX * 4 * BT];
	float (*const sacc)[BT] = reinterpret_cast<float (*)[BT]>(smem_rows);
	float4* const stage = reinterpret_cast<float4*>(smem_rows);
	__shared__ float sw[MAXQ], sphi[MAXQ][4], sdxi[MAXQ][4], sdeta[MAXQ][4], swphi[4], swsum;
	__shared__ int first_rs, long_rows;
	int const tid = threadIdx.x;
	int const r = blockIdx.x * BT + tid;
	bool const valid = r < a.N;
	int const rs = valid ? a.row_ptr[r] : 0;
	int const len = valid ? a.row_ptr[r + 1] - rs : 0;
	if (tid == 0) {
		first_rs = a.row_ptr[blockIdx.x * BT];
		long_rows = 0;
	}
	for (int k = tid; k < MAXQ * 4; k += BT) {
		int const q = k >> 2, j = k & 3;
		sphi[q][j] = (float) a.rule.phi[q][j];
		sdxi[q][j] = (float) a.rule.dxi[q][j];
		sdeta[q][j] = (float) a.rule.deta[q][j];
	}
	if (tid < MAXQ) sw[tid] = (float) a.rule.w[tid];
	if (tid < 4) {
		// constant-gradient rules (P1): one evaluation with the summed weights
		double wp = 0.0;
		for (int q = 0; q < a.rule.nq; q++) wp += a.rule.w[q] * a.rule.phi[q][tid];
		swphi[tid] = (float) wp;
	}
	if (tid == 0) {
		double ws = 0.0;
		for (int q = 0; q < a.rule.nq; q++) ws += a.rule.w[q];
		swsum = (float) ws;
	}
#pragma unroll
	for (int t = 0; t < RMAX * 4; t++) sacc[t][tid] = 0.f;
	__syncthreads();
	if (len > RMAX) atomicOr(&long_rows, 1);
	bool const mine = valid && len <= RMAX;

	int col[RMAX];
#pragma unroll
	for (int t = 0; t < RMAX; t++) col[t] = (mine && t < len) ? a.cols[rs + t] : -1;
	int const kind = a.kind;
	int const nq = a.const_grad ? 1 : a.rule.nq;
	bool const per_elem = a.elemE || a.elemNu;
	float ca = 0.f, cb = 0.f, cc = 0.f;
	if (!per_elem) {
		double da, db, dc;
		material_abc(a.E, a.nu, a.stress, da, db, dc);
		ca = (float) da;
		cb = (float) db;
		cc = (float) dc;
	}
	// body forces at this node (the reference evaluates them at the node), times rho
	float gfx = 0.f, gfy = 0.f;
	if (mine)
		for (int f = 0; f < a.forces.nf; f++) {
			double fx = a.forces.f[f][0], fy = a.forces.f[f][1];
			if (a.forces.field[f]) {
				fx = a.forces.field[f][2l * r];
				fy = a.forces.field[f][2l * r + 1];
			}
			gfx += (float) fx * (float) a.rho;
			gfy += (float) fy * (float) a.rho;
		}
	float bf0 = 0.f, bf1 = 0.f;
	int const is = mine ? a.inc_ptr[r] : 0, ie = mine ? a.inc_ptr[r + 1] : 0;
	int prev_e = -1;
	for (int t = is; t < ie; t++) {
		int const e = a.inc[t];
		if (e == prev_e) continue;
		prev_e = e;
		int slot[4];
		float lx[4], ly[4];
		int jr = 0;
		float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
		for (int j = 0; j < 4; j++) {
			lx[j] = ly[j] = 0.f;
			slot[j] = -1;
			if (j < kind) {
				int const m = a.elems[(long) e * kind + j];
				float4 const cj = a.coords32[m];
				if (j == 0) c0 = cj;
				lx[j] = __fadd_rn(__fsub_rn(cj.x, c0.x), __fsub_rn(cj.z, c0.z));
				ly[j] = __fadd_rn(__fsub_rn(cj.y, c0.y), __fsub_rn(cj.w, c0.w));
				if (m == r) jr = j;
				int s = 0;
#pragma unroll
				for (int u = 1; u < RMAX; u++) s = col[u] == m ? u : s;
				slot[j] = s;
			}
		}
		float fa = ca, fb = cb, fc = cc;
		if (per_elem) {
			float4 const m = a.mat32[e];
			fa = m.x;
			fb = m.y;
			fc = m.z;
		}
		float ek[4][4];
#pragma unroll
		for (int k = 0; k < 4; k++) ek[k][0] = ek[k][1] = ek[k][2] = ek[k][3] = 0.f;
		for (int q = 0; q < nq; q++) {
			float dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0;
			float gx[4], ge[4];
#pragma unroll
			for (int j = 0; j < 4; j++) {
				gx[j] = sdxi[q][j];
				ge[j] = sdeta[q][j];
				dx_dxsi += lx[j] * gx[j];
				dx_deta += lx[j] * ge[j];
				dy_dxsi += ly[j] * gx[j];
				dy_deta += ly[j] * ge[j];
			}
			float const det = fabsf(dx_dxsi * dy_deta - dx_deta * dy_dxsi);
			float const idet = 1.0f / det;
			float dx[4], dy[4];
#pragma unroll
			for (int j = 0; j < 4; j++) {
				dx[j] = (gx[j] * dy_deta - ge[j] * dy_dxsi) * idet;
				dy[j] = (ge[j] * dx_dxsi - gx[j] * dx_deta) * idet;
			}
			float const dw = det * (a.const_grad ? swsum : sw[q]);
			float const dwp = det * (a.const_grad ? swphi[jr] : sw[q] * sphi[q][jr]);
			bf0 += dwp * gfx;
			bf1 += dwp * gfy;
			float xj = dx[0], yj = dy[0];
#pragma unroll
			for (int j = 1; j < 4; j++)
				if (j == jr) {
					xj = dx[j];
					yj = dy[j];
				}
			// gradient products first: the owner of the transposed block forms
			// the same products (multiplication commutes exactly), so the FP32
			// operator is exactly symmetric
#pragma unroll
			for (int k = 0; k < 4; k++) {
				float const pxx = xj * dx[k], pyy = yj * dy[k], pxy = xj * dy[k], pyx = yj * dx[k];
				ek[k][0] += dw * (fa * pxx + fc * pyy);
				ek[k][1] += dw * (fb * pxy + fc * pyx);
				ek[k][2] += dw * (fb * pyx + fc * pxy);
				ek[k][3] += dw * (fa * pyy + fc * pxx);
			}
		}
#pragma unroll
		for (int k = 0; k < 4; k++) {
			if (k >= kind || slot[k] < 0) continue;
			int const s4 = 4 * slot[k];
			sacc[s4 + 0][tid] += ek[k][0];
			sacc[s4 + 1][tid] += ek[k][1];
			sacc[s4 + 2][tid] += ek[k][2];
			sacc[s4 + 3][tid] += ek[k][3];
		}
	}
	float acc[RMAX][4];
#pragma unroll
	for (int t = 0; t < RMAX; t++)
#pragma unroll
		for (int k = 0; k < 4; k++) acc[t][k] = sacc[4 * t + k][tid];
	// translation-preserving diagonal: minus the double-float sum of the off-diagonal blocks
	float dh[4] = {0.f, 0.f, 0.f, 0.f}, dl[4] = {0.f, 0.f, 0.f, 0.f};
	bool has_diag = false;
#pragma unroll
	for (int t = 0; t < RMAX; t++) {
		if (col[t] == r) has_diag = true;
		else if (col[t] >= 0)
#pragma unroll
			for (int k = 0; k < 4; k++) two_sum_acc(dh[k], dl[k], -acc[t][k]);
	}
#pragma unroll
	for (int k = 0; k < 4; k++) {
		float const h = __fadd_rn(dh[k], dl[k]);
		dl[k] = __fsub_rn(dl[k], __fsub_rn(h, dh[k]));
		dh[k] = h;
	}
	{
		// one FP32 value for both off-diagonal entries of the diagonal block
		// (a symmetric stored matrix); each entry keeps its remainder in the
		// row-sum block
		float const m = __fmul_rn(0.5f, __fadd_rn(dh[1], dh[2]));
		dl[1] = __fadd_rn(__fsub_rn(dh[1], m), dl[1]);
		dl[2] = __fadd_rn(__fsub_rn(dh[2], m), dl[2]);
		dh[1] = dh[2] = m;
	}
	bool const fix = has_diag && is < ie;
	int const r0 = 2 * r, r1 = 2 * r + 1;
	bool const c0 = mine && a.last_ci[r0] >= 0, c1 = mine && a.last_ci[r1] >= 0;
	float k00 = 0.f, k01 = 0.f, k10 = 0.f, k11 = 0.f;
	// S block of the difference form: double-float row sum of what is stored
	// plus the diagonal's low parts (zero for an interior node)
	float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
	double b0 = bf0, b1 = bf1;
	__syncthreads();
	bool const staged = long_rows == 0;
#pragma unroll
	for (int t = 0; t < RMAX; t++) {
		int const c = col[t];
		if (c < 0) continue;
		int const d0 = 2 * c, d1 = 2 * c + 1;
		bool const e0 = a.last_ci[d0] >= 0, e1 = a.last_ci[d1] >= 0;
		bool const dg = c == r && fix;
		float v[4] = {acc[t][0], acc[t][1], acc[t][2], acc[t][3]};
		float lo[4] = {0.f, 0.f, 0.f, 0.f};
		if (dg) {
#pragma unroll
			for (int k = 0; k < 4; k++) {
				v[k] = dh[k];
				lo[k] = dl[k];
			}
		}
		if (e0 || e1) {
			// non-homogeneous Dirichlet values leave the row through b (rare rows)
			double const f0 = e0 ? a.first[d0] : 0.0, f1 = e1 ? a.first[d1] : 0.0;
			if (!c0) {
				if (e0) b0 -= f0 * ((double) v[0] + lo[0]);
				if (e1) b0 -= f1 * ((double) v[1] + lo[1]);
			}
			if (!c1) {
				if (e0) b1 -= f0 * ((double) v[2] + lo[2]);
				if (e1) b1 -= f1 * ((double) v[3] + lo[3]);
			}
		}
		if (c0 || e0) { v[0] = (r0 == d0) ? 1.f : 0.f; lo[0] = 0.f; }
		if (c0 || e1) { v[1] = 0.f; lo[1] = 0.f; }
		if (c1 || e0) { v[2] = 0.f; lo[2] = 0.f; }
		if (c1 || e1) { v[3] = (r1 == d1) ? 1.f : 0.f; lo[3] = 0.f; }
#pragma unroll
		for (int k = 0; k < 4; k++) {
			two_sum_acc(sh[k], sl[k], v[k]);
			sl[k] = __fadd_rn(sl[k], lo[k]);
		}
		float4 const f4 = make_float4(v[0], v[1], v[2], v[3]);
		if (staged) stage[rs - first_rs + t] = f4;
		else reinterpret_cast<float4*>(a.vals32)[rs + t] = f4;
		if (c == r) {
			k00 = v[0]; k01 = v[1];
			k10 = v[2]; k11 = v[3];
		}
	}
	if (mine) {
		reinterpret_cast<float4*>(a.corr32)[r] =
			make_float4(__fadd_rn(sh[0], sl[0]), __fadd_rn(sh[1], sl[1]), __fadd_rn(sh[2], sl[2]), __fadd_rn(sh[3], sl[3]));
		if (c0) b0 = a.last[r0];
		if (c1) b1 = a.last[r1];
		reinterpret_cast<double2*>(a.b)[r] = make_double2(b0, b1);
		if (a.precond != BFM_GPU_PC_JACOBI) {
			float const det = k00 * k11 - k01 * k10;
			float const id = det != 0.f ? 1.f / det : 0.f;
			reinterpret_cast<float4*>(a.dinv32)[r] = make_float4(k11 * id, -k01 * id, -k10 * id, k00 * id);
		}
		else {
			reinterpret_cast<float2*>(a.dinv32)[r] = make_float2(k00 != 0.f ? 1.f / k00 : 0.f, k11 != 0.f ? 1.f / k11 : 0.f);
		}
	}
	__syncthreads();
	if (staged) {
		int const last_row = min(a.N, (int) (blockIdx.x + 1) * (int) blockDim.x);
		int const end = a.row_ptr[last_row];
		float4* const out = reinterpret_cast<float4*>(a.vals32);
		for (int k = first_rs + threadIdx.x; k < end; k += blockDim.x) out[k] = stage[k - first_rs];
	}
}

// Neumann X/Y loads (system.c:477-498), gathered per node in condition order
// then edge order (deterministic, no atomics).  A load on a constrained DOF
// survives only when applied after that DOF's last Dirichlet condition.
struct NeuArgs {
	int N, n_conds, stress;
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
		const uint8_t* m = a.masks + (long) ci * a.N;
		if (kd == BFM_CONDITION_KIND_NEUMANN_NORMAL || kd == BFM_CONDITION_KIND_NEUMANN_TANGENT) {
			if (a.stress >= 2) continue;  // the axisymmetric system (system.c:573-616) has no such loads
			// system.c:500-522: each end of a flagged edge gets
			// 0.5 value (dx, dy) (tangent) or 0.5 value (-dy, dx) (normal),
			// (dx, dy) = first end - second end (the length cancels)
			if (!m[r]) continue;
			bool const tangent = kd == BFM_CONDITION_KIND_NEUMANN_TANGENT;
			bool const on0 = a.last_ci[2 * r] <= ci, on1 = a.last_ci[2 * r + 1] <= ci;
			for (int k = s; k < t; k++) {
				int const ed = a.elist[k];
				int const n1 = a.edges[2 * ed], n2 = a.edges[2 * ed + 1];
				if (!m[n1] || !m[n2]) continue;
				double const dx = xs(a.coords[2l * n1], a.coords[2l * n2]);
				double const dy = xs(a.coords[2l * n1 + 1], a.coords[2l * n2 + 1]);
				double const hv = xm(0.5, a.values[ci]);
				if (on0) add0 = xa(add0, xm(hv, tangent ? dx : -dy));
				if (on1) add1 = xa(add1, xm(hv, tangent ? dy : dx));
			}
			continue;
		}
		if (kd != BFM_CONDITION_KIND_NEUMANN_X && kd != BFM_CONDITION_KIND_NEUMANN_Y) continue;
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
			double load = jac * a.values[ci];
			if (a.stress == 3) {
				// system.c:591-601: both ends get (r1 + r2) jac value, r1 and
				// r2 as written there (from the x and y of one node each)
				double const g0 = (1.0 - 1.0 / sqrt(3.0)) / 2, g1 = (1.0 + 1.0 / sqrt(3.0)) / 2;
				double const r1 = a.coords[2l * n1] * g0 + a.coords[2l * n1 + 1] * g1;
				double const r2 = a.coords[2l * n2] * g0 + a.coords[2l * n2 + 1] * g1;
				load = (r1 + r2) * jac * a.values[ci];
			}
			else if (a.stress == 2) {
				// consistent load: value jac times the integral over [-1, 1] of
				// (this end's shape function) x (radius) = (2 r_this + r_other) / 3
				double const rt = a.coords[2l * (n1 == r ? n1 : n2)], ro = a.coords[2l * (n1 == r ? n2 : n1)];
				load = (2.0 * rt + ro) / 3.0 * jac * a.values[ci];
			}
			// an edge whose two ends are the same node adds twice, as in the reference
			int const mult = (n1 == r) + (n2 == r);
			for (int u = 0; u < mult; u++) {
				if (shift == 0) add0 += load;
				else add1 += load;
			}
		}
	}
	a.b[2 * r] += add0;
	a.b[2 * r + 1] += add1;
}

// Per-edge tractions (fx, fy per unit length): each end of an edge receives
// (length/2) * load, as the reference's Neumann X/Y loop does for a flagged
// edge (system.c:477-498).  Gathered per node over its edges in ascending
// order (deterministic); constrained DOFs keep their Dirichlet value, as if
// the loads were listed before the Dirichlet conditions.
__global__ void k_edge_loads(int N, const int* __restrict__ ledges, const double* __restrict__ lloads,
                             const int* __restrict__ lptr, const int* __restrict__ llist, const double* __restrict__ coords,
                             const int* __restrict__ last_ci, double* __restrict__ b) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= N) return;
	double add0 = 0.0, add1 = 0.0;
	for (int k = lptr[r]; k < lptr[r + 1]; k++) {
		int const e = llist[k];
		int const n1 = ledges[2 * e], n2 = ledges[2 * e + 1];
		double const dx = coords[2l * n1] - coords[2l * n2];
		double const dy = coords[2l * n1 + 1] - coords[2l * n2 + 1];
		double const jac = sqrt(dx * dx + dy * dy) / 2;
		int const mult = (n1 == r) + (n2 == r);
		for (int u = 0; u < mult; u++) {
			add0 += jac * lloads[2 * e];
			add1 += jac * lloads[2 * e + 1];
		}
	}
	if (last_ci[2 * r] < 0) b[2 * r] += add0;
	if (last_ci[2 * r + 1] < 0) b[2 * r + 1] += add1;
}

// Per-node 2x2 preconditioner blocks into the layout of the iteration:
// 0 FP64 (4 doubles), 1 FP32 (4 floats), 2 double-float (4 hi, then 4 lo).
// blocks == nullptr: Jacobi blocks from the diagonal of the operator.
__global__ void k_store_blocks(int N, const double* __restrict__ blocks, const int* __restrict__ row_ptr,
                               const int* __restrict__ cols, const double* __restrict__ v64, const float* __restrict__ v32,
                               int layout, int block, double* __restrict__ dinv64, float* __restrict__ dinv32) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double m[4];
	if (blocks) {
		for (int k = 0; k < 4; k++) m[k] = blocks[4l * i + k];
	}
	else {
		double k00 = 0.0, k01 = 0.0, k10 = 0.0, k11 = 0.0;
		for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++)
			if (cols[k] == i) {
				k00 = v64 ? v64[4l * k] : (double) v32[4l * k];
				k01 = v64 ? v64[4l * k + 1] : (double) v32[4l * k + 1];
				k10 = v64 ? v64[4l * k + 2] : (double) v32[4l * k + 2];
				k11 = v64 ? v64[4l * k + 3] : (double) v32[4l * k + 3];
			}
		if (block) {
			double const det = k00 * k11 - k01 * k10;
			double const id = det != 0.0 ? 1.0 / det : 0.0;
			m[0] = k11 * id;
			m[1] = -k01 * id;
			m[2] = -k10 * id;
			m[3] = k00 * id;
		}
		else {
			m[0] = k00 != 0.0 ? 1.0 / k00 : 0.0;
			m[1] = m[2] = 0.0;
			m[3] = k11 != 0.0 ? 1.0 / k11 : 0.0;
		}
	}
	if (layout == 0) {
		for (int k = 0; k < 4; k++) dinv64[4l * i + k] = m[k];
	}
	else if (layout == 1) {
		for (int k = 0; k < 4; k++) dinv32[4l * i + k] = (float) m[k];
	}
	else {
		float h[4], l[4];
		for (int k = 0; k < 4; k++) {
			h[k] = (float) m[k];
			l[k] = (float) (m[k] - (double) h[k]);
			dinv64[4l * i + k] = m[k];  // the FP64 tail of the double-float solve
		}
		reinterpret_cast<float4*>(dinv32)[2l * i] = make_float4(h[0], h[1], h[2], h[3]);
		reinterpret_cast<float4*>(dinv32)[2l * i + 1] = make_float4(l[0], l[1], l[2], l[3]);
	}
}

// y = K x with the FP64 operator (one thread per block row)
__global__ void k_apply64(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols, const double* __restrict__ vals,
                          const double* __restrict__ x, double* __restrict__ y) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double y0 = 0.0, y1 = 0.0;
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
		int const c = cols[k];
		double const x0 = x[2l * c], x1 = x[2l * c + 1];
		y0 += vals[4l * k] * x0 + vals[4l * k + 1] * x1;
		y1 += vals[4l * k + 2] * x0 + vals[4l * k + 3] * x1;
	}
	y[2l * i] = y0;
	y[2l * i + 1] = y1;
}

}  // namespace

#include "cg_kernels.cuh"
#include "ssor_tma.cuh"

namespace {

int g_num_sms = 0;

// A learned solve that stagnates above this relative residual is redone with Jacobi
constexpr double LEARNED_FALLBACK_REL = 1e-6;

// The double-float path iterates to DF_SWITCH x rtol, then finishes in FP64
constexpr double DF_SWITCH = 100.0;

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
	uint8_t* eboundary;  // per edge: 1 if it has one adjacent element (normal/tangent Dirichlet)

	// pattern
	int *cnt, *inc_ptr, *inc, *cand, *row_len, *row_ptr, *cols;
	int *ecnt, *eptr, *elist;
	int* scan_sums;
	int* scan_total;
	long nb_cap;

	// system
	double* vals64;
	float* vals32;
	float* corr32;  // mixed: per-node 2x2 block row sum S of the FP32 operator (difference form)
	float* vals32lo;  // double-float path: low parts of the block values
	float* srow_df;   // double-float path: block row sums (difference-form SpMV)
	float4* coords32; // FP32 integration: hi/lo float split of the coordinates
	float4* mat32;    // FP32 integration: per-element material constants
	double* egrad;    // exact P1 integration: per-element gradients, det w and materials
	int egrad_cap;
	double* b;
	int* last_ci;
	double *first, *last;
	double* dinv64;
	float* dinv32;
	int precision, precond;

	// CG
	double* x;
	void* vec[6];  // r, u, p, s, w (FP64 path), + x (double-float path); r, dx, p, pn, q (mixed path)
	int lpr;       // lanes per block row of the SpMV kernels (autotuned)
	double* partials;
	unsigned* ticket;
	CgState* st;
	CgState* st_host;  // pinned
	int* err;
	int* err_host;     // pinned

	cudaGraphExec_t graph;
	int graph_precision, graph_precond, graph_lpr;
	int tuned;
	bfm_gpu_opts_t graph_opts;

	cudaEvent_t ev[4];
	bool assembled, solved;
	int fallback;  // the last learned solve was taken over by Jacobi

	// per-edge tractions (extension of the Neumann conditions)
	int n_loads, cap_loads;
	int* ledges;
	double* lloads;
	int *lcnt, *lptr, *llist;

	unsigned inputs_gen;     // bumped by every bfm_gpu_problem_set_* (captured assemblies bake some inputs in)
	void* ext;               // batch solver state (batch.cu)
	void (*ext_free)(void*);

	// multicolour node order of the SSOR preconditioners: the problem is
	// assembled and solved with its nodes renumbered colour by colour.
	// iperm: caller's node -> working node, perm: its inverse.  `ordered`
	// holds an ORD_* bit for every input array kept in the working order.
	unsigned ordered;
	bool colored;  // perm is the colouring of the current geometry
	unsigned long long color_hash;  // fingerprint of the element array perm was made for (0: none)
	int ncol;
	int col_off[65];
	int *perm, *iperm, *dpos;
	void* otmp;    // scratch of the in-place permutations
	float* ssor_y; // sweep vector (double-float, 4 floats per node)
	float4* ssor_d;  // the relaxation blocks' FP32 halves, packed (k_pack_hi) before every solve
	// the sweeps' blocks as sliced ELL (lower-colour and higher-colour parts)
	int sl_n;            // slices
	int sl_base[65];     // first slice of each colour
	int *sl_lw, *sl_uw, *sl_lp, *sl_up;  // widths and slice offsets (n + 1 each)
	int* sl_wm;          // device copy of sl_wmax
	long sl_lcap, sl_ucap;
	float4 *sl_lv, *sl_uv;
	int *sl_lc, *sl_uc;
	int sl_wmax[64][2];  // widest slice of each colour: lower-colour, higher-colour blocks
	unsigned* ssor_bar;  // grid barrier words of the persistent sweep kernel
	int ssor_grid;       // its cooperative grid (0: the per-phase kernels)
	int tma_grid;        // the TMA-staged sweep kernel's grid (one block per SM; 0: not used)
	int tma_smem_max;    // dynamic shared memory a block of it may have
	int linv_grid;       // cooperative grid of k_linv_all (0: not sized yet, -1: per-row launches)
	long polls;          // polls per grid barrier before it gives up (the solve graph's)

	// two-level SSOR: aggregates are the cells of an agx x agy grid over the
	// bounding box (origin ax0, ay0, cell acw x ach, rotation scale aH),
	// numbered along the shorter side first (axfast: x is that side)
	bool agg_valid;      // the aggregation belongs to the current node order and coordinates
	unsigned long long* e64;  // staging of 64-bit element ids (bfmi_set_geometry_u64), and its error word
	unsigned long long* e64_bad;
	int coarse_ok;       // the coarse factor is ready (else the solve runs plain SSOR)
	int na, nc, nc_cap, agx, agy, axfast, abw;
	double ax0, ay0, acw, ach, aH;
	int *agg, *agg_ptr, *agg_nodes;
	int nchunk, chunk_cap;
	int *chunk_start, *chunk_agg, *agg_chunk;
	double* cpart;  // per chunk partial sums (81 doubles)
	float4* pnode;
	float2* aband;          // band A_c then L (double-float pairs)
	double* diag0;          // the diagonal of A_c
	float *xl, *xu;         // X = L^-1 and X^T by rows (FP32, padded rows)
	float2 *lbm, *lbd, *lbw;  // blocked inversion: M_k, X_kk (nc_cap + COARSE_MAX_BW rows of bw), two block rows of X
	float2 *rc, *ayt, *yc;  // coarse vectors (double-float pairs, zero pads)
	int* coarse_err;
	int coarse_grid;        // cooperative grid of k_coarse_apply (0: not sized yet, -1: none)
	// the coarse factorisation and inverse run on a side stream while the
	// main stream builds the sweeps' sliced-ELL copies (coarse_setup forks,
	// coarse_finish joins): the factorisation holds one SM for milliseconds
	cudaStream_t side;
	cudaEvent_t fork_ev, join_ev;
	int coarse_pending;
	// the TMA sweep kernel's work list for the triangular products
	// (CoarseArgs::tri_*), packed: built for tri_n coarse DOFs and tri_g blocks
	int* tri;
	long tri_cap;
	int tri_g, tri_n;
	long tri_seg_off, tri_row_off;

};

enum : unsigned { ORD_COORDS = 1, ORD_ELEMS = 2, ORD_MASKS = 4, ORD_EDGES = 8, ORD_FIELDS = 16, ORD_LEDGES = 32, ORD_ALL = 63 };

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

bool ssor_pc(int pc) {
	return pc == BFM_GPU_PC_SSOR || pc == BFM_GPU_PC_LEARNED_SSOR || pc == BFM_GPU_PC_SSOR2 || pc == BFM_GPU_PC_LEARNED_SSOR2;
}
bool coarse_pc(int pc) { return pc == BFM_GPU_PC_SSOR2 || pc == BFM_GPU_PC_LEARNED_SSOR2; }
bool learned_pc(int pc) {
	return pc == BFM_GPU_PC_LEARNED || pc == BFM_GPU_PC_LEARNED_SSOR || pc == BFM_GPU_PC_LEARNED_SSOR2;
}
bool mixed_prec(int precision) { return precision == BFM_GPU_MIXED || precision == BFM_GPU_MIXED_EXACT; }
// the layout of the Krylov vectors the SSOR sweeps read and write
int precision_vt(int precision) {
	return precision == BFM_GPU_FP64_DF ? VT_DF : mixed_prec(precision) ? VT_F32 : VT_F64;
}

// Node-block pattern of the current element array (steps 1-2 of the assembly).
int build_pattern(bfm_gpu_problem* P) {
	cudaStream_t const st = P->stream;
	if (incidence(P, P->elems, P->NE, P->kind, P->cnt, P->inc_ptr, P->inc, MAXV, ERR_VALENCE)) return -1;
	k_rows_count<<<blocks_for(P->N), TPB, 0, st>>>(P->N, P->kind, P->elems, P->inc_ptr, P->inc, P->cand, P->row_len, P->err);
	if (scan(P, P->row_len, P->row_ptr, P->N)) return -1;
	k_rows_fill<<<blocks_for(P->N), TPB, 0, st>>>(P->N, P->kind, P->inc_ptr, P->cand, P->row_ptr, P->cols);
	CK(cudaGetLastError());
	return 0;
}

// Colour the node graph of the current (caller-order) pattern and derive the
// colour-major numbering: colour by colour, ascending caller index within a
// colour.  DSATUR on the host (the uncoloured node with the most distinct
// colours among its neighbours goes next, saturation buckets, most recent
// first within a bucket: linear in the edges, 60 ms for a million nodes):
// every colour is a grid-wide step of every sweep, and DSATUR finds 3
// colours on triangle meshes where greedy in node order needs 4 and the
// parallel random-priority colourings 6-7.  Deterministic; the pattern is
// copied to the host once, and the result is reused while the element array
// keeps its fingerprint.
static int dsatur(long n, const int* rp, const int* cols, int* col) {
	uint64_t* mask = (uint64_t*) calloc(n + 1, sizeof(uint64_t));
	int* sat = (int*) calloc(n + 1, sizeof(int));
	long* nxt = (long*) malloc((n + 1) * sizeof(long));
	long* prv = (long*) malloc((n + 1) * sizeof(long));
	if (!mask || !sat || !nxt || !prv) {
		free(mask);
		free(sat);
		free(nxt);
		free(prv);
		return -1;
	}
	long head[65];
	for (int b = 0; b < 65; b++) head[b] = -1;
	for (long v = n - 1; v >= 0; v--) {
		col[v] = -1;
		nxt[v] = head[0];
		prv[v] = -1;
		if (head[0] >= 0) prv[head[0]] = v;
		head[0] = v;
	}
	int top = 0;
	for (long done = 0; done < n; done++) {
		while (top > 0 && head[top] < 0) top--;
		long const v = head[top];
		head[top] = nxt[v];
		if (nxt[v] >= 0) prv[nxt[v]] = -1;
		int c = 0;
		while (c < 63 && ((mask[v] >> c) & 1)) c++;
		col[v] = c;
		for (int k = rp[v]; k < rp[v + 1]; k++) {
			long const u = cols[k];
			if (u < 0 || u >= n || u == v || col[u] >= 0 || ((mask[u] >> c) & 1)) continue;
			mask[u] |= 1ull << c;
			int b = sat[u];
			if (prv[u] >= 0) nxt[prv[u]] = nxt[u];
			else head[b] = nxt[u];
			if (nxt[u] >= 0) prv[nxt[u]] = prv[u];
			b = sat[u] = b < 64 ? b + 1 : 64;
			prv[u] = -1;
			nxt[u] = head[b];
			if (head[b] >= 0) prv[head[b]] = u;
			head[b] = u;
			if (b > top) top = b;
		}
	}
	free(mask);
	free(sat);
	free(nxt);
	free(prv);
	return 0;
}

// Cells of the coarse grid for n nodes in a w x h box: about one per
// `per_cell` nodes (BFM_GPU_COARSE_NODES, default 1000), at most 1024, as
// square as the box allows, and fewer while the band factorisation (one
// block, about 3 cells x bw^2 / 2 double-float updates) would exceed 8e6.
// Returns the half-bandwidth of A_c for the short-side-first numbering.
int coarse_grid(long n, double w, double h, int* gx_out, int* gy_out) {
	long per_cell = 1000;
	if (const char* e = getenv("BFM_GPU_COARSE_NODES")) {
		long const v = atol(e);
		if (v > 0) per_cell = v;
	}
	long target = n / per_cell;
	target = target < 1 ? 1 : target > 1024 ? 1024 : target;
	for (;;) {
		int gx = 1, gy = 1;
		if (w > 0 && h > 0) {
			gx = (int) lround(sqrt((double) target * w / h));
			gx = gx < 1 ? 1 : gx > target ? (int) target : gx;
			gy = (int) lround((double) target / gx);
			// rounding both counts may overshoot: at most `target` cells
			gy = gy > target / gx ? (int) (target / gx) : gy;
			gy = gy < 1 ? 1 : gy;
		}
		else if (w > 0) gx = (int) target;
		else if (h > 0) gy = (int) target;
		int const gs = gx < gy ? gx : gy;
		int const bw = 3 * (gs + 1) + 2;
		double const cost = 1.5 * gx * gy * (double) bw * bw;
		if ((bw <= COARSE_MAX_BW && cost <= 8e6) || target == 1) {
			*gx_out = gx;
			*gy_out = gy;
			return bw;
		}
		target = target * 9 / 10;
	}
}

// The coarse cells of n nodes with coordinates xy (x, y per node): the
// coarse_grid cells over the bounding box, numbered along the shorter side
// first, cells a hair wider than the box so the far edge falls inside the
// last one.  Depends only on the set of coordinates, not on the node order.
struct CellGrid {
	int gx = 1, gy = 1, bw = 8;
	double x0 = 0, y0 = 0, cw = 1, ch = 1;
};
void node_cells(long N, const double* xy, int* ag, CellGrid* g) {
	double x0 = 0, y0 = 0, x1 = 0, y1 = 0;
	for (long i = 0; i < N; i++) {
		double const x = xy[2 * i], y = xy[2 * i + 1];
		if (i == 0 || x < x0) x0 = x;
		if (i == 0 || x > x1) x1 = x;
		if (i == 0 || y < y0) y0 = y;
		if (i == 0 || y > y1) y1 = y;
	}
	double const w = x1 - x0, h = y1 - y0;
	int gx = 1, gy = 1;
	int const bw = coarse_grid(N, w, h, &gx, &gy);
	double const cw = w > 0 ? w * (1.0 + 1e-12) / gx : 1.0;
	double const ch = h > 0 ? h * (1.0 + 1e-12) / gy : 1.0;
	for (long i = 0; i < N; i++) {
		int cx = (int) ((xy[2 * i] - x0) / cw), cy = (int) ((xy[2 * i + 1] - y0) / ch);
		cx = cx < 0 ? 0 : cx >= gx ? gx - 1 : cx;
		cy = cy < 0 ? 0 : cy >= gy ? gy - 1 : cy;
		ag[i] = cell_id(cx, cy, gx, gy, gx <= gy);
	}
	g->gx = gx;
	g->gy = gy;
	g->bw = bw;
	g->x0 = x0;
	g->y0 = y0;
	g->cw = cw;
	g->ch = ch;
}

int color_nodes(bfm_gpu_problem* P) {
	BFM_RANGE("color_nodes");
	cudaStream_t const st = P->stream;
	long const N = P->N;
	if (!P->perm && (dalloc(&P->perm, N) || dalloc(&P->iperm, N) || dalloc(&P->dpos, N))) return -1;
	int* rp = (int*) malloc((N + 1) * sizeof(int));
	int* col = (int*) malloc((N + 1) * sizeof(int));
	int* perm = (int*) malloc((N + 1) * sizeof(int));
	int* iperm = (int*) malloc((N + 1) * sizeof(int));
	int* cols = nullptr;
	int rc = 0;
	if (!rp || !col || !perm || !iperm) rc = fail("out of host memory");
	if (!rc && cudaMemcpyAsync(rp, P->row_ptr, (N + 1) * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
		rc = fail("pattern copy failed");
	if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = fail("pattern copy failed");
	if (!rc && !(cols = (int*) malloc((size_t) rp[N] * sizeof(int) + 4))) rc = fail("out of host memory");
	if (!rc && (cudaMemcpyAsync(cols, P->cols, (size_t) rp[N] * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	            cudaStreamSynchronize(st) != cudaSuccess))
		rc = fail("pattern copy failed");
	if (!rc && dsatur(N, rp, cols, col)) rc = fail("out of host memory");
	if (!rc) {
		int counts[64] = {0};
		for (long i = 0; i < N; i++) counts[col[i]]++;
		P->ncol = 0;
		P->col_off[0] = 0;
		for (int c = 0; c < 64; c++) {
			if (counts[c]) P->ncol = c + 1;
			P->col_off[c + 1] = P->col_off[c] + counts[c];
		}
		// within a colour (rows that share no element, so their order does not
		// change the sweeps) the nodes go by coarse cell, then by index: a
		// cell's nodes are then three or four contiguous runs, which the
		// two-level form's restriction reads in whole sectors
		double* xy = (double*) malloc((2 * N + 2) * sizeof(double));
		int* cell = (int*) malloc((N + 1) * sizeof(int));
		CellGrid g;
		if (!xy || !cell) rc = fail("out of host memory");
		else if (cudaMemcpyAsync(xy, P->coords, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
		         cudaStreamSynchronize(st) != cudaSuccess)
			rc = fail("coordinate copy failed");
		else node_cells(N, xy, cell, &g);
		long const nb = 64l * g.gx * g.gy;
		long* next = rc ? nullptr : (long*) calloc(nb + 1, sizeof(long));
		if (!rc && !next) rc = fail("out of host memory");
		if (!rc) {
			// counting sort on (colour, cell), stable in the node index
			for (long i = 0; i < N; i++) next[(long) col[i] * g.gx * g.gy + cell[i] + 1]++;
			for (long k = 0; k < nb; k++) next[k + 1] += next[k];
			for (long i = 0; i < N; i++) {
				int const w = (int) next[(long) col[i] * g.gx * g.gy + cell[i]]++;
				iperm[i] = w;
				perm[w] = (int) i;
			}
		}
		free(xy);
		free(cell);
		free(next);
	}
	if (!rc) {
		if (cudaMemcpyAsync(P->perm, perm, N * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		    cudaMemcpyAsync(P->iperm, iperm, N * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
		    cudaStreamSynchronize(st) != cudaSuccess)
			rc = fail("ordering upload failed");
	}
	free(rp);
	free(col);
	free(perm);
	free(iperm);
	free(cols);
	if (rc) return rc;
	P->colored = true;
	P->agg_valid = false;
	P->graph_precision = -1;  // the solve graph's sweep phases follow the colour ranges
	return 0;
}

// scratch of the in-place permutations (also the fingerprint's word)
int ensure_otmp(bfm_gpu_problem* P) {
	if (P->otmp) return 0;
	long const N = P->N;
	size_t const bytes = (size_t) (16 * N > (long) P->max_conds * N ? 16 * N : (long) P->max_conds * N) + 16;
	CK(cudaMalloc(&P->otmp, bytes));
	return 0;
}

// fingerprint of the current element array (caller order)
int elems_hash(bfm_gpu_problem* P, unsigned long long* h) {
	if (ensure_otmp(P)) return -1;
	unsigned long long* d = (unsigned long long*) P->otmp;
	CK(cudaMemsetAsync(d, 0, sizeof *d, P->stream));
	long const n = (long) P->NE * P->kind;
	k_elems_hash<<<4 * num_sms(), TPB, 0, P->stream>>>(n, P->elems, d);
	CK(cudaMemcpyAsync(h, d, sizeof *h, cudaMemcpyDeviceToHost, P->stream));
	CK(cudaStreamSynchronize(P->stream));
	*h ^= mix64((unsigned long long) P->N * 0x9e3779b97f4a7c15ull + (unsigned long long) P->kind) | 1ull;
	return 0;
}

// Bring the node-indexed inputs into the working order (to_work) or back to
// the caller's, each array once: `ordered` tracks which are permuted.
int reorder_inputs(bfm_gpu_problem* P, bool to_work) {
	cudaStream_t const st = P->stream;
	long const N = P->N;
	if (ensure_otmp(P)) return -1;
	const int* data_map = to_work ? P->perm : P->iperm;  // dst[i] = src[map[i]]
	const int* id_map = to_work ? P->iperm : P->perm;
	auto todo = [&](unsigned bit) { return to_work ? !(P->ordered & bit) : (P->ordered & bit) != 0; };
	auto gather_d2 = [&](double* a) -> int {
		k_gather_nodes<double><<<blocks_for(2 * N), TPB, 0, st>>>(N, 2, a, data_map, (double*) P->otmp);
		CK(cudaMemcpyAsync(a, P->otmp, 2 * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
		return 0;
	};
	if (todo(ORD_COORDS) && gather_d2(P->coords)) return -1;
	for (int f = 0; f < P->forces.nf; f++)
		if (todo(ORD_FIELDS) && P->forces.field[f] && gather_d2(P->force_fields[f])) return -1;
	if (todo(ORD_MASKS)) {
		for (int c = 0; c < P->n_conds; c++)
			k_gather_nodes<uint8_t><<<blocks_for(N), TPB, 0, st>>>(N, 1, P->masks + c * N, data_map,
			                                                     (uint8_t*) P->otmp + c * N);
		if (P->n_conds) CK(cudaMemcpyAsync(P->masks, P->otmp, (long) P->n_conds * N, cudaMemcpyDeviceToDevice, st));
	}
	if (todo(ORD_ELEMS)) k_map_ids<<<blocks_for((long) P->NE * P->kind), TPB, 0, st>>>((long) P->NE * P->kind, P->N, P->elems, id_map);
	if (todo(ORD_EDGES) && P->n_edges) k_map_ids<<<blocks_for(2l * P->n_edges), TPB, 0, st>>>(2l * P->n_edges, P->N, P->edges, id_map);
	if (todo(ORD_LEDGES) && P->n_loads) k_map_ids<<<blocks_for(2l * P->n_loads), TPB, 0, st>>>(2l * P->n_loads, P->N, P->ledges, id_map);
	CK(cudaGetLastError());
	P->ordered = to_work ? ORD_ALL : 0u;
	return 0;
}

// Node order for this assembly: colour-major for the SSOR preconditioners
// (colouring the caller's graph when the geometry changed), else the caller's.
int prepare_order(bfm_gpu_problem* P) {
	bool const want = ssor_pc(P->precond);
	if (P->ordered && (!want || !P->colored))
		if (reorder_inputs(P, false)) return -1;
	if (!want) return 0;
	if (!P->colored) {
		// the element array is in the caller's order here: reuse the colouring of the same mesh
		unsigned long long h = 0;
		if (elems_hash(P, &h)) return -1;
		if (h == P->color_hash && P->perm) {
			P->colored = true;
		}
		else {
			if (build_pattern(P) || color_nodes(P)) return -1;
			P->color_hash = h;
		}
	}
	return reorder_inputs(P, true);
}

// ---- two-level SSOR: aggregation, coarse operator
// Cooperative grid of the one-launch coarse correction (every block resident:
// its grid barriers wait for all of them); -1 where it does not fit
int coarse_apply_grid(bfm_gpu_problem* P) {
	if (P->coarse_grid == 0) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*) k_coarse_apply, CX_T, 0) != cudaSuccess || nb < 1) {
			cudaGetLastError();
			P->coarse_grid = -1;
		}
		else P->coarse_grid = nb * num_sms();
	}
	return P->coarse_grid;
}

CoarseArgs coarse_args(bfm_gpu_problem* P, const void* r, int vt) {
	CoarseArgs c;
	memset(&c, 0, sizeof c);
	c.na = P->na;
	c.nc = P->nc;
	c.gx = P->agx;
	c.gy = P->agy;
	c.xfast = P->axfast;
	c.bw = P->abw;
	c.agg_ptr = P->agg_ptr;
	c.agg_nodes = P->agg_nodes;
	c.agg = P->agg;
	c.pnode = P->pnode;
	c.band = P->aband;
	c.diag0 = P->diag0;
	c.xl = P->xl;
	c.xu = P->xu;
	c.yc = P->yc;
	c.rc = P->rc;
	c.yt = P->ayt;
	c.r = r;
	c.df = vt;
	c.row_ptr = P->row_ptr;
	c.cols = P->cols;
	// A_c from the FP64 operator where the precision assembles one, else from
	// the FP32 operator (MIXED)
	c.vals64 = P->precision != BFM_GPU_MIXED ? P->vals64 : nullptr;
	c.vals32 = P->vals32;
	c.corr32 = P->corr32;
	c.err = P->coarse_err;
	c.bar = P->ssor_bar;
	c.berr = P->st ? &P->st->ssor_err : P->coarse_err;
	c.polls = P->polls;
	c.nchunk = P->nchunk;
	c.chunk_start = P->chunk_start;
	c.chunk_agg = P->chunk_agg;
	c.agg_chunk = P->agg_chunk;
	c.part = P->cpart;
	// BFM_GPU_SSOR_STAGE_TABLES=0: the sweep kernel's coarse stages take
	// their fallback paths (tested against the tables on the same problem)
	char const* tb = getenv("BFM_GPU_SSOR_STAGE_TABLES");
	c.tables = !(tb && tb[0] == '0');
	c.tri_g = c.tables ? P->tri_g : 0;
	if (c.tri_g > 0) {
		c.tri_sp = P->tri;
		c.tri_rp = P->tri + P->tri_g + 1;
		c.tri_seg = reinterpret_cast<const int4*>(P->tri + P->tri_seg_off);
		c.tri_row = reinterpret_cast<const int4*>(P->tri + P->tri_row_off);
	}
	return c;
}

// Work list of the TMA sweep kernel's triangular products (y_t = X r_c, y_c =
// X^T y_t) for a grid of G blocks.  Rows go to blocks in zig-zag order (block
// b: rows 2 G m + b and 2 G m + 2 G - 1 - b, m = 0, 1, .., so every block's
// rows add up to about the same length), each row cut into segments of at
// most TRI_SEG entries, a block's segments sorted longest first (the kernel
// deals them to its warps in turn).  Packed into one device buffer; left
// unbuilt (tri_g = 0: the kernel's per-warp rows instead) when a block would
// need more than TRI_SLOTS segment sums.
int build_tri_lists(bfm_gpu_problem* P, int G) {
	int const n = P->nc;
	if (G <= 0 || (P->tri_g == G && P->tri_n == n)) return 0;
	P->tri_g = 0;
	std::vector<int> sp(G + 1), rp(G + 1);
	std::vector<int4> segs, rows;
	for (int b = 0; b < G; b++) {
		sp[b] = (int) segs.size();
		rp[b] = (int) rows.size();
		size_t const first = segs.size();
		int slot = 0;
		for (long m = 0;; m++) {
			long const pair[2] = {2l * G * m + b, 2l * G * m + 2l * G - 1 - b};
			if (pair[0] >= n) break;
			for (long i : pair) {
				if (i >= n) continue;
				int const len = (int) i + 1, cnt = (len + TRI_SEG - 1) / TRI_SEG;
				rows.push_back(make_int4((int) i, slot, cnt, 0));
				for (int q = 0; q < cnt; q++)
					segs.push_back(make_int4((int) i, q * TRI_SEG, std::min(TRI_SEG, len - q * TRI_SEG), slot++));
			}
		}
		if (slot > TRI_SLOTS) return 0;
		std::stable_sort(segs.begin() + first, segs.end(), [](const int4& x, const int4& y) { return x.z > y.z; });
	}
	sp[G] = (int) segs.size();
	rp[G] = (int) rows.size();
	long const hdr = (2l * G + 2 + 3) / 4 * 4;
	long const total = hdr + 4l * (long) (segs.size() + rows.size());
	if (total > P->tri_cap) {
		if (P->tri) cudaFree(P->tri);
		P->tri = nullptr;
		P->tri_cap = 0;
		if (dalloc(&P->tri, total)) return -1;
		P->tri_cap = total;
	}
	std::vector<int> h((size_t) total, 0);
	std::copy(sp.begin(), sp.end(), h.begin());
	std::copy(rp.begin(), rp.end(), h.begin() + G + 1);
	memcpy(h.data() + hdr, segs.data(), segs.size() * sizeof(int4));
	memcpy(h.data() + hdr + 4 * segs.size(), rows.data(), rows.size() * sizeof(int4));
	CK(cudaMemcpy(P->tri, h.data(), (size_t) total * sizeof(int), cudaMemcpyHostToDevice));
	P->tri_seg_off = hdr;
	P->tri_row_off = hdr + 4l * (long) segs.size();
	P->tri_g = G;
	P->tri_n = n;
	return 0;
}


// Aggregates for the current (working-order) coordinates: cells of a grid
// over the bounding box (coarse_grid), numbered along the shorter side
// first; node lists per cell in ascending node order (a host counting sort:
// deterministic).  Redone when the colouring is.
int build_aggregates(bfm_gpu_problem* P) {
	BFM_RANGE("build_aggregates");
	cudaStream_t const st = P->stream;
	long const N = P->N;
	double* xy = (double*) malloc((2 * N + 2) * sizeof(double));
	int* ag = (int*) malloc((N + 1) * sizeof(int));
	int* nodes = (int*) malloc((N + 1) * sizeof(int));
	int rc = 0;
	if (!xy || !ag || !nodes) rc = fail("out of host memory");
	if (!rc && (cudaMemcpyAsync(xy, P->coords, 2 * N * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
	            cudaStreamSynchronize(st) != cudaSuccess))
		rc = fail("coordinate copy failed");
	CellGrid cg;
	if (!rc) node_cells(N, xy, ag, &cg);
	int const gx = cg.gx, gy = cg.gy, bw = cg.bw;
	double const x0 = cg.x0, y0 = cg.y0, cw = cg.cw, ch = cg.ch;
	int const na = gx * gy, nc = 3 * na;
	int* ptr = (int*) calloc(na + 1, sizeof(int));
	if (!rc && !ptr) rc = fail("out of host memory");
	if (!rc) {
		for (long i = 0; i < N; i++) ptr[ag[i] + 1]++;
		for (int I = 0; I < na; I++) ptr[I + 1] += ptr[I];
		int* next = (int*) malloc((na + 1) * sizeof(int));
		if (!next) rc = fail("out of host memory");
		else {
			memcpy(next, ptr, na * sizeof(int));
			for (long i = 0; i < N; i++) nodes[next[ag[i]]++] = (int) i;
			free(next);
		}
	}
	// chunks for the parallel reductions: runs of consecutive nodes of one
	// aggregate, at most COARSE_CHUNK each (a chunk's nodes are the rows
	// agg_nodes[chunk start] onwards)
	auto new_chunk = [&](int I, int k) { return k == ptr[I] || nodes[k] != nodes[k - 1] + 1; };
	int nchunk = 0;
	if (!rc)
		for (int I = 0; I < na; I++)
			for (int k = ptr[I], len = 0; k < ptr[I + 1]; k++, len++)
				if (new_chunk(I, k) || len == COARSE_CHUNK) {
					nchunk++;
					len = 0;
				}
	int* cst = (int*) malloc((nchunk + 1) * sizeof(int));
	int* cag = (int*) malloc((nchunk + 1) * sizeof(int));
	int* ach = (int*) malloc((na + 1) * sizeof(int));
	if (!rc && (!cst || !cag || !ach)) rc = fail("out of host memory");
	if (!rc) {
		int q = 0;
		for (int I = 0; I < na; I++) {
			ach[I] = q;
			for (int k = ptr[I], len = 0; k < ptr[I + 1]; k++, len++)
				if (new_chunk(I, k) || len == COARSE_CHUNK) {
					cst[q] = k;
					cag[q] = I;
					q++;
					len = 0;
				}
		}
		ach[na] = q;
		cst[q] = ptr[na];
	}
	if (!rc && nchunk + 1 > P->chunk_cap) {
		void* old[] = {P->chunk_start, P->chunk_agg, P->cpart};
		for (void* o : old)
			if (o) cudaFree(o);
		P->chunk_start = P->chunk_agg = nullptr;
		P->cpart = nullptr;
		if (dalloc(&P->chunk_start, nchunk + 1) || dalloc(&P->chunk_agg, nchunk + 1) || dalloc(&P->cpart, 81l * (nchunk + 1)))
			rc = -1;
		else P->chunk_cap = nchunk + 1;
	}
	if (!rc && nc > P->nc_cap) {
		// (re)allocate for the larger coarse space (the band at the widest bandwidth)
		void* old[] = {P->agg_ptr, P->agg_chunk, P->aband, P->diag0, P->rc, P->ayt, P->yc, P->xl, P->xu, P->lbm, P->lbd, P->lbw};
		for (void* q : old)
			if (q) cudaFree(q);
		P->lbm = P->lbd = P->lbw = nullptr;
		P->agg_ptr = P->agg_chunk = nullptr;
		P->aband = nullptr;
		P->diag0 = nullptr;
		P->xl = P->xu = nullptr;
		P->rc = P->ayt = P->yc = nullptr;
		if (dalloc(&P->agg_ptr, na + 1) || dalloc(&P->agg_chunk, na + 1) ||
		    dalloc(&P->aband, (long) nc * (COARSE_MAX_BW + 1)) || dalloc(&P->diag0, nc) || dalloc(&P->rc, nc + 4) ||
		    dalloc(&P->ayt, nc + 4) || dalloc(&P->yc, nc) || dalloc(&P->xl, xrow(nc)) || dalloc(&P->xu, xrow(nc)) ||
		    dalloc(&P->lbm, (long) (nc + COARSE_MAX_BW) * COARSE_MAX_BW) ||
		    dalloc(&P->lbd, (long) (nc + COARSE_MAX_BW) * COARSE_MAX_BW) || dalloc(&P->lbw, 2l * COARSE_MAX_BW * nc) ||
		    cudaMemsetAsync(P->rc, 0, (nc + 4) * sizeof(float2), st) != cudaSuccess ||
		    cudaMemsetAsync(P->ayt, 0, (nc + 4) * sizeof(float2), st) != cudaSuccess)
			rc = -1;
		else P->nc_cap = nc;
	}
	if (!rc && !P->agg && (dalloc(&P->agg, N) || dalloc(&P->agg_nodes, N) || dalloc(&P->pnode, N) || dalloc(&P->coarse_err, 2) ||
	                       cudaMemsetAsync(P->coarse_err, 0, 2 * sizeof(int), st) != cudaSuccess))
		rc = -1;
	if (!rc && (cudaMemcpyAsync(P->agg, ag, N * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaMemcpyAsync(P->agg_nodes, nodes, N * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaMemcpyAsync(P->agg_ptr, ptr, (na + 1) * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaMemcpyAsync(P->chunk_start, cst, (nchunk + 1) * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaMemcpyAsync(P->chunk_agg, cag, (nchunk + 1) * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaMemcpyAsync(P->agg_chunk, ach, (na + 1) * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
	            cudaStreamSynchronize(st) != cudaSuccess))
		rc = fail("aggregate upload failed");
	free(xy);
	free(ag);
	free(nodes);
	free(ptr);
	free(cst);
	free(cag);
	free(ach);
	if (rc) return rc;
	P->na = na;
	P->nc = nc;
	P->nchunk = nchunk;
	P->agx = gx;
	P->agy = gy;
	P->axfast = gx <= gy;
	P->abw = bw;
	P->ax0 = x0;
	P->ay0 = y0;
	P->acw = cw;
	P->ach = ch;
	P->aH = cw > ch ? cw : ch;
	P->agg_valid = true;
	P->graph_precision = -1;  // the graph's coarse kernels take the new sizes
	return 0;
}

// Per assembly: node offsets and free DOFs, A_c = P^T A P (band), its band
// Cholesky factor and X = L^-1.  A neighbour beyond the adjacent cells leaves
// the solve on plain SSOR (coarse_ok = 0).
// The sweeps' sliced-ELL copy of the FP32 blocks of the current assembly
// (after the values; the colour order must be the matrix's).  The slice
// widths are read back to size the arrays: one host sync per assembly.
int build_sell(bfm_gpu_problem* P) {
	cudaStream_t const st = P->stream;
	int const nc = P->ncol > 0 ? P->ncol : 1;
	SellMap m;
	memset(&m, 0, sizeof m);
	m.ncol = nc;
	int ns = 0;
	for (int c = 0; c < nc; c++) {
		m.off[c] = P->ncol > 0 ? P->col_off[c] : 0;
		m.sbase[c] = ns;
		int const rows = (P->ncol > 0 ? P->col_off[c + 1] : P->N) - m.off[c];
		ns += (rows + 31) / 32;
	}
	m.off[nc] = P->N;
	m.sbase[nc] = ns;
	P->sl_n = ns;
	memcpy(P->sl_base, m.sbase, sizeof m.sbase);
	long const cap_s = P->N / 32 + 66;
	if (!P->sl_lw && (dalloc(&P->sl_lw, cap_s) || dalloc(&P->sl_uw, cap_s) || dalloc(&P->sl_lp, cap_s + 1) ||
	                  dalloc(&P->sl_up, cap_s + 1)))
		return -1;
	if (ns == 0) return 0;
	int const warps_tpb = TPB / 32;
	k_sell_width<<<(ns + warps_tpb - 1) / warps_tpb, TPB, 0, st>>>(ns, m, P->row_ptr, P->cols, P->sl_lw, P->sl_uw);
	if (scan(P, P->sl_lw, P->sl_lp, ns) || scan(P, P->sl_uw, P->sl_up, ns)) return -1;
	if (!P->sl_wm && dalloc(&P->sl_wm, 2 * 64)) return -1;
	k_sell_wmax<<<nc, TPB, 0, st>>>(m, P->sl_lw, P->sl_uw, P->sl_wm);
	int tot[2] = {0, 0};
	CK(cudaMemcpyAsync(&tot[0], P->sl_lp + ns, sizeof(int), cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(&tot[1], P->sl_up + ns, sizeof(int), cudaMemcpyDeviceToHost, st));
	CK(cudaMemcpyAsync(P->sl_wmax, P->sl_wm, 2 * nc * sizeof(int), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (tot[0] > P->sl_lcap) {
		if (P->sl_lv) cudaFree(P->sl_lv);
		if (P->sl_lc) cudaFree(P->sl_lc);
		P->sl_lv = nullptr;
		P->sl_lc = nullptr;
		P->sl_lcap = 0;
		if (dalloc(&P->sl_lv, tot[0]) || dalloc(&P->sl_lc, tot[0])) return -1;
		P->sl_lcap = tot[0];
	}
	if (tot[1] > P->sl_ucap) {
		if (P->sl_uv) cudaFree(P->sl_uv);
		if (P->sl_uc) cudaFree(P->sl_uc);
		P->sl_uv = nullptr;
		P->sl_uc = nullptr;
		P->sl_ucap = 0;
		if (dalloc(&P->sl_uv, tot[1]) || dalloc(&P->sl_uc, tot[1])) return -1;
		P->sl_ucap = tot[1];
	}
	k_sell_fill<<<(ns + warps_tpb - 1) / warps_tpb, TPB, 0, st>>>(ns, m, P->row_ptr, P->cols,
	                                                            reinterpret_cast<const float4*>(P->vals32), P->sl_lp,
	                                                            P->sl_up, P->sl_lv, P->sl_lc, P->sl_uv, P->sl_uc);
	CK(cudaGetLastError());
	return 0;
}

int coarse_finish(bfm_gpu_problem* P);

// fork: the factorisation and inverse go to the side stream (coarse_finish
// joins it); else everything runs on the problem's stream
int coarse_setup(bfm_gpu_problem* P, bool fork) {
	BFM_RANGE("coarse_setup");
	cudaStream_t st = P->stream;
	P->coarse_ok = 0;
	P->coarse_pending = 0;
	if (P->N == 0) return 0;
	if (!P->agg_valid && build_aggregates(P)) return -1;
	k_pnode<<<blocks_for(P->N), TPB, 0, st>>>(P->N, P->coords, P->agg, P->last_ci, P->ax0, P->ay0, P->acw, P->ach, P->agx,
	                                          P->agy, P->axfast, 1.0 / P->aH, P->pnode);
	CK(cudaMemsetAsync(P->aband, 0, (size_t) P->nc * (P->abw + 1) * sizeof(float2), st));
	CK(cudaMemsetAsync(P->diag0, 0, (size_t) P->nc * sizeof(double), st));
	CK(cudaMemsetAsync(P->coarse_err, 0, 2 * sizeof(int), st));
	CoarseArgs ca = coarse_args(P, nullptr, VT_DF);
	// The set-up's grid barriers wait with the default limit (the solver
	// options' limit belongs to the solves) and report a timeout in
	// coarse_err[1], which no solve resets
	ca.polls = BARRIER_POLLS_DEFAULT;
	ca.berr = P->coarse_err + 1;
	k_coarse_ac<<<blocks_for(32l * P->nchunk), TPB, 0, st>>>(ca);
	k_coarse_ac_sum<<<blocks_for(81l * P->na), TPB, 0, st>>>(ca);
	int err = 0;
	CK(cudaMemcpyAsync(&err, P->coarse_err, sizeof(int), cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (err) return 0;
	if (fork && P->side) {
		CK(cudaEventRecord(P->fork_ev, st));
		CK(cudaStreamWaitEvent(P->side, P->fork_ev, 0));
		st = P->side;
	}
	CK(cudaFuncSetAttribute((const void*) k_coarse_chol, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                        (int) chol_smem(COARSE_MAX_BW, 3 * 1024)));
	k_coarse_chol<<<1, CHOL_T, chol_smem(P->abw, P->nc), st>>>(ca);
	// the padding of X's rows stays zero (the products read whole 16-byte groups)
	CK(cudaMemsetAsync(P->xl, 0, xrow(P->nc) * sizeof(float), st));
	CK(cudaMemsetAsync(P->xu, 0, xrow(P->nc) * sizeof(float), st));
	char const* lv = getenv("BFM_GPU_COARSE_LINV_COLUMNS");
	if (lv && lv[0] == '1') {
		// the column-wise inversion (one dependent chain of nc steps per column)
		k_coarse_linv<<<(P->nc + LINV_C * LINV_W - 1) / (LINV_C * LINV_W), 32 * LINV_W, linv_smem(P->abw), st>>>(ca);
	}
	else {
		// by block rows of b = bw: nc / b dependent launches
		int const b = P->abw > 0 ? P->abw : 1, nb = (P->nc + b - 1) / b;
		CK(cudaFuncSetAttribute((const void*) k_linv_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                        (int) linv_diag_smem(COARSE_MAX_BW)));
		k_linv_diag<<<nb, LB_T, linv_diag_smem(b), st>>>(ca, b, P->lbm, P->lbd);
		// the block rows in one cooperative launch (BFM_GPU_COARSE_LINV_LAUNCHES=1: a launch each)
		char const* ll = getenv("BFM_GPU_COARSE_LINV_LAUNCHES");
		bool one = false;
		if (!(ll && ll[0] == '1') && P->ssor_bar && nb > 1) {
			if (!P->linv_grid) {
				int nbk = 0;
				P->linv_grid = -1;
				if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbk, (const void*) k_linv_all, LB_T, 0) == cudaSuccess &&
				    nbk > 0)
					P->linv_grid = num_sms() * nbk;
				cudaGetLastError();
			}
			if (P->linv_grid > 0) {
				CK(cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), st));
				float2* lbw = P->lbw;
				void* pa[] = {&ca, (void*) &b, (void*) &P->lbm, (void*) &P->lbd, (void*) &lbw};
				one = cudaLaunchCooperativeKernel((const void*) k_linv_all, dim3(P->linv_grid), dim3(LB_T), pa, 0, st) ==
				      cudaSuccess;
				if (!one) {
					cudaGetLastError();
					P->linv_grid = -1;
				}
			}
		}
		if (!one)
			for (int k = 1; k < nb; k++) {
				long const outs = (long) std::min(b, P->nc - k * b) * (k * b);
				k_linv_step<<<(int) ((outs + LB_T - 1) / LB_T), LB_T, 0, st>>>(ca, b, k, P->lbm, P->lbd,
				                                                               P->lbw + (long) ((k + 1) & 1) * b * P->nc,
				                                                               P->lbw + (long) (k & 1) * b * P->nc);
			}
	}
	CK(cudaGetLastError());
	if (st != P->stream) CK(cudaEventRecord(P->join_ev, st));
	P->coarse_pending = 1;
	return st == P->stream ? coarse_finish(P) : 0;
}

// the end of the coarse set-up: the problem's stream waits for the side
// stream, then the work list and the inverse's timeout flag
int coarse_finish(bfm_gpu_problem* P) {
	if (!P->coarse_pending) return 0;
	P->coarse_pending = 0;
	cudaStream_t const st = P->stream;
	CK(cudaStreamWaitEvent(st, P->join_ev, 0));
	if (P->tma_grid > 0 && build_tri_lists(P, P->tma_grid)) return -1;
	if (P->linv_grid > 0) {
		int err = 0;
		CK(cudaMemcpyAsync(&err, P->coarse_err + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		if (err) return fail("a grid barrier of the coarse inverse timed out");
	}
	P->coarse_ok = 1;
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
		a.corr = P->corr32;
		a.vals64 = P->precision == BFM_GPU_MIXED_EXACT ? P->vals64 : nullptr;
	}
	a.block_pc = P->precond != BFM_GPU_PC_JACOBI;
	a.b = P->b;
	a.x = P->x;
	a.r = (V*) P->vec[0];
	a.u = (V*) P->vec[1];
	a.p = (V*) P->vec[2];
	a.s = (V*) P->vec[3];
	a.pn = (V*) P->vec[3];
	a.w = (V*) P->vec[4];
	a.z = (V*) P->vec[5];
	a.partials = P->partials;
	a.ticket = P->ticket;
	a.st = P->st;
	if (o) {
		a.opts.rtol = o->rtol;
		a.opts.drop2 = o->replace_drop * o->replace_drop;
		a.opts.max_iters = o->max_iters;
		// mixed precisions: restart the inner PCG at each FP64 refinement step,
		// or keep its direction (the default: fewer iterations on the plates)
		a.opts.restart = o->refine_restart == 1;
	}
	return a;
}

DfArgs df_args(bfm_gpu_problem* P, const bfm_gpu_opts_t* o) {
	DfArgs a;
	memset(&a, 0, sizeof a);
	a.N = P->N;
	a.row_ptr = P->row_ptr;
	a.cols = P->cols;
	a.hi = P->vals32;
	a.lo = P->vals32lo;
	a.srow = P->srow_df;
	a.vals64 = P->vals64;
	a.dinv = P->dinv32;
	a.block_pc = P->precond != BFM_GPU_PC_JACOBI;
	a.b = P->b;
	a.x = (float*) P->vec[5];
	a.x64 = P->x;
	a.r = (float*) P->vec[0];
	a.u = (float*) P->vec[1];
	a.p = (float*) P->vec[2];
	a.s = (float*) P->vec[3];
	a.w = (float*) P->vec[4];
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

int add_node(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* dep, void* fn, int grid, void** params,
             size_t smem = 0, int block = TPB) {
	cudaKernelNodeParams kp = {};
	kp.func = fn;
	kp.gridDim = dim3(grid);
	kp.blockDim = dim3(block);
	kp.sharedMemBytes = (unsigned) smem;
	kp.kernelParams = params;
	CK(cudaGraphAddKernelNode(node, g, dep, dep ? 1 : 0, &kp));
	return 0;
}

int add_conditional(cudaGraph_t g, cudaGraphNode_t* node, const cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                    cudaGraphConditionalNodeType type, cudaGraph_t* body) {
	cudaGraphNodeParams cp = {};
	cp.type = cudaGraphNodeTypeConditional;
	cp.conditional.handle = h;
	cp.conditional.type = type;
	cp.conditional.size = 1;
	CK(cudaGraphAddNode(node, g, dep, nullptr, dep ? 1 : 0, &cp));
	*body = cp.conditional.phGraph_out[0];
	return 0;
}

SsorArgs ssor_args(bfm_gpu_problem* P, const void* r, void* z) {
	SsorArgs a;
	memset(&a, 0, sizeof a);
	a.row_ptr = P->row_ptr;
	a.cols = P->cols;
	a.dpos = P->dpos;
	a.hi = P->vals32;
	a.dinv = reinterpret_cast<const float*>(P->ssor_d);
	a.r = r;
	a.z = z;
	a.y = P->ssor_y;
	a.partials = P->partials;
	a.ticket = P->ticket;
	a.st = P->st;
	a.polls = P->polls;
	a.lv = P->sl_lv;
	a.lc = P->sl_lc;
	a.lp = P->sl_lp;
	a.uv = P->sl_uv;
	a.uc = P->sl_uc;
	a.up = P->sl_up;
	memcpy(a.sbase, P->sl_base, sizeof a.sbase);
	return a;
}

// The two-level correction inside the persistent sweep kernel: at least three
// colours (its four stages need the sweeps' first four grid barriers);
// BFM_GPU_COARSE_SEPARATE=1 keeps it in a launch of its own
bool fuse_coarse(bfm_gpu_problem* P) {
	char const* e = getenv("BFM_GPU_COARSE_SEPARATE");
	return P->ssor_grid > 0 && P->ncol >= 3 && !(e && e[0] == '1');
}

// Tiling of the TMA-staged sweep kernel for the current colouring: the ring
// takes what the block's shared memory leaves after the coarse vector (fused
// two-level form); each phase's tiles hold as many whole slices as a stage
// fits at the colour's widest slice.  Returns the dynamic shared memory of a
// block, 0 when the kernel cannot be used here.
size_t tma_tiling(bfm_gpu_problem* P, SsorArgs& a, bool fused) {
	if (P->tma_grid <= 0 || P->ncol <= 0 || P->ncol > 63) return 0;
	// the staged coarse vector and the triangular products' work list
	size_t const vec = fused ? st_vec_bytes(P->nc) + ST_LIST_BYTES + (ST_RST_BYTES + 127) / 128 * 128 : 0;
	if ((size_t) P->tma_smem_max < vec + ST_NS * 4096) return 0;
	int const stage = (int) ((((size_t) P->tma_smem_max - vec) / ST_NS) / 128 * 128);
	int const nc = P->ncol;
	for (int ph = 0; ph < 2 * nc - 1; ph++) {
		bool const fwd = ph < nc;
		int const c = fwd ? ph : 2 * nc - 2 - ph;
		int const w = P->sl_wmax[c][fwd ? 0 : 1];
		int spt = (stage - ST_HDR) / (32 * (20 * w + 16));
		if (spt > ST_MAX_SPT) spt = ST_MAX_SPT;
		if (spt < 1) return 0;
		a.spt[ph] = spt;
	}
	a.stage_bytes = stage;
	return (size_t) stage * ST_NS + vec;
}

void* ssor_tma_kernel(int vt) {
	return vt == VT_DF ? (void*) k_ssor_tma<VT_DF> : vt == VT_F32 ? (void*) k_ssor_tma<VT_F32> : (void*) k_ssor_tma<VT_F64>;
}

// the sweep kernels of a vector layout (VT_*)
void* ssor_all_kernel(int vt) {
	return vt == VT_DF ? (void*) k_ssor_all<VT_DF> : vt == VT_F32 ? (void*) k_ssor_all<VT_F32> : (void*) k_ssor_all<VT_F64>;
}
void* ssor_fwd_kernel(int vt) {
	return vt == VT_DF ? (void*) k_ssor_fwd<VT_DF> : vt == VT_F32 ? (void*) k_ssor_fwd<VT_F32> : (void*) k_ssor_fwd<VT_F64>;
}
void* ssor_bwd_kernel(int vt) {
	return vt == VT_DF ? (void*) k_ssor_bwd<VT_DF> : vt == VT_F32 ? (void*) k_ssor_bwd<VT_F32> : (void*) k_ssor_bwd<VT_F64>;
}

// The 2 nc - 1 sweep phases of one z = M^-1 r after node `dep` (nullptr: first
// in the graph), in graph g; *last gets the final node.  mode as SsorArgs.
int add_ssor(bfm_gpu_problem* P, cudaGraph_t g, cudaGraphNode_t* last, const cudaGraphNode_t* dep, SsorArgs base, int vt,
             int mode) {
	int const nc = P->ncol > 0 ? P->ncol : 1;
	if (coarse_pc(P->precond) && P->coarse_ok && fuse_coarse(P)) {
		// two-level, fused: the persistent sweep kernel runs the coarse stages
		base.fuse = 1;
		base.co = coarse_args(P, base.r, vt);
		base.agg = P->agg;
		base.pnode = P->pnode;
		base.yc = P->yc;
	}
	else if (coarse_pc(P->precond) && P->coarse_ok) {
		// two-level: yc = A_c^-1 P^T r first; the sweeps add P yc to z
		CoarseArgs ca = coarse_args(P, base.r, vt);
		void* pc[1] = {&ca};
		static_assert(CX_T == TPB, "graph kernel nodes run TPB threads per block");
		bool one = false;
		if (P->ssor_grid > 0 && coarse_apply_grid(P) > 0) {
			// one cooperative launch for the whole correction
			cudaGraphNode_t n;
			if (add_node(g, &n, dep, (void*) k_coarse_apply, P->coarse_grid, pc)) return -1;
			cudaLaunchAttributeValue v;
			memset(&v, 0, sizeof v);
			v.cooperative = 1;
			if (cudaGraphKernelNodeSetAttribute(n, cudaLaunchAttributeCooperative, &v) == cudaSuccess) {
				*last = n;
				one = true;
			}
			else {
				cudaGetLastError();
				cudaGraphDestroyNode(n);
				P->coarse_grid = -1;
			}
		}
		if (!one) {
			cudaGraphNode_t n1, n2, n3, n4;
			if (add_node(g, &n1, dep, (void*) k_restrict, blocks_for(32l * P->nchunk), pc)) return -1;
			if (add_node(g, &n2, &n1, (void*) k_restrict_sum, blocks_for(P->nc), pc)) return -1;
			if (add_node(g, &n3, &n2, (void*) k_coarse_x, P->nc, pc)) return -1;
			if (add_node(g, &n4, &n3, (void*) k_coarse_xt, P->nc, pc)) return -1;
			*last = n4;
		}
		dep = last;
		base.agg = P->agg;
		base.pnode = P->pnode;
		base.yc = P->yc;
	}
	if (P->tma_grid > 0) {
		// one cooperative launch, operands staged by TMA
		SsorArgs a = base;
		a.ncol = nc;
		for (int c = 0; c <= nc && c < 65; c++) a.off[c] = P->ncol > 0 ? P->col_off[c] : 0;
		a.bar = P->ssor_bar;
		a.first_acc = 1;
		a.final_phase = 1;
		a.mode = mode;
		size_t const smem = tma_tiling(P, a, a.fuse);
		if (smem > 0) {
			void* pa[1] = {&a};
			cudaGraphNode_t n;
			if (add_node(g, &n, dep, ssor_tma_kernel(vt), P->tma_grid, pa, smem, ST_THREADS)) return -1;
			cudaLaunchAttributeValue v;
			memset(&v, 0, sizeof v);
			v.cooperative = 1;
			if (cudaGraphKernelNodeSetAttribute(n, cudaLaunchAttributeCooperative, &v) == cudaSuccess) {
				*last = n;
				return 0;
			}
			cudaGetLastError();
			cudaGraphDestroyNode(n);
			P->tma_grid = 0;
		}
	}
	if (P->ssor_grid > 0) {
		// one cooperative launch for every phase
		SsorArgs a = base;
		a.ncol = nc;
		for (int c = 0; c <= nc && c < 65; c++) a.off[c] = P->ncol > 0 ? P->col_off[c] : 0;
		char const* e = getenv("BFM_GPU_SSOR_PREFETCH");  // 0: no L2 prefetch of the next phase
		a.pf = !(e && e[0] == '0');
		a.bar = P->ssor_bar;
		a.first_acc = 1;
		a.final_phase = 1;
		a.mode = mode;
		void* pa[1] = {&a};
		cudaGraphNode_t n;
		if (add_node(g, &n, dep, ssor_all_kernel(vt), P->ssor_grid, pa)) return -1;
		cudaLaunchAttributeValue v;
		memset(&v, 0, sizeof v);
		v.cooperative = 1;
		if (cudaGraphKernelNodeSetAttribute(n, cudaLaunchAttributeCooperative, &v) == cudaSuccess) {
			*last = n;
			return 0;
		}
		// no cooperative kernel nodes here: the per-phase kernels instead
		// (and the coarse correction in kernels of its own)
		cudaGetLastError();
		cudaGraphDestroyNode(n);
		P->ssor_grid = 0;
		if (base.fuse) {
			base.fuse = 0;
			base.yc = nullptr;
			return add_ssor(P, g, last, dep, base, vt, mode);
		}
	}
	void* fwd = ssor_fwd_kernel(vt);
	void* bwd = ssor_bwd_kernel(vt);
	const cudaGraphNode_t* d = dep;
	cudaGraphNode_t n;
	for (int ph = 0; ph < 2 * nc - 1; ph++) {
		SsorArgs a = base;
		bool const forward = ph < nc;
		int const c = forward ? ph : 2 * nc - 2 - ph;
		a.lo = P->col_off[c];
		a.hi_row = P->col_off[c + 1];
		a.slice0 = P->sl_base[c];
		a.fwd_last = forward && c == nc - 1;
		a.first_acc = a.fwd_last;
		a.final_phase = ph == 2 * nc - 2;
		a.mode = mode;
		void* pa[1] = {&a};
		if (add_node(g, &n, d, forward ? fwd : bwd, P->grid, pa)) return -1;
		*last = n;
		d = last;
	}
	return 0;
}

// FP64:  init -> while(running){ A ; B } -> true residual
// mixed: init -> while(running){ K1 ; K2 ; if(replace){R} ; K1' ; K2' ; if(replace'){R'} } -> true residual
//        (two iterations per body pass, so each node has fixed ping-pong direction buffers)
int build_graph(bfm_gpu_problem* P, const bfm_gpu_opts_t* o) {
	bool const mixed = P->precision == BFM_GPU_MIXED || P->precision == BFM_GPU_MIXED_EXACT;
	CgKernels const K = kernels_lpr(P->lpr);
	cudaGraph_t g, body;
	CK(cudaGraphCreate(&g, 0));
	cudaGraphConditionalHandle h;
	CK(cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault));
	cudaGraphNode_t n_init, n_loop, n_res, prev = nullptr;
	int imixed = mixed;
	if (P->precision == BFM_GPU_FP64_DF) {
		// double-float iterations to DF_SWITCH x rtol, then FP64 iterations from the same state
		bfm_gpu_opts_t od = *o;
		od.rtol = o->rtol * DF_SWITCH < 1.0 ? o->rtol * DF_SWITCH : 1.0;
		bool const ssor = ssor_pc(P->precond);
		DfArgs a[2];
		a[0] = df_args(P, &od);
		a[0].use_cond = 1;
		a[0].cond = h;
		a[0].no_pc = ssor;
		a[1] = a[0];
		a[1].p = a[0].s;
		a[1].s = a[0].p;
		CgArgs<double> b[2];
		b[0] = cg_args<double>(P, o);
		CK(cudaGraphConditionalHandleCreate(&b[0].cond, g, 0u, cudaGraphCondAssignDefault));
		b[0].use_cond = 1;
		b[0].no_pc = ssor;
		b[1] = b[0];
		b[1].p = b[0].pn;
		b[1].pn = b[0].p;
		CgKernels const K64 = kernels_lpr(1001);
		SsorArgs sa = ssor_args(P, a[0].r, a[0].u);
		sa.use_cond = 1;
		sa.cond = h;
		void* pi[1] = {&a[0]};
		if (add_node(g, &n_init, nullptr, (void*) k_df_init, P->grid, pi)) return -1;
		if (ssor && add_ssor(P, g, &n_init, &n_init, sa, VT_DF, 1)) return -1;
		if (add_conditional(g, &n_loop, &n_init, h, cudaGraphCondTypeWhile, &body)) return -1;
		for (int half = 0; half < 2; half++) {
			CK(cudaGraphConditionalHandleCreate(&a[half].cond_repl, body, 0u, cudaGraphCondAssignDefault));
			void* pa[1] = {&a[half]};
			cudaGraphNode_t n1, n2, nif, nr;
			cudaGraph_t ifbody;
			if (shape_split(P->lpr)) {
				cudaGraphNode_t n0;
				if (add_node(body, &n0, prev ? &prev : nullptr, (void*) k_hsdf_dir, P->grid, pa)) return -1;
				if (add_node(body, &n1, &n0, K.hsdfs, P->grid, pa)) return -1;
			}
			else if (add_node(body, &n1, prev ? &prev : nullptr, K.hsdf, P->grid, pa)) return -1;
			if (add_node(body, &n2, &n1, (void*) k_hsdf_update, P->grid, pa)) return -1;
			SsorArgs sh = sa;
			sh.cond_repl = a[half].cond_repl;
			if (ssor && add_ssor(P, body, &n2, &n2, sh, VT_DF, 0)) return -1;
			if (add_conditional(body, &nif, &n2, a[half].cond_repl, cudaGraphCondTypeIf, &ifbody)) return -1;
			cudaGraphNode_t nf;
			if (add_node(ifbody, &nf, nullptr, (void*) k_df_flush, P->grid, pa)) return -1;
			if (add_node(ifbody, &nr, &nf, K.hsdfrepl, P->grid, pa)) return -1;
			if (ssor && add_ssor(P, ifbody, &nr, &nr, sh, VT_DF, 1)) return -1;
			prev = nif;
		}
		cudaGraphNode_t n_fin, n_sw, n_loop2;
		if (add_node(g, &n_fin, &n_loop, (void*) k_df_flush, P->grid, pi)) return -1;
		// half 0 of the double-float loop writes its direction into a[0].s, half 1 into a[1].s
		const float* dir_a = a[0].s;
		const float* dir_b = a[1].s;
		double rtol_final = o->rtol;
		void* ps[4] = {&b[0], &dir_a, &dir_b, &rtol_final};
		if (add_node(g, &n_sw, &n_fin, (void*) k_df_switch, P->grid, ps)) return -1;
		SsorArgs sb = ssor_args(P, b[0].r, b[0].u);
		sb.use_cond = 1;
		sb.cond = b[0].cond;
		if (ssor && add_ssor(P, g, &n_sw, &n_sw, sb, VT_F64, 1)) return -1;
		cudaGraph_t body2;
		if (add_conditional(g, &n_loop2, &n_sw, b[0].cond, cudaGraphCondTypeWhile, &body2)) return -1;
		cudaGraphNode_t prev2 = nullptr;
		for (int half = 0; half < 2; half++) {
			CK(cudaGraphConditionalHandleCreate(&b[half].cond_repl, body2, 0u, cudaGraphCondAssignDefault));
			void* pa[1] = {&b[half]};
			cudaGraphNode_t n0, n1, n2, nif, nr;
			cudaGraph_t ifbody;
			if (add_node(body2, &n0, prev2 ? &prev2 : nullptr, (void*) k_hs64_dir, P->grid, pa)) return -1;
			if (add_node(body2, &n1, &n0, K64.hs64s, P->grid, pa)) return -1;
			if (add_node(body2, &n2, &n1, (void*) k_hs64_update, P->grid, pa)) return -1;
			SsorArgs sh = sb;
			sh.cond_repl = b[half].cond_repl;
			if (ssor && add_ssor(P, body2, &n2, &n2, sh, VT_F64, 0)) return -1;
			if (add_conditional(body2, &nif, &n2, b[half].cond_repl, cudaGraphCondTypeIf, &ifbody)) return -1;
			if (add_node(ifbody, &nr, nullptr, K64.hs64repl, P->grid, pa)) return -1;
			if (ssor && add_ssor(P, ifbody, &nr, &nr, sh, VT_F64, 1)) return -1;
			prev2 = nif;
		}
		void* pr[1] = {&b[0]};
		if (add_node(g, &n_res, &n_loop2, K.res64, P->grid, pr)) return -1;
	}
	else if (!mixed) {
		bool const ssor = ssor_pc(P->precond);
		CgArgs<double> a[2];
		a[0] = cg_args<double>(P, o);
		a[0].use_cond = 1;
		a[0].cond = h;
		a[0].no_pc = ssor;
		a[1] = a[0];
		a[1].p = a[0].pn;
		a[1].pn = a[0].p;
		SsorArgs sa = ssor_args(P, a[0].r, a[0].u);
		sa.use_cond = 1;
		sa.cond = h;
		void* pi[2] = {&a[0], &imixed};
		if (add_node(g, &n_init, nullptr, (void*) k_cg_init<double>, P->grid, pi)) return -1;
		if (ssor && add_ssor(P, g, &n_init, &n_init, sa, VT_F64, 1)) return -1;
		if (add_conditional(g, &n_loop, &n_init, h, cudaGraphCondTypeWhile, &body)) return -1;
		for (int half = 0; half < 2; half++) {
			CK(cudaGraphConditionalHandleCreate(&a[half].cond_repl, body, 0u, cudaGraphCondAssignDefault));
			void* pa[1] = {&a[half]};
			cudaGraphNode_t n1, n2, nif, nr;
			cudaGraph_t ifbody;
			if (shape_split(P->lpr)) {
				cudaGraphNode_t n0;
				if (add_node(body, &n0, prev ? &prev : nullptr, (void*) k_hs64_dir, P->grid, pa)) return -1;
				if (add_node(body, &n1, &n0, K.hs64s, P->grid, pa)) return -1;
			}
			else if (add_node(body, &n1, prev ? &prev : nullptr, K.hs64, P->grid, pa)) return -1;
			if (add_node(body, &n2, &n1, (void*) k_hs64_update, P->grid, pa)) return -1;
			SsorArgs sh = sa;
			sh.cond_repl = a[half].cond_repl;
			if (ssor && add_ssor(P, body, &n2, &n2, sh, VT_F64, 0)) return -1;
			if (add_conditional(body, &nif, &n2, a[half].cond_repl, cudaGraphCondTypeIf, &ifbody)) return -1;
			if (add_node(ifbody, &nr, nullptr, K.hs64repl, P->grid, pa)) return -1;
			if (ssor && add_ssor(P, ifbody, &nr, &nr, sh, VT_F64, 1)) return -1;
			prev = nif;
		}
		void* pa[1] = {&a[0]};
		if (add_node(g, &n_res, &n_loop, K.res64, P->grid, pa)) return -1;
	}
	else {
		// mixed: FP32 operator and vectors, FP64 dots; each replacement is an
		// FP64 iterative-refinement step (x += dx, r = b - A x in FP64)
		bool const ssor = ssor_pc(P->precond);
		CgArgs<float> a[2];
		a[0] = cg_args<float>(P, o);
		a[0].use_cond = 1;
		a[0].cond = h;
		a[0].no_pc = ssor;
		a[1] = a[0];
		a[1].p = a[0].pn;
		a[1].pn = a[0].p;
		SsorArgs sa = ssor_args(P, a[0].r, a[0].z);
		sa.use_cond = 1;
		sa.cond = h;
		void* pi[2] = {&a[0], &imixed};
		if (add_node(g, &n_init, nullptr, (void*) k_cg_init<float>, P->grid, pi)) return -1;
		if (ssor && add_ssor(P, g, &n_init, &n_init, sa, VT_F32, 1)) return -1;
		if (add_conditional(g, &n_loop, &n_init, h, cudaGraphCondTypeWhile, &body)) return -1;
		for (int half = 0; half < 2; half++) {
			CK(cudaGraphConditionalHandleCreate(&a[half].cond_repl, body, 0u, cudaGraphCondAssignDefault));
			void* pa[1] = {&a[half]};
			cudaGraphNode_t n1, n2, nif, nr;
			cudaGraph_t ifbody;
			if (add_node(body, &n1, prev ? &prev : nullptr, K.spmvmx, P->grid, pa)) return -1;
			if (add_node(body, &n2, &n1, (void*) k_mx_update, P->grid, pa)) return -1;
			SsorArgs sh = sa;
			sh.cond_repl = a[half].cond_repl;
			if (ssor && add_ssor(P, body, &n2, &n2, sh, VT_F32, 0)) return -1;
			if (add_conditional(body, &nif, &n2, a[half].cond_repl, cudaGraphCondTypeIf, &ifbody)) return -1;
			cudaGraphNode_t nf;
			if (add_node(ifbody, &nf, nullptr, (void*) k_mx_flush, P->grid, pa)) return -1;
			if (add_node(ifbody, &nr, &nf, K.replace, P->grid, pa)) return -1;
			if (ssor && add_ssor(P, ifbody, &nr, &nr, sh, VT_F32, 1)) return -1;
			prev = nif;
		}
		void* pa[1] = {&a[0]};
		cudaGraphNode_t n_flush;
		if (add_node(g, &n_flush, &n_loop, (void*) k_mx_flush, P->grid, pa)) return -1;
		if (add_node(g, &n_res, &n_flush, K.resmx, P->grid, pa)) return -1;
	}
	if (P->graph) cudaGraphExecDestroy(P->graph);
	P->graph = nullptr;
	CK(cudaGraphInstantiate(&P->graph, g, 0));
	cudaGraphDestroy(g);
	return 0;
}

// Mean duration (ms) of the two per-iteration steps with SpMV shape `lpr`
// (the SpMV step includes the direction kernel of the split form), launched
// standalone on a scratch solver state.  Overwrites the Krylov vectors.
int time_iteration(bfm_gpu_problem* P, int lpr, int reps, double* ms_spmv, double* ms_update) {
	CgState* scratch = nullptr;
	if (dalloc(&scratch, 1)) return -1;
	CgKernels const K = kernels_lpr(lpr);
	cudaEvent_t e[3];
	for (auto& x : e) cudaEventCreate(&x);
	int const grid = P->grid;
	cudaStream_t const st = P->stream;
	if (P->precision == BFM_GPU_FP64_DF) {
		DfArgs a = df_args(P, nullptr);
		a.opts.rtol = 0.0;
		a.opts.max_iters = 1 << 30;
		a.st = scratch;
		a.timing = 1;
		k_df_init<<<grid, TPB, 0, st>>>(a);
		void* pa[1] = {&a};
		cudaEventRecord(e[0], st);
		for (int i = 0; i < reps; i++) {
			if (shape_split(lpr)) {
				k_hsdf_dir<<<grid, TPB, 0, st>>>(a);
				cudaLaunchKernel(K.hsdfs, dim3(grid), dim3(TPB), pa, 0, st);
			}
			else cudaLaunchKernel(K.hsdf, dim3(grid), dim3(TPB), pa, 0, st);
		}
		cudaEventRecord(e[1], st);
		for (int i = 0; i < reps; i++) k_hsdf_update<<<grid, TPB, 0, st>>>(a);
		cudaEventRecord(e[2], st);
	}
	else if (P->precision == BFM_GPU_FP64) {
		CgArgs<double> a = cg_args<double>(P, nullptr);
		a.opts.rtol = 0.0;
		a.opts.max_iters = 1 << 30;
		a.st = scratch;
		a.timing = 1;
		k_cg_init<double><<<grid, TPB, 0, st>>>(a, 0);
		void* pa[1] = {&a};
		cudaEventRecord(e[0], st);
		for (int i = 0; i < reps; i++) {
			if (shape_split(lpr)) {
				k_hs64_dir<<<grid, TPB, 0, st>>>(a);
				cudaLaunchKernel(K.hs64s, dim3(grid), dim3(TPB), pa, 0, st);
			}
			else cudaLaunchKernel(K.hs64, dim3(grid), dim3(TPB), pa, 0, st);
		}
		cudaEventRecord(e[1], st);
		for (int i = 0; i < reps; i++) k_hs64_update<<<grid, TPB, 0, st>>>(a);
		cudaEventRecord(e[2], st);
	}
	else {
		CgArgs<float> a = cg_args<float>(P, nullptr);
		a.opts.rtol = 0.0;
		a.opts.max_iters = 1 << 30;
		a.st = scratch;
		a.timing = 1;
		k_cg_init<float><<<grid, TPB, 0, st>>>(a, 1);
		void* pa[1] = {&a};
		cudaEventRecord(e[0], st);
		for (int i = 0; i < reps; i++) cudaLaunchKernel(K.spmvmx, dim3(grid), dim3(TPB), pa, 0, st);
		cudaEventRecord(e[1], st);
		for (int i = 0; i < reps; i++) k_mx_update<<<grid, TPB, 0, st>>>(a);
		cudaEventRecord(e[2], st);
	}
	cudaError_t const err = cudaStreamSynchronize(st);
	float t1 = 0, t2 = 0;
	cudaEventElapsedTime(&t1, e[0], e[1]);
	cudaEventElapsedTime(&t2, e[1], e[2]);
	for (auto& x : e) cudaEventDestroy(x);
	cudaFree(scratch);
	CK(err);
	*ms_spmv = t1 / reps;
	*ms_update = t2 / reps;
	return 0;
}

// Mean duration (ms) of one SSOR application z = M^-1 r (every sweep phase),
// launched standalone on a scratch solver state.  Overwrites the Krylov vectors.
int time_ssor(bfm_gpu_problem* P, int reps, double* ms, double* ms_sweeps) {
	if (!ssor_pc(P->precond)) return fail("time the SSOR sweeps of a problem solved with an SSOR preconditioner");
	CgState* scratch = nullptr;
	if (dalloc(&scratch, 1)) return -1;
	cudaStream_t const st = P->stream;
	CK(cudaMemsetAsync(scratch, 0, sizeof(CgState), st));
	int const vt = precision_vt(P->precision);
	SsorArgs base = ssor_args(P, P->vec[0], P->vec[1]);
	base.st = scratch;
	base.timing = 1;
	int const nc = P->ncol > 0 ? P->ncol : 1;
	cudaEvent_t e[2];
	for (auto& x : e) cudaEventCreate(&x);
	CoarseArgs ca = coarse_args(P, P->vec[0], vt);
	ca.berr = &scratch->ssor_err;
	bool const coarse = coarse_pc(P->precond) && P->coarse_ok;
	if (coarse) {
		base.agg = P->agg;
		base.pnode = P->pnode;
		base.yc = P->yc;
	}
	bool const fused = coarse && fuse_coarse(P);
	auto once = [&](bool with_coarse) {
		if (coarse && with_coarse && !fused) {
			if (P->ssor_grid > 0 && coarse_apply_grid(P) > 0) {
				void* pa[1] = {&ca};
				cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), st);
				cudaLaunchCooperativeKernel((const void*) k_coarse_apply, dim3(P->coarse_grid), dim3(CX_T), pa, 0, st);
			}
			else {
				k_restrict<<<blocks_for(32l * P->nchunk), TPB, 0, st>>>(ca);
				k_restrict_sum<<<blocks_for(P->nc), TPB, 0, st>>>(ca);
				k_coarse_x<<<P->nc, CX_T, 0, st>>>(ca);
				k_coarse_xt<<<P->nc, CX_T, 0, st>>>(ca);
			}
		}
		if (P->tma_grid > 0) {
			SsorArgs a = base;
			a.ncol = nc;
			for (int c = 0; c <= nc && c < 65; c++) a.off[c] = P->ncol > 0 ? P->col_off[c] : 0;
			a.bar = P->ssor_bar;
			a.first_acc = a.final_phase = 1;
			if (fused && with_coarse) {
				a.fuse = 1;
				a.co = ca;
			}
			size_t const smem = tma_tiling(P, a, a.fuse);
			if (smem > 0) {
				void* pa[1] = {&a};
				cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), st);
				cudaLaunchCooperativeKernel(ssor_tma_kernel(vt), dim3(P->tma_grid), dim3(ST_THREADS), pa, smem, st);
				return;
			}
		}
		if (P->ssor_grid > 0) {
			SsorArgs a = base;
			a.ncol = nc;
			for (int c = 0; c <= nc && c < 65; c++) a.off[c] = P->ncol > 0 ? P->col_off[c] : 0;
			a.bar = P->ssor_bar;
			a.first_acc = a.final_phase = 1;
			if (fused && with_coarse) {
				a.fuse = 1;
				a.co = ca;
			}
			void* pa[1] = {&a};
			cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), st);
			cudaLaunchCooperativeKernel(ssor_all_kernel(vt), dim3(P->ssor_grid),
			                            dim3(TPB), pa, 0, st);
			return;
		}
		for (int ph = 0; ph < 2 * nc - 1; ph++) {
			SsorArgs a = base;
			bool const forward = ph < nc;
			int const c = forward ? ph : 2 * nc - 2 - ph;
			a.lo = P->col_off[c];
			a.hi_row = P->col_off[c + 1];
			a.slice0 = P->sl_base[c];
			a.fwd_last = forward && c == nc - 1;
			a.first_acc = a.fwd_last;
			a.final_phase = ph == 2 * nc - 2;
			void* pa[1] = {&a};
			cudaLaunchKernel(forward ? ssor_fwd_kernel(vt) : ssor_bwd_kernel(vt),
			                 dim3(P->grid), dim3(TPB), pa, 0, st);
		}
	};
	once(true);
	cudaEventRecord(e[0], st);
	for (int i = 0; i < reps; i++) once(true);
	cudaEventRecord(e[1], st);
	cudaError_t err = cudaStreamSynchronize(st);
	float t = 0;
	cudaEventElapsedTime(&t, e[0], e[1]);
	if (ms_sweeps && err == cudaSuccess) {
		// the sweeps alone (the coarse correction's yc from the last application)
		cudaEventRecord(e[0], st);
		for (int i = 0; i < reps; i++) once(false);
		cudaEventRecord(e[1], st);
		err = cudaStreamSynchronize(st);
		float t2 = 0;
		cudaEventElapsedTime(&t2, e[0], e[1]);
		*ms_sweeps = t2 / reps;
	}
	for (auto& x : e) cudaEventDestroy(x);
	cudaFree(scratch);
	CK(err);
	*ms = t / reps;
	return 0;
}

// Project autotuner: time every SpMV shape (lanes per block row, blocks in
// flight per lane, split or fused direction) on this problem's matrix, 20
// launches each, and keep the fastest.
int autotune_lpr(bfm_gpu_problem* P) {
	BFM_RANGE("autotune_lpr");
	double best = 1e30;
	int best_lpr = 8;
	bool const mixed = P->precision == BFM_GPU_MIXED || P->precision == BFM_GPU_MIXED_EXACT;
	for (int lpr : SHAPES) {
		if (mixed && shape_split(lpr)) continue;  // the mixed path has no split form
		double t_spmv = 0, t_upd = 0;
		if (time_iteration(P, lpr, 20, &t_spmv, &t_upd)) return -1;
		if (t_spmv < best) {
			best = t_spmv;
			best_lpr = lpr;
		}
	}
	P->lpr = best_lpr;
	return 0;
}

}  // namespace

extern "C" {

const char* bfm_gpu_last_error(void) { return g_err; }

void bfm_gpu_set_last_error(const char* msg) { snprintf(g_err, sizeof g_err, "%s", msg); }

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
	o->replace_drop = 1e-1;
	o->deterministic = 1;
	o->autotune = 1;
	o->barrier_polls = 0;
	o->refine_restart = 0;
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
	P->polls = BARRIER_POLLS_DEFAULT;
	P->lpr = 8;
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
	// persistent-style grids for the Krylov kernels: as many blocks as stay
	// resident on every SM at once (occupancy of the most demanding one)
	int const sms = num_sms();
	int occ = 8;
	void* const ks[] = {(void*) k_cg64_spmv<1>, (void*) k_cg64_spmv<8>, (void*) k_mx_spmv<1>, (void*) k_mx_spmv<8>,
	                    (void*) k_cg64_update, (void*) k_mx_update, (void*) k_mx_replace<8>, (void*) k_hs64_spmv<1>,
	                    (void*) k_hs64_spmv<8>,
	                    (void*) k_hs64_update, (void*) k_hsdf_spmv<1>, (void*) k_hsdf_spmv<8>, (void*) k_hsdf_update};
	for (void* k : ks) {
		int nb = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, TPB, 0) == cudaSuccess && nb > 0 && nb < occ) occ = nb;
	}
	cudaGetLastError();
	P->grid = sms * occ;
	long const N = n_nodes, E = n_elems;
	long const inc_total = E * kind;
	P->nb_cap = inc_total * kind > N ? inc_total * kind : N;
	long const tiles = (N + SCAN_TILE) / SCAN_TILE + 1;
	*out = P;
	if (dalloc(&P->coords, 2 * N) || dalloc(&P->elems, inc_total) || dalloc(&P->masks, (long) (n_conds ? n_conds : 1) * N) ||
	    dalloc(&P->edges, 2l * n_edges) || dalloc(&P->eboundary, n_edges) || dalloc(&P->cnt, N + 1) || dalloc(&P->inc_ptr, N + 1) || dalloc(&P->inc, inc_total) ||
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
	if (cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking) != cudaSuccess ||
	    cudaEventCreateWithFlags(&P->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
	    cudaEventCreateWithFlags(&P->join_ev, cudaEventDisableTiming) != cudaSuccess) {
		cudaGetLastError();
		if (P->side) cudaStreamDestroy(P->side);
		P->side = nullptr;  // the coarse set-up then runs on the problem's stream
	}
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
	void* bufs[] = {P->coords, P->elems, P->elemE, P->elemNu, P->masks, P->edges, P->eboundary, P->cnt, P->inc_ptr, P->inc, P->cand,
	                P->row_len, P->row_ptr, P->cols, P->ecnt, P->eptr, P->elist, P->scan_sums, P->scan_total, P->vals64,
	                P->vals32, P->corr32, P->vals32lo, P->srow_df, P->coords32, P->mat32, P->egrad, P->b, P->last_ci, P->first, P->last, P->dinv64, P->dinv32, P->x, P->vec[0], P->vec[1], P->vec[2], P->vec[3], P->vec[4], P->vec[5],
	                P->partials, P->ticket, P->st, P->err};
	for (void* p : bufs)
		if (p) cudaFree(p);
	for (int i = 0; i < MAXF; i++)
		if (P->force_fields[i]) cudaFree(P->force_fields[i]);
	void* lb[] = {P->ledges, P->lloads, P->lcnt, P->lptr, P->llist, P->perm, P->iperm, P->dpos, P->otmp, P->ssor_y, P->ssor_d,
	              P->e64, P->e64_bad,
	              P->ssor_bar, P->agg, P->agg_ptr, P->agg_nodes, P->pnode, P->aband, P->diag0, P->rc, P->yc,
	              P->ayt, P->xl, P->xu, P->coarse_err, P->chunk_start, P->chunk_agg, P->agg_chunk, P->cpart,
	              P->sl_lw, P->sl_uw, P->sl_lp, P->sl_up, P->sl_lv, P->sl_uv, P->sl_lc, P->sl_uc, P->sl_wm, P->tri, P->lbm, P->lbd,
	              P->lbw};
	for (void* q : lb)
		if (q) cudaFree(q);
	if (P->ext && P->ext_free) P->ext_free(P->ext);
	if (P->st_host) cudaFreeHost(P->st_host);
	if (P->err_host) cudaFreeHost(P->err_host);
	for (int i = 0; i < 4; i++)
		if (P->ev[i]) cudaEventDestroy(P->ev[i]);
	if (P->fork_ev) cudaEventDestroy(P->fork_ev);
	if (P->join_ev) cudaEventDestroy(P->join_ev);
	if (P->side) cudaStreamDestroy(P->side);
	if (P->own_stream && P->stream) cudaStreamDestroy(P->stream);
	free(P);
	return 0;
}

void* bfm_gpu_problem_stream(bfm_gpu_problem_t* P) { return (void*) P->stream; }

static cudaMemcpyKind kind_of(int where) { return where == BFM_GPU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }

int bfmi_set_geometry_u64(bfm_gpu_problem_t* P, const double* coords, const uint64_t* elems, long* bad_index) {
	P->inputs_gen++;
	g_err[0] = 0;
	*bad_index = -1;
	long const n = (long) P->NE * P->kind;
	cudaStream_t const st = P->stream;
	if (!P->e64 && dalloc(&P->e64, n > 0 ? n : 1)) return -1;
	if (!P->e64_bad && dalloc(&P->e64_bad, 1)) return -1;
	CK(cudaMemcpyAsync(P->coords, coords, 2l * P->N * sizeof(double), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(P->e64, elems, n * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
	CK(cudaMemsetAsync(P->e64_bad, 0xff, sizeof(unsigned long long), st));
	if (n > 0) k_elems_from_u64<<<blocks_for(n), TPB, 0, st>>>(n, P->N, P->e64, P->elems, P->e64_bad);
	CK(cudaGetLastError());
	unsigned long long bad = 0;
	CK(cudaMemcpyAsync(&bad, P->e64_bad, sizeof bad, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (bad != ~0ull) *bad_index = (long) bad;
	P->ordered &= ~(ORD_COORDS | ORD_ELEMS);
	P->colored = false;
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_geometry(bfm_gpu_problem_t* P, const double* coords, const int32_t* elems, int where) {
	P->inputs_gen++;
	g_err[0] = 0;
	CK(cudaMemcpyAsync(P->coords, coords, 2l * P->N * sizeof(double), kind_of(where), P->stream));
	CK(cudaMemcpyAsync(P->elems, elems, (long) P->NE * P->kind * sizeof(int), kind_of(where), P->stream));
	P->ordered &= ~(ORD_COORDS | ORD_ELEMS);
	P->colored = false;
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_material(bfm_gpu_problem_t* P, double E, double nu, double rho, int stress, const double* elem_E,
                                 const double* elem_nu, int where) {
	P->inputs_gen++;
	g_err[0] = 0;
	if (stress < 0 || stress > 3) return fail("element formulation %d is not one of 0..3", stress);
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
	P->inputs_gen++;
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
	P->inputs_gen++;
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
	// every field in use now holds the caller's order
	P->ordered &= ~ORD_FIELDS;
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_conditions(bfm_gpu_problem_t* P, int n_conds, const int* kinds, const double* values, const uint8_t* masks,
                                   int n_edges, const int32_t* edges, int where) {
	P->inputs_gen++;
	g_err[0] = 0;
	if (n_conds > P->max_conds || n_conds < 0) return fail("more conditions than the problem was created for");
	if (n_edges > P->max_edges || n_edges < 0) return fail("more edges than the problem was created for");
	for (int c = 0; c < n_conds; c++) {
		int const k = kinds[c];
		if (k < BFM_CONDITION_KIND_DIRICHLET_X || k > BFM_CONDITION_KIND_DIRICHLET_TANGENT)
			return fail("unknown condition kind %d", k);
		P->kinds[c] = k;
		P->values[c] = values[c];
	}
	P->n_conds = n_conds;
	P->n_edges = n_edges;
	if (n_conds) CK(cudaMemcpyAsync(P->masks, masks, (long) n_conds * P->N, kind_of(where), P->stream));
	if (n_edges) CK(cudaMemcpyAsync(P->edges, edges, 2l * n_edges * sizeof(int), kind_of(where), P->stream));
	// every edge counts as a boundary edge until bfm_gpu_problem_set_edge_boundary says otherwise
	if (n_edges) CK(cudaMemsetAsync(P->eboundary, 1, n_edges, P->stream));
	P->ordered &= ~(ORD_MASKS | ORD_EDGES);
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_edge_boundary(bfm_gpu_problem_t* P, const uint8_t* boundary, int where) {
	P->inputs_gen++;
	g_err[0] = 0;
	if (P->n_edges) CK(cudaMemcpyAsync(P->eboundary, boundary, P->n_edges, kind_of(where), P->stream));
	P->assembled = false;
	return 0;
}

int bfm_gpu_problem_set_edge_loads(bfm_gpu_problem_t* P, int n_loads, const int32_t* edges, const double* loads, int where) {
	P->inputs_gen++;
	g_err[0] = 0;
	if (n_loads < 0) return fail("negative load count");
	if (n_loads > P->cap_loads) {
		void* lb[] = {P->ledges, P->lloads, P->lcnt, P->lptr, P->llist};
		for (void* q : lb)
			if (q) cudaFree(q);
		P->ledges = P->lcnt = P->lptr = P->llist = nullptr;
		P->lloads = nullptr;
		P->cap_loads = 0;
		if (dalloc(&P->ledges, 2l * n_loads) || dalloc(&P->lloads, 2l * n_loads) || dalloc(&P->lcnt, P->N + 1l) ||
		    dalloc(&P->lptr, P->N + 1l) || dalloc(&P->llist, 2l * n_loads))
			return -1;
		P->cap_loads = n_loads;
	}
	P->n_loads = n_loads;
	if (n_loads) {
		CK(cudaMemcpyAsync(P->ledges, edges, 2l * n_loads * sizeof(int), kind_of(where), P->stream));
		CK(cudaMemcpyAsync(P->lloads, loads, 2l * n_loads * sizeof(double), kind_of(where), P->stream));
	}
	P->ordered &= ~ORD_LEDGES;
	P->assembled = false;
	return 0;
}

int bfmi_buffers(bfm_gpu_problem_t* P, bfmi_buffers_t* o) {
	memset(o, 0, sizeof *o);
	o->N = P->N;
	o->n_elems = P->NE;
	o->kind = P->kind;
	o->precision = P->precision;
	o->precond = P->precond;
	o->assembled = P->assembled;
	o->grid = P->grid;
	o->row_ptr = P->row_ptr;
	o->cols = P->cols;
	o->vals32 = P->vals32;
	o->corr32 = P->corr32;
	o->dinv32 = P->dinv32;
	o->vals64 = P->precision == BFM_GPU_MIXED_EXACT || P->precision == BFM_GPU_FP64 ? P->vals64 : nullptr;
	o->vals64_any = P->precision != BFM_GPU_MIXED ? P->vals64 : nullptr;
	o->dinv64 = P->dinv64;
	o->b = P->b;
	o->x = P->x;
	for (int i = 0; i < 5; i++) o->vec[i] = P->vec[i];
	o->stream = (void*) P->stream;
	o->inputs_gen = P->inputs_gen;
	if (P->ordered) {
		o->ncol = P->ncol;
		for (int c = 0; c <= P->ncol && c < 65; c++) o->col_off[c] = P->col_off[c];
		o->dpos = P->dpos;
	}
	return 0;
}

int bfmi_set_precond(bfm_gpu_problem_t* P, int precond) {
	if (precond != BFM_GPU_PC_JACOBI && precond != BFM_GPU_PC_BLOCK_JACOBI)
		return fail("bfmi_set_precond: Jacobi or block Jacobi only, got %d", precond);
	if (P->precond != precond) {
		P->precond = precond;
		P->assembled = 0;  // the preconditioner is formed by the assembly epilogue
	}
	return 0;
}

void** bfmi_ext_slot(bfm_gpu_problem_t* P, void (**free_fn)(void*)) {
	if (free_fn) P->ext_free = *free_fn;
	return &P->ext;
}

int bfmi_mesh(bfm_gpu_problem_t* P, bfmi_mesh_t* o) {
	memset(o, 0, sizeof *o);
	o->coords = P->coords;
	o->inc_ptr = P->inc_ptr;
	o->inc = P->inc;
	o->elemE = P->has_elemE ? P->elemE : nullptr;
	o->elemNu = P->has_elemNu ? P->elemNu : nullptr;
	o->E = P->E;
	o->nu = P->nu;
	o->last_ci = P->last_ci;
	return 0;
}

int bfmi_solve_rhs(bfm_gpu_problem_t* P, const double* b, double* x, const bfm_gpu_opts_t* opts, int* status, int* iterations,
                   double* rel_residual) {
	g_err[0] = 0;
	bfm_gpu_opts_t o = *opts;
	o.precision = BFM_GPU_FP64;
	// the right-hand side is replaced after the assembly, so the assembly
	// (with this preconditioner, in FP64) comes first
	if (!P->assembled || P->precision != BFM_GPU_FP64 || o.precond != P->precond) {
		P->precond = o.precond;
		if (bfm_gpu_problem_assemble(P, BFM_GPU_FP64)) return -1;
	}
	long const n = 2l * P->N;
	if (P->ordered) {
		// into the working (colour-major) order: b_w[w] = b[perm[w]]
		if (ensure_otmp(P)) return -1;
		CK(cudaMemcpyAsync(P->otmp, b, n * sizeof(double), cudaMemcpyHostToDevice, P->stream));
		k_gather_nodes<double><<<blocks_for(n), TPB, 0, P->stream>>>(P->N, 2, (const double*) P->otmp, P->perm, P->b);
		CK(cudaGetLastError());
	}
	else {
		CK(cudaMemcpyAsync(P->b, b, n * sizeof(double), cudaMemcpyHostToDevice, P->stream));
	}
	if (bfm_gpu_problem_solve(P, &o)) return -1;
	bfm_gpu_stats_t s;
	if (bfm_gpu_problem_stats(P, &s)) return -1;
	if (status) *status = s.status;
	if (iterations) *iterations = s.iterations;
	if (rel_residual) *rel_residual = s.rel_residual;
	return bfm_gpu_problem_solution(P, x, BFM_GPU_HOST);
}

int bfmi_set_precond_blocks(bfm_gpu_problem_t* P, const double* blocks) {
	if (!P->assembled) return fail("assemble before setting the preconditioner");
	// FP64 SSOR sweeps read FP32 relaxation blocks: the double-float layout;
	// the mixed precisions keep FP32 blocks, 4 per node, for every preconditioner
	int const layout = P->precision == BFM_GPU_FP64_DF || (ssor_pc(P->precond) && P->precision == BFM_GPU_FP64) ? 2
	                   : P->precision == BFM_GPU_FP64 ? 0 : 1;
	// without blocks: Jacobi, or block Jacobi as the SSOR relaxation blocks
	k_store_blocks<<<blocks_for(P->N), TPB, 0, P->stream>>>(P->N, blocks, P->row_ptr, P->cols,
	                                                        P->precision != BFM_GPU_MIXED ? P->vals64 : nullptr, P->vals32,
	                                                        layout, ssor_pc(P->precond), P->dinv64, P->dinv32);
	CK(cudaGetLastError());
	return 0;
}

int bfm_gpu_problem_apply(bfm_gpu_problem_t* P, const double* x, double* y, int where) {
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble before applying the operator");
	if (P->precision == BFM_GPU_MIXED) return fail("the FP64 operator is not assembled in the MIXED precision");
	long const n = 2l * P->N;
	const double* dx = x;
	double* dy = y;
	double* tmp = nullptr;
	if (where != BFM_GPU_DEVICE) {
		if (dalloc(&tmp, 2 * n)) return -1;
		CK(cudaMemcpyAsync(tmp, x, n * sizeof(double), cudaMemcpyHostToDevice, P->stream));
		dx = tmp;
		dy = tmp + n;
	}
	k_apply64<<<blocks_for(P->N), TPB, 0, P->stream>>>(P->N, P->row_ptr, P->cols, P->vals64, dx, dy);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess && tmp) {
		e = cudaMemcpyAsync(y, dy, n * sizeof(double), cudaMemcpyDeviceToHost, P->stream);
		if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
	}
	if (tmp) cudaFree(tmp);
	if (e != cudaSuccess) return fail("CUDA error %s in bfm_gpu_problem_apply", cudaGetErrorString(e));
	return 0;
}

int bfm_gpu_problem_assemble(bfm_gpu_problem_t* P, int precision) {
	BFM_RANGE("bfm_gpu_problem_assemble");
	g_err[0] = 0;
	if (precision != BFM_GPU_FP64 && precision != BFM_GPU_MIXED && precision != BFM_GPU_MIXED_EXACT &&
	    precision != BFM_GPU_FP64_DF)
		return fail("unknown precision %d", precision);
	bool const dfp = precision == BFM_GPU_FP64_DF;
	bool const want64 = precision != BFM_GPU_MIXED;  // FP64 values: the operator, or the residual operator
	bool const want32 = precision != BFM_GPU_FP64;   // FP32 values: the mixed iteration operator / hi parts
	// the preconditioner here is the last solve's (every precision has the SSOR ones)
	bool const ssor = ssor_pc(P->precond);
	bool const fp64_ssor = ssor && precision == BFM_GPU_FP64;  // FP32 blocks and relaxation blocks for the sweeps
	cudaStream_t const st = P->stream;
	long const N = P->N;
	// value storage for this precision (allocated once, on first use)
	if (want64 && !P->vals64 && dalloc(&P->vals64, 4 * P->nb_cap)) return -1;
	if ((want32 || fp64_ssor) && !P->vals32 && dalloc(&P->vals32, 4 * P->nb_cap)) return -1;
	if ((!want32 || dfp) && !P->dinv64 && dalloc(&P->dinv64, 4 * N)) return -1;
	if ((want32 || fp64_ssor) && !P->dinv32 && dalloc(&P->dinv32, 8 * N)) return -1;  // up to a double-float 2x2 block per node
	if (want32 && !P->corr32 && dalloc(&P->corr32, 4 * N)) return -1;
	if (dfp && !P->vals32lo && dalloc(&P->vals32lo, 4 * P->nb_cap)) return -1;
	if (dfp && !P->srow_df && dalloc(&P->srow_df, 8 * N)) return -1;
	// 16 bytes per node per vector for FP64 and double-float, 8 for the mixed FP32 vectors
	bool const wide = precision == BFM_GPU_FP64 || dfp;
	size_t const vsz = wide ? sizeof(double) : sizeof(float);
	bool const was_wide = P->precision == BFM_GPU_FP64 || P->precision == BFM_GPU_FP64_DF;
	if (was_wide != wide || !P->vec[0]) {
		for (void*& v : P->vec) {
			if (v) cudaFree(v);
			v = nullptr;
			CK(cudaMalloc(&v, 2 * (N ? N : 1) * vsz));
		}
	}
	// the SpMV shape is tuned per precision (each has its own kernels)
	if (P->precision != precision) P->tuned = 0;
	P->precision = precision;
	// timing events only outside a stream capture (a captured assembly is
	// timed by whoever launches the graph)
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	CK(cudaStreamIsCapturing(st, &cap));
	bool const capturing = cap != cudaStreamCaptureStatusNone;
	if (!capturing) CK(cudaEventRecord(P->ev[0], st));
	CK(cudaMemsetAsync(P->err, 0, sizeof(int), st));
	// 0. node order (colour-major for the SSOR preconditioners)
	if (prepare_order(P)) return -1;
	// 1. node -> element incidence, ascending; 2. node-block pattern
	if (build_pattern(P)) return -1;
	if (ssor_pc(P->precond)) {
		k_diag_pos<<<blocks_for(N), TPB, 0, st>>>(P->N, P->row_ptr, P->cols, P->dpos);
		if (!P->ssor_y && dalloc(&P->ssor_y, 4 * N)) return -1;
		if (!P->ssor_d && dalloc(&P->ssor_d, N)) return -1;
		if (!P->ssor_bar) {
			if (dalloc(&P->ssor_bar, BAR_WORDS)) return -1;
			CK(cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), st));
			// every block of the persistent sweep kernel resident at once
			int nb = 0, dev = 0, coop = 0;
			CK(cudaGetDevice(&dev));
			CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
			// BFM_GPU_SSOR_PER_COLOUR=1: one launch per colour phase, as where the
			// graph cannot hold a cooperative kernel node
			char const* pcol = getenv("BFM_GPU_SSOR_PER_COLOUR");
			if (pcol && pcol[0] == '1') coop = 0;
			if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, ssor_all_kernel(VT_DF), TPB, 0) == cudaSuccess &&
			    nb > 0) {
				// one grid for every vector layout: the fewest resident blocks of the three
				for (int vt : {VT_F64, VT_F32}) {
					int nb2 = 0;
					if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, ssor_all_kernel(vt), TPB, 0) == cudaSuccess &&
					    nb2 > 0 && nb2 < nb)
						nb = nb2;
				}
				P->ssor_grid = num_sms() * nb;
			}
			cudaGetLastError();
			// the TMA-staged sweep kernel: one block of ST_THREADS per SM with
			// (nearly) all of the SM's shared memory (BFM_GPU_SSOR_TMA=0: not used)
			char const* tma = getenv("BFM_GPU_SSOR_TMA");
			int optin = 0;
			P->tma_grid = 0;
			if (coop && !(tma && tma[0] == '0') &&
			    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess) {
				int const smem = optin - 2048;  // the kernel's static shared memory and a margin
				bool ok = smem > 64 * 1024;
				for (void* f : {(void*) k_ssor_tma<VT_F64>, (void*) k_ssor_tma<VT_DF>, (void*) k_ssor_tma<VT_F32>}) {
					int nb2 = 0;
					ok = ok && cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess &&
					     cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb2, f, ST_THREADS, smem) == cudaSuccess && nb2 >= 1;
				}
				if (ok) {
					P->tma_grid = num_sms();
					P->tma_smem_max = smem;
				}
				cudaGetLastError();
			}
		}
	}
	// 3. Dirichlet bookkeeping, conditions in order (node -> edge incidence
	// first when edges are needed: normal/tangent conditions, Neumann loads)
	bool need_edges = false;
	for (int c = 0; c < P->n_conds; c++) need_edges |= P->kinds[c] >= BFM_CONDITION_KIND_NEUMANN_X;
	need_edges = need_edges && P->n_edges > 0;
	if (need_edges && incidence(P, P->edges, P->n_edges, 2, P->ecnt, P->eptr, P->elist, 2 * MAXV, ERR_EDGE_VALENCE)) return -1;
	CK(cudaMemsetAsync(P->last_ci, 0xff, 2 * N * sizeof(int), st));
	for (int c = 0; c < P->n_conds; c++) {
		int const k = P->kinds[c];
		if (k == BFM_CONDITION_KIND_DIRICHLET_X || k == BFM_CONDITION_KIND_DIRICHLET_Y)
			k_dirichlet_mark<<<blocks_for(N), TPB, 0, st>>>(P->N, c, k == BFM_CONDITION_KIND_DIRICHLET_X ? 0 : 1, P->values[c],
			                                                 P->masks + (long) c * N, P->last_ci, P->first, P->last);
		if (k == BFM_CONDITION_KIND_DIRICHLET_NORMAL || k == BFM_CONDITION_KIND_DIRICHLET_TANGENT)
			k_dirichlet_nt_mark<<<blocks_for(N), TPB, 0, st>>>(P->N, c, k == BFM_CONDITION_KIND_DIRICHLET_TANGENT, P->values[c],
			                                                    P->masks + (long) c * N, need_edges ? P->eptr : nullptr,
			                                                    P->elist, P->edges, P->eboundary, P->coords, P->last_ci,
			                                                    P->first, P->last);
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
	a.vals32 = want32 || fp64_ssor ? P->vals32 : nullptr;
	a.corr32 = want32 ? P->corr32 : nullptr;
	a.vals32lo = dfp ? P->vals32lo : nullptr;
	a.srow_df = dfp ? P->srow_df : nullptr;
	a.b = P->b;
	a.dinv64 = want32 && !dfp ? nullptr : P->dinv64;
	a.dinv32 = want32 && !dfp ? P->dinv32 : nullptr;
	a.precond = P->precond;
	a.err = P->err;
	if (precision != BFM_GPU_MIXED || P->stress >= 2) {
		// (the FP32 element integration is planar only: axisymmetric
		// mixed-precision solves round the exact FP64 values)
		bool same_points = P->kind == 3 && P->stress < 2 && P->NE > 0;
		for (int q = 1; q < P->rule.nq; q++) {
			same_points &= P->rule.w[q] == P->rule.w[0];
			for (int j = 0; j < P->kind; j++)
				same_points &= P->rule.dxi[q][j] == P->rule.dxi[0][j] && P->rule.deta[q][j] == P->rule.deta[0][j];
		}
		if (same_points) {
			if (P->NE > P->egrad_cap) {
				if (P->egrad) cudaFree(P->egrad);
				P->egrad = nullptr;
				P->egrad_cap = 0;
				if (dalloc(&P->egrad, 10l * P->NE)) return -1;
				P->egrad_cap = P->NE;
			}
			a.NE = P->NE;
			k_elem_grad<<<blocks_for(P->NE), TPB, 0, st>>>(a, P->egrad);
			a.egrad = P->egrad;
		}
		k_assemble<true><<<blocks_for(N, 128), 128, 0, st>>>(a);
		if (dfp || fp64_ssor) k_df_dinv<<<blocks_for(N), TPB, 0, st>>>(P->N, P->dinv64, P->dinv32, P->precond != BFM_GPU_PC_JACOBI);
	}
	else {
		if (!P->coords32 && dalloc(&P->coords32, N)) return -1;
		k_split_coords<<<blocks_for(N), TPB, 0, st>>>(P->N, P->coords, P->coords32);
		a.coords32 = P->coords32;
		if (a.elemE || a.elemNu) {
			if (!P->mat32 && dalloc(&P->mat32, P->NE)) return -1;
			k_elem_mat32<<<blocks_for(P->NE), TPB, 0, st>>>(P->NE, a.elemE, a.elemNu, P->E, P->nu, P->stress, P->mat32);
			a.mat32 = P->mat32;
		}
		// P1-type rules: every Gauss point has the same shape gradients, so the
		// FP32 kernel integrates once with the summed weights
		a.const_grad = 1;
		for (int q = 1; q < P->rule.nq; q++)
			for (int j = 0; j < P->kind; j++)
				a.const_grad &= P->rule.dxi[q][j] == P->rule.dxi[0][j] && P->rule.deta[q][j] == P->rule.deta[0][j];
		// register rows: 8 blocks cover structured P1 meshes (7 per row), 10 cover Q1 (9)
		int const rmax = P->kind == 3 ? 8 : 10;
		if (rmax == 8) k_assemble32<8><<<blocks_for(N, 128), 128, 0, st>>>(a);
		else k_assemble32<10><<<blocks_for(N, 128), 128, 0, st>>>(a);
		a.skip_upto = rmax;
		k_assemble<false><<<blocks_for(N, 128), 128, 0, st>>>(a);
	}
	// 5. Neumann loads (X/Y, normal/tangent)
	bool has_neu = false;
	for (int c = 0; c < P->n_conds; c++)
		has_neu |= P->kinds[c] >= BFM_CONDITION_KIND_NEUMANN_X && P->kinds[c] <= BFM_CONDITION_KIND_NEUMANN_TANGENT;
	if (has_neu && P->n_edges) {
		NeuArgs na;
		memset(&na, 0, sizeof na);
		na.N = P->N;
		na.n_conds = P->n_conds;
		na.stress = P->stress;
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
	if (P->n_loads) {
		if (P->stress >= 2) return fail("per-edge loads are planar only");
		// the incidence helper counts into a buffer of N+1 ints and scans N entries
		if (incidence(P, P->ledges, P->n_loads, 2, P->lcnt, P->lptr, P->llist, 1 << 30, 0)) return -1;
		k_edge_loads<<<blocks_for(N), TPB, 0, st>>>(P->N, P->ledges, P->lloads, P->lptr, P->llist, P->coords, P->last_ci, P->b);
	}
	CK(cudaGetLastError());
	// two-level SSOR: the coarse operator of this matrix (its factorisation
	// and inverse on the side stream), while the main stream builds the
	// sweeps' sliced-ELL blocks of this matrix
	if (coarse_pc(P->precond) && coarse_setup(P, ssor)) return -1;
	if (ssor && build_sell(P)) return -1;
	if (coarse_pc(P->precond) && coarse_finish(P)) return -1;
	if (!capturing) CK(cudaEventRecord(P->ev[1], st));
	P->assembled = true;
	P->solved = false;
	return 0;
}

// The sweeps' FP32 relaxation blocks, 16 bytes per node: the high halves of
// the double-float blocks (FP64 and FP64_DF), or the mixed precisions' FP32
// blocks as they are
static int pack_relaxation_blocks(bfm_gpu_problem_t* P) {
	if (mixed_prec(P->precision))
		CK(cudaMemcpyAsync(P->ssor_d, P->dinv32, 16l * P->N, cudaMemcpyDeviceToDevice, P->stream));
	else
		k_pack_hi<<<blocks_for(P->N), TPB, 0, P->stream>>>(P->N, reinterpret_cast<const float4*>(P->dinv32), P->ssor_d);
	CK(cudaGetLastError());
	return 0;
}

int bfm_gpu_problem_solve(bfm_gpu_problem_t* P, const bfm_gpu_opts_t* opts) {
	BFM_RANGE("bfm_gpu_problem_solve");
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble before solving");
	bfm_gpu_opts_t o;
	if (opts) o = *opts;
	else bfm_gpu_default_opts(&o);
	if (!(o.rtol >= 0.0) || o.max_iters < 0) return fail("invalid solver options");
	if (o.precond < BFM_GPU_PC_JACOBI || o.precond > BFM_GPU_PC_LEARNED_SSOR2) return fail("unknown preconditioner %d", o.precond);
	if (o.precond != P->precond) {
		// the preconditioner is formed by the assembly epilogue
		P->precond = o.precond;
		if (bfm_gpu_problem_assemble(P, P->precision)) return -1;
	}
	if (o.autotune && !P->tuned) {
		if (autotune_lpr(P)) return -1;
		P->tuned = 1;
		P->graph_lpr = -1;
	}
	// options are baked into the graph's kernel parameters: rebuild only when they change
	bool const same = P->graph && P->graph_precision == P->precision && P->graph_precond == P->precond &&
	                  P->graph_lpr == P->lpr && P->graph_opts.rtol == o.rtol &&
	                  P->graph_opts.max_iters == o.max_iters && P->graph_opts.replace_drop == o.replace_drop &&
	                  P->graph_opts.refine_restart == o.refine_restart &&
	                  P->polls == (o.barrier_polls > 0 ? (long) o.barrier_polls : BARRIER_POLLS_DEFAULT);
	if (!same) {
		P->polls = o.barrier_polls > 0 ? (long) o.barrier_polls : BARRIER_POLLS_DEFAULT;
		if (build_graph(P, &o)) return -1;
		P->graph_precision = P->precision;
		P->graph_precond = P->precond;
		P->graph_lpr = P->lpr;
		P->graph_opts = o;
	}
	bool const learned = learned_pc(P->precond);
	P->fallback = 0;
	CK(cudaEventRecord(P->ev[2], P->stream));
	// the learned blocks depend on the load vector: formed for every solve, inside the timed region
	if (learned && bfmi_learned_precond(P, 0)) return -1;
	if (ssor_pc(P->precond) && P->ssor_bar) {
		CK(cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), P->stream));
		if (pack_relaxation_blocks(P)) return -1;
	}
	CK(cudaGraphLaunch(P->graph, P->stream));
	if (learned) {
		// Jacobi takes over when the learned preconditioner breaks down (a non-SPD
		// or non-finite block) or stagnates well above the roundoff floor
		CK(cudaMemcpyAsync(P->st_host, P->st, sizeof(CgState), cudaMemcpyDeviceToHost, P->stream));
		CK(cudaStreamSynchronize(P->stream));
		CgState const* h = P->st_host;
		double const rel = h->bnorm2 > 0 ? sqrt(h->true_res2 / h->bnorm2) : 0.0;
		if (h->status == BFM_GPU_BREAKDOWN || !(rel == rel) ||
		    (h->status == BFM_GPU_STAGNATED && rel > LEARNED_FALLBACK_REL)) {
			if (bfmi_set_precond_blocks(P, nullptr)) return -1;
			if (ssor_pc(P->precond) && P->ssor_bar) {
				CK(cudaMemsetAsync(P->ssor_bar, 0, BAR_WORDS * sizeof(unsigned), P->stream));
				if (pack_relaxation_blocks(P)) return -1;
			}
			CK(cudaGraphLaunch(P->graph, P->stream));
			P->fallback = 1;
		}
	}
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
		s->fallback = P->fallback;
	}
	return 0;
}

int bfm_gpu_problem_solution(bfm_gpu_problem_t* P, double* out, int where) {
	g_err[0] = 0;
	const double* x = P->x;
	if (P->ordered) {
		// back to the caller's node order
		double* dst = where == BFM_GPU_DEVICE ? out : (double*) P->otmp;
		k_gather_nodes<double><<<blocks_for(2l * P->N), TPB, 0, P->stream>>>(P->N, 2, P->x, P->iperm, dst);
		CK(cudaGetLastError());
		if (where == BFM_GPU_DEVICE) return 0;
		x = dst;
	}
	CK(cudaMemcpyAsync(out, x, 2l * P->N * sizeof(double),
	                   where == BFM_GPU_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
	if (where != BFM_GPU_DEVICE) CK(cudaStreamSynchronize(P->stream));
	return 0;
}

int bfm_gpu_problem_ordering(bfm_gpu_problem_t* P, int32_t* perm, int32_t* color_offsets, int* n_colors) {
	g_err[0] = 0;
	bool const on = P->ordered != 0;
	if (perm) {
		if (on) {
			CK(cudaMemcpyAsync(perm, P->perm, P->N * sizeof(int), cudaMemcpyDeviceToHost, P->stream));
			CK(cudaStreamSynchronize(P->stream));
		}
		else
			for (int i = 0; i < P->N; i++) perm[i] = i;
	}
	if (color_offsets && on)
		for (int c = 0; c <= P->ncol; c++) color_offsets[c] = P->col_off[c];
	if (n_colors) *n_colors = on ? P->ncol : 0;
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
		if (P->precision != BFM_GPU_MIXED) CK(cudaMemcpy(vals, P->vals64, 4 * nb * sizeof(double), cudaMemcpyDeviceToHost));
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
	return time_iteration(P, P->lpr, reps > 0 ? reps : 1, ms_spmv, ms_update);
}

int bfm_gpu_problem_time_precond(bfm_gpu_problem_t* P, int reps, double* ms, double* ms_sweeps, int* persistent) {
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble first");
	if (persistent) *persistent = P->tma_grid > 0 ? 2 : P->ssor_grid > 0 ? 1 : 0;
	return time_ssor(P, reps > 0 ? reps : 1, ms, ms_sweeps);
}

int bfm_gpu_problem_coarse_info(bfm_gpu_problem_t* P, int64_t* n_coarse, int64_t* n_chunks, int64_t* x_bytes, int* fused) {
	g_err[0] = 0;
	bool const on = coarse_pc(P->precond) && P->coarse_ok;
	if (n_coarse) *n_coarse = on ? P->nc : 0;
	if (n_chunks) *n_chunks = on ? P->nchunk : 0;
	if (x_bytes) *x_bytes = on ? 2 * (int64_t) xrow(P->nc) * (int64_t) sizeof(float) : 0;
	if (fused) *fused = on && fuse_coarse(P);
	return 0;
}

int bfm_gpu_problem_autotune(bfm_gpu_problem_t* P, int* lanes_per_row) {
	g_err[0] = 0;
	if (!P->assembled) return fail("assemble first");
	if (autotune_lpr(P)) return -1;
	P->tuned = 1;
	if (lanes_per_row) *lanes_per_row = shape_lanes(P->lpr);
	return 0;
}

int bfm_gpu_problem_shape(bfm_gpu_problem_t* P, int* shape) {
	g_err[0] = 0;
	*shape = P->lpr;
	return 0;
}

int bfm_gpu_problem_set_shape(bfm_gpu_problem_t* P, int shape) {
	g_err[0] = 0;
	if (shape == 0) {
		P->tuned = 0;
		return 0;
	}
	bool known = false;
	for (int c : SHAPES) known |= c == shape;
	if (!known) return fail("unknown SpMV shape %d", shape);
	if (shape_split(shape) && (P->precision == BFM_GPU_MIXED || P->precision == BFM_GPU_MIXED_EXACT))
		return fail("the split SpMV form exists for the FP64 and FP64_DF paths only");
	P->lpr = shape;
	P->tuned = 1;
	return 0;
}

}  // extern "C"
