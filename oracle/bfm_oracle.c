/*
 * bfm_oracle.c -- CPU restatement of libbfm's FEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU path is
 * compared against; nothing in the shipped library links or calls it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * Parity pin: the restatement is checked against the reference's golden
 * outputs data/U.txt and data/V.txt (meshes/8.lepl1110 + problems/problem.txt)
 * and against fixtures produced by the reference library itself, compiled from
 * its own sources by oracle/Makefile (see tests/golden/make_golden.py).
 *
 * Every floating-point expression keeps the reference's evaluation order, and
 * the file must be compiled with -ffp-contract=off so that no multiply-add is
 * fused (gcc contracts by default on aarch64).  Under that rule the dense
 * stiffness matrix is bit-identical to the reference's, which the RCM
 * renumbering (driven by exact zeros of K) depends on.
 *
 * All arrays are plain C arrays so the file can be driven through ctypes.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;

/* condition kinds, numbered as libbfm/src/bfm/condition.h:5-14 */
enum { ORC_DIR_X = 0, ORC_DIR_Y = 1, ORC_NEU_X = 2, ORC_NEU_Y = 3, ORC_NEU_N = 4, ORC_NEU_T = 5, ORC_DIR_N = 6, ORC_DIR_T = 7 };

typedef struct {
	int kind;              /* nodes per element: 3 (P1 triangle) or 4 (Q1 quad) */
	int stress;            /* 1: plane stress, 0: plane strain, 2: axisymmetric,
	                          3: axisymmetric with the reference's constant a     */
	i64 n_nodes, n_elems;
	const double* coords;  /* [n_nodes*2] interleaved x,y                        */
	const i64* elems;      /* [n_elems*kind]                                     */
	double E, nu, rho;     /* uniform material (libbfm/src/bfm/material.h:12-21) */
	const double* elem_E;  /* optional per-element E  (NULL: uniform)            */
	const double* elem_nu; /* optional per-element nu (NULL: uniform)            */
	int n_points;          /* Gauss rule                                          */
	const double* weights; /* [n_points]                                          */
	const double* phi;     /* [n_points*kind] shape values at the points          */
	const double* dxi;     /* [n_points*kind] d phi / d xsi                       */
	const double* deta;    /* [n_points*kind] d phi / d eta                       */
	int n_forces;
	const double* forces;  /* [n_forces*2] constant body accelerations            */
	int n_conds;
	const int* cond_kind;          /* [n_conds]                                   */
	const double* cond_value;      /* [n_conds]                                   */
	const unsigned char* cond_nodes; /* [n_conds*n_nodes] node masks              */
	i64 n_edges;
	const i64* edges;      /* [n_edges*2] node pairs (libbfm/src/bfm/mesh.h:17-23) */
	const unsigned char* edge_boundary; /* [n_edges] 1: one adjacent element (elems[1] == -1); NULL: all */
} orc_problem_t;

/* Gauss rule and shape tables, libbfm/src/rule.c:90-111 and shape.c:3-85. */
int orc_gauss_tables(int kind, double* weights, double* phi, double* dxi, double* deta) {
	double const third = 1. / 3, sixth = 1. / 6;
	double const s = 0.577350269189626; /* the reference's truncated literal, rule.c:92 */
	if (kind == 3) {
		double const pts[3][2] = {{sixth, sixth}, {1 - third, sixth}, {sixth, 1 - third}};
		for (int q = 0; q < 3; q++) {
			double const x = pts[q][0], e = pts[q][1];
			weights[q] = sixth;
			phi[q * 3 + 0] = 1 - x - e;
			phi[q * 3 + 1] = x;
			phi[q * 3 + 2] = e;
			dxi[q * 3 + 0] = -1; dxi[q * 3 + 1] = 1; dxi[q * 3 + 2] = 0;
			deta[q * 3 + 0] = -1; deta[q * 3 + 1] = 0; deta[q * 3 + 2] = 1;
		}
		return 3;
	}
	if (kind == 4) {
		double const pts[4][2] = {{-s, s}, {-s, -s}, {s, -s}, {s, s}};
		for (int q = 0; q < 4; q++) {
			double const x = pts[q][0], e = pts[q][1];
			weights[q] = 1;
			phi[q * 4 + 0] = (1 + x) * (1 + e) / 4;
			phi[q * 4 + 1] = (1 - x) * (1 + e) / 4;
			phi[q * 4 + 2] = (1 - x) * (1 - e) / 4;
			phi[q * 4 + 3] = (1 + x) * (1 - e) / 4;
			dxi[q * 4 + 0] = (1 + e) / 4;  deta[q * 4 + 0] = (1 + x) / 4;
			dxi[q * 4 + 1] = (-1 - e) / 4; deta[q * 4 + 1] = (1 - x) / 4;
			dxi[q * 4 + 2] = (-1 + e) / 4; deta[q * 4 + 2] = (-1 + x) / 4;
			dxi[q * 4 + 3] = (1 - e) / 4;  deta[q * 4 + 3] = (-1 - x) / 4;
		}
		return 4;
	}
	return -1;
}

/* Material constants, libbfm/src/system.c:454-458; axisymmetric ones,
 * system.c:241-243 (mode 3 keeps the reference's a = E(1-nu)/(1+nu)*(1-2nu),
 * mode 2 the divided form of plane strain). */
static void material_abc(double E, double nu, int stress, double* a, double* b, double* c) {
	int const strain = stress != 1;
	*a = strain ? E * (1 - nu) / (1 + nu) / (1 - 2 * nu) : E / (1 - nu * nu);
	if (stress == 3) *a = E * (1 - nu) / (1 + nu) * (1 - 2 * nu);
	*b = strain ? E * nu / (1 + nu) / (1 - 2 * nu) : E * nu / (1 - nu * nu);
	*c = E / (2 * (1 + nu));
}

/*
 * Element loop body, libbfm/src/system.c:109-227 (fill_elasticity_elem).
 * `add(ctx, row, col, v)` receives every stiffness term in the reference's
 * order: Gauss point outer, then local node j, then local node k, then the
 * four (u,v) components.  Body-force terms go straight into b.
 */
typedef void (*orc_add_fn)(void* ctx, i64 row, i64 col, double v);

static void element_terms(const orc_problem_t* P, i64 e, double* bvec, orc_add_fn add, void* ctx) {
	int const kind = P->kind;
	i64 map[4];
	double x[4], y[4];
	for (int j = 0; j < kind; j++) {
		map[j] = P->elems[e * kind + j];
		x[j] = P->coords[map[j] * 2 + 0];
		y[j] = P->coords[map[j] * 2 + 1];
	}
	double const E = P->elem_E ? P->elem_E[e] : P->E;
	double const nu = P->elem_nu ? P->elem_nu[e] : P->nu;
	double a, b, c;
	material_abc(E, nu, P->stress, &a, &b, &c);

	for (int q = 0; q < P->n_points; q++) {
		double const w = P->weights[q];
		double const* phi = P->phi + q * kind;
		double const* dxi = P->dxi + q * kind;
		double const* deta = P->deta + q * kind;
		double dx_dxsi = 0, dx_deta = 0, dy_dxsi = 0, dy_deta = 0;
		for (int j = 0; j < kind; j++) {
			dx_dxsi += x[j] * dxi[j];
			dx_deta += x[j] * deta[j];
			dy_dxsi += y[j] * dxi[j];
			dy_deta += y[j] * deta[j];
		}
		double const det = fabs(dx_dxsi * dy_deta - dx_deta * dy_dxsi);
		double dx[4], dy[4];
		for (int j = 0; j < kind; j++) {
			dx[j] = (dxi[j] * dy_deta - deta[j] * dy_dxsi) / det;
			dy[j] = (deta[j] * dx_dxsi - dxi[j] * dx_deta) / det;
		}
		if (P->stress >= 2) {
			/* axisymmetric element, libbfm/src/system.c:229-356 */
			double rr = 0;
			for (int j = 0; j < kind; j++) rr += x[j] * phi[j];
			for (int j = 0; j < kind; j++) {
				i64 const r = 2 * map[j];
				for (int f = 0; f < P->n_forces; f++) {
					bvec[r + 0] += det * w * P->forces[2 * f + 0] * P->rho * phi[j] * rr;
					bvec[r + 1] += det * w * P->forces[2 * f + 1] * P->rho * phi[j] * rr;
				}
			}
			for (int j = 0; j < kind; j++) {
				i64 const r = 2 * map[j];
				for (int k = 0; k < kind; k++) {
					i64 const s = 2 * map[k];
					double const f11 = a * dx[j] * dx[k] * rr + c * dy[j] * dy[k] * rr + phi[j] * (b * dx[k] + a * phi[k] / rr) + dx[j] * b * phi[k];
					double const f12 = b * dx[j] * dy[k] * rr + c * dy[j] * dx[k] * rr + phi[j] * b * dy[k];
					double const f21 = b * dy[j] * dx[k] * rr + c * dx[j] * dy[k] * rr + dy[j] * b * phi[k];
					/* the reference leaves the radius off this c term; mode 2 puts it back */
					double const f22 = a * dy[j] * dy[k] * rr + (P->stress == 2 ? c * dx[j] * dx[k] * rr : c * dx[j] * dx[k]);
					add(ctx, r + 0, s + 0, det * w * f11);
					add(ctx, r + 0, s + 1, det * w * f12);
					add(ctx, r + 1, s + 0, det * w * f21);
					add(ctx, r + 1, s + 1, det * w * f22);
				}
			}
			continue;
		}
		for (int j = 0; j < kind; j++) {
			i64 const r = 2 * map[j];
			for (int f = 0; f < P->n_forces; f++) {
				bvec[r + 0] += det * w * P->forces[2 * f + 0] * P->rho * phi[j];
				bvec[r + 1] += det * w * P->forces[2 * f + 1] * P->rho * phi[j];
			}
		}
		for (int j = 0; j < kind; j++) {
			i64 const r = 2 * map[j];
			for (int k = 0; k < kind; k++) {
				i64 const s = 2 * map[k];
				double const f11 = a * dx[j] * dx[k] + c * dy[j] * dy[k];
				double const f12 = b * dx[j] * dy[k] + c * dy[j] * dx[k];
				double const f21 = b * dy[j] * dx[k] + c * dx[j] * dy[k];
				double const f22 = a * dy[j] * dy[k] + c * dx[j] * dx[k];
				add(ctx, r + 0, s + 0, det * w * f11);
				add(ctx, r + 0, s + 1, det * w * f12);
				add(ctx, r + 1, s + 0, det * w * f21);
				add(ctx, r + 1, s + 1, det * w * f22);
			}
		}
	}
}

/* Neumann X/Y edge loads, libbfm/src/system.c:477-498. */
static void neumann(const orc_problem_t* P, int ci, double* bvec) {
	int const shift = P->cond_kind[ci] == ORC_NEU_X ? 0 : 1;
	const unsigned char* mask = P->cond_nodes + (i64) ci * P->n_nodes;
	for (i64 j = 0; j < P->n_edges; j++) {
		i64 const n1 = P->edges[2 * j], n2 = P->edges[2 * j + 1];
		if (!mask[n1] || !mask[n2]) continue;
		double const c2 = pow(P->coords[n1 * 2 + 0] - P->coords[n2 * 2 + 0], 2) +
		                  pow(P->coords[n1 * 2 + 1] - P->coords[n2 * 2 + 1], 2);
		double const jac = sqrt(c2) / 2;
		if (P->stress == 2) {
			/* consistent axisymmetric load: value jac times the integral over
			 * [-1, 1] of (shape function) x (radius) = (2 r_this + r_other) / 3 */
			double const x1 = P->coords[n1 * 2 + 0], x2 = P->coords[n2 * 2 + 0];
			bvec[n1 * 2 + shift] += (2.0 * x1 + x2) / 3.0 * jac * P->cond_value[ci];
			bvec[n2 * 2 + shift] += (2.0 * x2 + x1) / 3.0 * jac * P->cond_value[ci];
			continue;
		}
		if (P->stress == 3) {
			/* axisymmetric loads, libbfm/src/system.c:583-612 (radius factor as written there) */
			double const r1 = P->coords[n1 * 2 + 0] * (1 - 1 / sqrt(3)) / 2 + P->coords[n1 * 2 + 1] * (1 + 1 / sqrt(3)) / 2;
			double const r2 = P->coords[n2 * 2 + 0] * (1 - 1 / sqrt(3)) / 2 + P->coords[n2 * 2 + 1] * (1 + 1 / sqrt(3)) / 2;
			double const fac = r1 + r2;
			bvec[n1 * 2 + shift] += fac * jac * P->cond_value[ci];
			bvec[n2 * 2 + shift] += fac * jac * P->cond_value[ci];
			continue;
		}
		bvec[n1 * 2 + shift] += jac * P->cond_value[ci];
		bvec[n2 * 2 + shift] += jac * P->cond_value[ci];
	}
}

/* Neumann normal/tangent edge loads, libbfm/src/system.c:500-522. */
static void neumann_nt(const orc_problem_t* P, int ci, double* bvec) {
	int const tangent = P->cond_kind[ci] == ORC_NEU_T;
	double const value = P->cond_value[ci];
	const unsigned char* mask = P->cond_nodes + (i64) ci * P->n_nodes;
	for (i64 j = 0; j < P->n_edges; j++) {
		i64 const n1 = P->edges[2 * j], n2 = P->edges[2 * j + 1];
		if (!mask[n1] || !mask[n2]) continue;
		double const dx = P->coords[n1 * 2 + 0] - P->coords[n2 * 2 + 0];
		double const dy = P->coords[n1 * 2 + 1] - P->coords[n2 * 2 + 1];
		bvec[n1 * 2 + 0] += 0.5 * value * (tangent ? dx : -dy);
		bvec[n1 * 2 + 1] += 0.5 * value * (tangent ? dy : dx);
		bvec[n2 * 2 + 0] += 0.5 * value * (tangent ? dx : -dy);
		bvec[n2 * 2 + 1] += 0.5 * value * (tangent ? dy : dx);
	}
}

/* The two values a Dirichlet normal/tangent condition prescribes at node i,
 * libbfm/src/system.c:388-425: half-sums over the node's boundary edges of
 * the unit vector from the other end, then value * (tx, ty) or (-ty, tx). */
static void dirichlet_nt_values(const orc_problem_t* P, int ci, i64 i, double* v0, double* v1) {
	double tx = 0, ty = 0;
	for (i64 j = 0; j < P->n_edges; j++) {
		int const boundary = P->edge_boundary ? P->edge_boundary[j] : 1;
		i64 n2 = -1;
		if (P->edges[2 * j] == i && boundary) n2 = P->edges[2 * j + 1];
		else if (P->edges[2 * j + 1] == i && boundary) n2 = P->edges[2 * j];
		if (n2 < 0) continue;
		double const length = sqrt(pow(P->coords[i * 2 + 0] - P->coords[n2 * 2 + 0], 2) +
		                           pow(P->coords[i * 2 + 1] - P->coords[n2 * 2 + 1], 2));
		tx += (P->coords[i * 2 + 0] - P->coords[n2 * 2 + 0]) / length / 2;
		ty += (P->coords[i * 2 + 1] - P->coords[n2 * 2 + 1]) / length / 2;
	}
	int const tangent = P->cond_kind[ci] == ORC_DIR_T;
	*v0 = P->cond_value[ci] * (tangent ? tx : -ty);
	*v1 = P->cond_value[ci] * (tangent ? ty : tx);
}

/* ---------------------------------------------------------------- dense */

typedef struct { double* K; i64 n; } dense_ctx_t;

static void dense_add(void* ctx, i64 r, i64 c, double v) {
	dense_ctx_t* d = ctx;
	d->K[r * d->n + c] += v;
}

/* Symmetric elimination of one DOF, libbfm/src/system.c:358-374. */
static void dense_constraint(double* K, double* bvec, i64 n, i64 d, double val) {
	for (i64 i = 0; i < n; i++) {
		bvec[i] -= val * K[i * n + d];
		K[i * n + d] = 0;
	}
	for (i64 i = 0; i < n; i++) K[d * n + i] = 0;
	K[d * n + d] = 1;
	bvec[d] = val;
}

/*
 * Dense K (row-major n*n, zeroed by the caller) and b (zeroed), assembled and
 * constrained exactly as libbfm/src/system.c:427-529 (create_planar).
 */
int orc_assemble_dense(const orc_problem_t* P, double* K, double* bvec) {
	i64 const n = 2 * P->n_nodes;
	dense_ctx_t ctx = {K, n};
	for (i64 e = 0; e < P->n_elems; e++) element_terms(P, e, bvec, dense_add, &ctx);
	for (int ci = 0; ci < P->n_conds; ci++) {
		int const k = P->cond_kind[ci];
		if (k == ORC_DIR_X || k == ORC_DIR_Y) {
			const unsigned char* mask = P->cond_nodes + (i64) ci * P->n_nodes;
			for (i64 j = 0; j < P->n_nodes; j++)
				if (mask[j]) dense_constraint(K, bvec, n, 2 * j + (k == ORC_DIR_X ? 0 : 1), P->cond_value[ci]);
		}
		else if (k == ORC_NEU_X || k == ORC_NEU_Y) {
			neumann(P, ci, bvec);
		}
		else if (k == ORC_NEU_N || k == ORC_NEU_T) {
			if (P->stress < 2) neumann_nt(P, ci, bvec);  /* the axisymmetric system skips them */
		}
		else if (k == ORC_DIR_N || k == ORC_DIR_T) {
			const unsigned char* mask = P->cond_nodes + (i64) ci * P->n_nodes;
			for (i64 j = 0; j < P->n_nodes; j++) {
				if (!mask[j]) continue;
				double v0, v1;
				dirichlet_nt_values(P, ci, j, &v0, &v1);
				dense_constraint(K, bvec, n, 2 * j + 0, v0);
				dense_constraint(K, bvec, n, 2 * j + 1, v1);
			}
		}
		else {
			return -1;
		}
	}
	return 0;
}

/* ---------------------------------------------------------------- RCM */

typedef struct { i64 i; i64 deg; } rcm_node_t;

/* stable insertion sort by degree; glibc's qsort behaved as a stable merge sort for the reference */
static void sort_by_degree(rcm_node_t* v, i64 cnt) {
	for (i64 i = 1; i < cnt; i++) {
		rcm_node_t const t = v[i];
		i64 j = i - 1;
		while (j >= 0 && (int) v[j].deg - (int) t.deg > 0) {
			v[j + 1] = v[j];
			j--;
		}
		v[j + 1] = t;
	}
}

/*
 * Reverse Cuthill-McKee on the numeric nonzeros of a dense matrix, restating
 * libbfm/src/perm.c:117-331: degree counts the diagonal; the root is the LAST
 * unvisited index of minimum degree; neighbours are marked visited when
 * enqueued and pushed in stable degree order; popped node p lands at n-1-p.
 */
int orc_rcm_dense(i64 n, const double* K, i64* perm, i64* inv_perm) {
	i64* degs = calloc(n ? n : 1, sizeof *degs);
	unsigned char* visited = calloc(n ? n : 1, 1);
	i64* queue = malloc((n ? n : 1) * sizeof *queue);
	rcm_node_t* to_sort = malloc((n ? n : 1) * sizeof *to_sort);
	if (!degs || !visited || !queue || !to_sort) return -1;
	for (i64 i = 0; i < n; i++)
		for (i64 j = 0; j < n; j++) degs[i] += K[i * n + j] != 0;
	i64 qs = 0, qe = 0, p = 0;
	while (p < n) {
		i64 min_deg = INT64_MAX, root = 0;
		for (i64 i = 0; i < n; i++) {
			if (visited[i]) continue;
			if (degs[i] <= min_deg) { min_deg = degs[i]; root = i; }
		}
		queue[qe++ % n] = root;
		while (qs != qe) {
			i64 const cur = queue[qs++ % n];
			visited[cur] = 1;
			i64 cnt = 0;
			for (i64 i = 0; i < n; i++) {
				if (visited[i] || K[cur * n + i] == 0) continue;
				to_sort[cnt].i = i;
				to_sort[cnt].deg = degs[i];
				cnt++;
				visited[i] = 1;
			}
			sort_by_degree(to_sort, cnt);
			for (i64 i = 0; i < cnt; i++) queue[qe++ % n] = to_sort[i].i;
			inv_perm[n - p - 1] = cur;
			p++;
		}
	}
	for (i64 i = 0; i < n; i++) perm[inv_perm[i]] = i;
	free(degs); free(visited); free(queue); free(to_sort);
	return 0;
}

/*
 * RCM on a CSR matrix (column indices ascending in each row).  Same ordering
 * rule as orc_rcm_dense; entries with value exactly 0 are ignored, as the
 * reference ignores numeric zeros of its dense matrix.
 */
int orc_rcm_csr(i64 n, const i64* row_ptr, const i64* cols, const double* vals, i64* perm, i64* inv_perm) {
	i64* degs = calloc(n ? n : 1, sizeof *degs);
	unsigned char* visited = calloc(n ? n : 1, 1);
	i64* queue = malloc((n ? n : 1) * sizeof *queue);
	rcm_node_t* to_sort = malloc((n ? n : 1) * sizeof *to_sort);
	if (!degs || !visited || !queue || !to_sort) return -1;
	for (i64 i = 0; i < n; i++)
		for (i64 k = row_ptr[i]; k < row_ptr[i + 1]; k++) degs[i] += vals[k] != 0;
	i64 qs = 0, qe = 0, p = 0;
	while (p < n) {
		i64 min_deg = INT64_MAX, root = 0;
		for (i64 i = 0; i < n; i++) {
			if (visited[i]) continue;
			if (degs[i] <= min_deg) { min_deg = degs[i]; root = i; }
		}
		queue[qe++ % n] = root;
		while (qs != qe) {
			i64 const cur = queue[qs++ % n];
			visited[cur] = 1;
			i64 cnt = 0;
			for (i64 k = row_ptr[cur]; k < row_ptr[cur + 1]; k++) {
				i64 const i = cols[k];
				if (visited[i] || vals[k] == 0) continue;
				to_sort[cnt].i = i;
				to_sort[cnt].deg = degs[i];
				cnt++;
				visited[i] = 1;
			}
			sort_by_degree(to_sort, cnt);
			for (i64 i = 0; i < cnt; i++) queue[qe++ % n] = to_sort[i].i;
			inv_perm[n - p - 1] = cur;
			p++;
		}
	}
	for (i64 i = 0; i < n; i++) perm[inv_perm[i]] = i;
	free(degs); free(visited); free(queue); free(to_sort);
	return 0;
}

/* ---------------------------------------------------------------- band LU */

/*
 * Permute (new[perm[i]][perm[j]] = old[i][j], libbfm/src/perm.c:26-68), find
 * the bandwidth (matrix.c:57-71), factor in band form without pivoting
 * (matrix.c:253-302) and substitute (matrix.c:351-404).  Returns -1 on a
 * pivot below 1e-20 like the reference; b is overwritten with the solution in
 * permuted order.
 */
static int band_solve(i64 n, const double* Kp, double* y) {
	i64 k = 0;
	for (i64 i = 0; i < n; i++)
		for (i64 j = 0; j < n; j++)
			if (Kp[i * n + j] != 0) {
				i64 const d = i > j ? i - j : j - i;
				if (d > k) k = d;
			}
	i64 const w = 2 * k + 1;
	double* B = calloc((size_t) (n * w) ? (size_t) (n * w) : 1, sizeof *B);
	if (!B) return -1;
#define BAND(i, j) B[(i) * w + ((j) - (i) + k)]
	for (i64 i = 0; i < n; i++)
		for (i64 j = (i - k > 0 ? i - k : 0); j <= i + k && j < n; j++) BAND(i, j) = Kp[i * n + j];
	int rv = 0;
	for (i64 p = 0; p + 1 < n; p++) {
		double const piv = BAND(p, p);
		if (piv != piv || fabs(piv) < 1e-20) { rv = -1; goto out; }
		i64 const len = p + k + 1 < n ? p + k + 1 : n;
		for (i64 i = p + 1; i < len; i++) {
			double const v = BAND(i, p) / piv;
			BAND(i, p) = v;
			for (i64 j = p + 1; j < len; j++) BAND(i, j) += -v * BAND(p, j);
		}
	}
	for (i64 p = 0; p < n; p++) {
		i64 const lo = p - k > 0 ? p - k : 0;
		for (i64 i = lo; i < p; i++) y[p] -= BAND(p, i) * y[i];
	}
	for (i64 p = n - 1; p >= 0; p--) {
		i64 const hi = p + k + 1 < n ? p + k + 1 : n;
		for (i64 i = p + 1; i < hi; i++) y[p] -= y[i] * BAND(p, i);
		double const piv = BAND(p, p);
		if (piv != piv || !piv) { rv = -1; goto out; }
		y[p] /= piv;
	}
out:
#undef BAND
	free(B);
	return rv;
}

/*
 * The whole reference pipeline for one instance, libbfm/src/sim.c:103-135:
 * dense assembly + conditions, RCM renumbering, band LU, inverse permutation.
 * effects[2*N] receives u,v per node; perm_out (optional) the RCM permutation.
 */
int orc_solve_reference(const orc_problem_t* P, double* effects, i64* perm_out, i64* bandwidth_out) {
	i64 const n = 2 * P->n_nodes;
	double* K = calloc((size_t) (n * n) ? (size_t) (n * n) : 1, sizeof *K);
	double* b = calloc(n ? n : 1, sizeof *b);
	i64* perm = malloc((n ? n : 1) * sizeof *perm);
	i64* inv = malloc((n ? n : 1) * sizeof *inv);
	if (!K || !b || !perm || !inv) return -1;
	int rv = orc_assemble_dense(P, K, b);
	if (rv == 0) rv = orc_rcm_dense(n, K, perm, inv);
	if (rv == 0) {
		double* Kp = malloc((size_t) (n * n) ? (size_t) (n * n) * sizeof *Kp : 1);
		double* bp = malloc((n ? n : 1) * sizeof *bp);
		for (i64 i = 0; i < n; i++) {
			bp[perm[i]] = b[i];
			for (i64 j = 0; j < n; j++) Kp[perm[i] * n + perm[j]] = K[i * n + j];
		}
		if (bandwidth_out) {
			i64 k = 0;
			for (i64 i = 0; i < n; i++)
				for (i64 j = 0; j < n; j++)
					if (Kp[i * n + j] != 0 && (i > j ? i - j : j - i) > k) k = i > j ? i - j : j - i;
			*bandwidth_out = k;
		}
		band_solve(n, Kp, bp); /* the reference ignores this status (sim.c:122) */
		for (i64 i = 0; i < n; i++) effects[inv[i]] = bp[i];
		if (perm_out) memcpy(perm_out, perm, n * sizeof *perm);
		free(Kp); free(bp);
	}
	free(K); free(b); free(perm); free(inv);
	return rv;
}

/* ---------------------------------------------------------------- CSR */

/*
 * Node-graph pattern: for each node the sorted set of nodes sharing an
 * element with it (itself included).  Returns the block count; row_ptr has
 * n_nodes+1 entries, cols is allocated by the callee.
 */
static i64 node_graph(const orc_problem_t* P, i64** row_ptr_out, i64** cols_out) {
	i64 const N = P->n_nodes, kind = P->kind;
	i64* cnt = calloc(N + 1, sizeof *cnt);
	for (i64 e = 0; e < P->n_elems; e++)
		for (int j = 0; j < kind; j++) cnt[P->elems[e * kind + j] + 1] += kind;
	for (i64 i = 0; i < N; i++) cnt[i + 1] += cnt[i];
	i64* cand = malloc((cnt[N] ? cnt[N] : 1) * sizeof *cand);
	i64* fill = calloc(N, sizeof *fill);
	for (i64 e = 0; e < P->n_elems; e++)
		for (int j = 0; j < kind; j++) {
			i64 const r = P->elems[e * kind + j];
			for (int k = 0; k < kind; k++) cand[cnt[r] + fill[r]++] = P->elems[e * kind + k];
		}
	i64* row_ptr = calloc(N + 1, sizeof *row_ptr);
	for (i64 r = 0; r < N; r++) {
		i64* v = cand + cnt[r];
		i64 const m = cnt[r + 1] - cnt[r];
		for (i64 i = 1; i < m; i++) {
			i64 const t = v[i];
			i64 j = i - 1;
			while (j >= 0 && v[j] > t) { v[j + 1] = v[j]; j--; }
			v[j + 1] = t;
		}
		i64 u = 0;
		for (i64 i = 0; i < m; i++)
			if (u == 0 || v[u - 1] != v[i]) v[u++] = v[i];
		/* isolated nodes still get their diagonal block */
		row_ptr[r + 1] = u ? u : 1;
		fill[r] = u;
	}
	for (i64 r = 0; r < N; r++) row_ptr[r + 1] += row_ptr[r];
	i64* cols = malloc((row_ptr[N] ? row_ptr[N] : 1) * sizeof *cols);
	for (i64 r = 0; r < N; r++) {
		if (fill[r]) memcpy(cols + row_ptr[r], cand + cnt[r], fill[r] * sizeof *cols);
		else cols[row_ptr[r]] = r;
	}
	free(cnt); free(cand); free(fill);
	*row_ptr_out = row_ptr;
	*cols_out = cols;
	return row_ptr[N];
}

typedef struct {
	const i64* node_ptr; const i64* node_cols; double* vals; /* scalar CSR, 2 entries per block column */
} csr_ctx_t;

static void csr_add(void* ctx, i64 r, i64 c, double v) {
	csr_ctx_t* s = ctx;
	i64 const rn = r / 2, cn = c / 2;
	i64 lo = s->node_ptr[rn], hi = s->node_ptr[rn + 1] - 1;
	while (lo < hi) {
		i64 const mid = (lo + hi) / 2;
		if (s->node_cols[mid] < cn) lo = mid + 1; else hi = mid;
	}
	/* scalar row r holds 2*(blocks of its node) entries, block-columns ascending */
	i64 const base = 2 * s->node_ptr[rn] * 2 + (r % 2) * 2 * (s->node_ptr[rn + 1] - s->node_ptr[rn]);
	s->vals[base + 2 * (lo - s->node_ptr[rn]) + (c % 2)] += v;
}

/*
 * Scalar CSR (2N rows) over the structural node-graph pattern, values summed
 * in the reference's order (element, then Gauss point), so each entry is
 * bit-identical to the dense restatement.  Dirichlet X/Y is applied
 * symmetrically with the reference's condition-order semantics: an
 * eliminated column subtracts the FIRST value given to that DOF; b at a
 * constrained DOF holds the LAST value plus any Neumann load applied after
 * it (system.c:358-386, 470-498).
 *
 * Two calls: first with vals == NULL to get nnz (returned), then with arrays
 * row_ptr[2N+1], cols[nnz], vals[nnz], b[2N] (b zeroed by the caller).
 */
i64 orc_assemble_csr(const orc_problem_t* P, i64* row_ptr, i64* cols, double* vals, double* bvec) {
	i64 *nptr, *ncols;
	i64 const nb = node_graph(P, &nptr, &ncols);
	i64 const N = P->n_nodes, n = 2 * N;
	if (!vals) { free(nptr); free(ncols); return 4 * nb; }
	for (i64 r = 0; r < n; r++) {
		i64 const rn = r / 2, len = nptr[rn + 1] - nptr[rn];
		row_ptr[r] = 4 * nptr[rn] + (r % 2) * 2 * len;
		for (i64 b = 0; b < len; b++) {
			cols[row_ptr[r] + 2 * b + 0] = 2 * ncols[nptr[rn] + b] + 0;
			cols[row_ptr[r] + 2 * b + 1] = 2 * ncols[nptr[rn] + b] + 1;
		}
	}
	row_ptr[n] = 4 * nb;
	memset(vals, 0, 4 * nb * sizeof *vals);
	csr_ctx_t ctx = {nptr, ncols, vals};
	for (i64 e = 0; e < P->n_elems; e++) element_terms(P, e, bvec, csr_add, &ctx);

	/* per-DOF Dirichlet bookkeeping in condition order */
	double* first = malloc(n * sizeof *first);
	double* last = malloc(n * sizeof *last);
	int* last_ci = malloc(n * sizeof *last_ci);
	for (i64 i = 0; i < n; i++) last_ci[i] = -1;
	for (int ci = 0; ci < P->n_conds; ci++) {
		int const k = P->cond_kind[ci];
		const unsigned char* mask = P->cond_nodes + (i64) ci * N;
		if (k == ORC_DIR_X || k == ORC_DIR_Y) {
			for (i64 j = 0; j < N; j++) {
				if (!mask[j]) continue;
				i64 const d = 2 * j + (k == ORC_DIR_X ? 0 : 1);
				if (last_ci[d] < 0) first[d] = P->cond_value[ci];
				last[d] = P->cond_value[ci];
				last_ci[d] = ci;
			}
		}
		else if (k == ORC_DIR_N || k == ORC_DIR_T) {
			for (i64 j = 0; j < N; j++) {
				if (!mask[j]) continue;
				double v[2];
				dirichlet_nt_values(P, ci, j, &v[0], &v[1]);
				for (int c = 0; c < 2; c++) {
					i64 const d = 2 * j + c;
					if (last_ci[d] < 0) first[d] = v[c];
					last[d] = v[c];
					last_ci[d] = ci;
				}
			}
		}
		else if (k < ORC_NEU_X || k > ORC_NEU_T) {
			free(first); free(last); free(last_ci); free(nptr); free(ncols);
			return -1;
		}
	}
	/* b_i -= K[i,d] * first[d] over constrained d, then zero rows/cols */
	for (i64 r = 0; r < n; r++) {
		for (i64 k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
			i64 const c = cols[k];
			if (last_ci[c] >= 0 && last_ci[r] < 0) bvec[r] -= first[c] * vals[k];
		}
	}
	for (i64 r = 0; r < n; r++) {
		for (i64 k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
			i64 const c = cols[k];
			if (last_ci[r] >= 0 || last_ci[c] >= 0) vals[k] = (r == c) ? 1.0 : 0.0;
		}
		if (last_ci[r] >= 0) bvec[r] = last[r];
	}
	/* Neumann in condition order; a load on a constrained DOF survives only after its last Dirichlet */
	double* tmp = calloc(n, sizeof *tmp);
	for (int ci = 0; ci < P->n_conds; ci++) {
		int const k = P->cond_kind[ci];
		if (k < ORC_NEU_X || k > ORC_NEU_T) continue;
		memset(tmp, 0, n * sizeof *tmp);
		if (k == ORC_NEU_X || k == ORC_NEU_Y) neumann(P, ci, tmp);
		else if (P->stress < 2) neumann_nt(P, ci, tmp);
		for (i64 i = 0; i < n; i++)
			if (tmp[i] != 0 && (last_ci[i] < 0 || last_ci[i] < ci)) bvec[i] += tmp[i];
	}
	free(tmp); free(first); free(last); free(last_ci); free(nptr); free(ncols);
	return 4 * nb;
}
