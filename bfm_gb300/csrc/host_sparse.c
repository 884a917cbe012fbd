/* Sparse system matrices (BFM_MATRIX_KIND_SPARSE, an addition to the
 * reference's matrix kinds, libbfm/src/bfm/matrix.h:10-43).
 *
 * The reference's bfm_system_create_planar_* store the stiffness matrix dense
 * (n^2 doubles, system.c:13), renumber it with RCM, convert it to band storage
 * and factor it (system.c:44-81, matrix.c:531-541): infeasible past some
 * 30,000 DOF.  A SPARSE system matrix keeps the GPU assembly's 2x2-block CSR
 * on the device (the assembled problem) with a host copy for reads, O(nnz) in
 * all.  bfm_system_renumber computes the reference's RCM permutation from it
 * and permutes the right-hand side, as the reference does, but the matrix keeps
 * its storage and only records the permutation; bfm_matrix_solve then solves
 * with the GPU PCG in the caller's order and returns the solution in the
 * renumbered one, so the reference's sequence (create, renumber, solve, inverse
 * permutation of the vector; sim.c:103-135) works unchanged. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <bfm/gpu.h>
#include <bfm/matrix.h>
#include <bfm/perm.h>

#include "internal.h"
#include "trace.h"

typedef struct {
	bfm_state_t* state;
	bfm_gpu_problem_t* P; /* the assembled problem: owns the device matrix */
	size_t nn;            /* nodes: the matrix has 2 nn rows               */
	int32_t* rp;          /* host copy, 2x2-block CSR in the caller's order */
	int32_t* cols;
	double* vals;
	size_t const* perm;   /* renumbering applied to the system (new = perm[old]), or NULL */
	size_t const* inv;
} sparse_t;

static sparse_t* handle_of(bfm_matrix_t* A) { return (sparse_t*) A->sparse.handle; }

int bfmi_sparse_wrap(bfm_matrix_t* A, bfm_state_t* state, bfm_gpu_problem_t* P, size_t nn, double* b) {
	int64_t nb = 0;
	if (bfm_gpu_problem_n_blocks(P, &nb) < 0) return -1;
	sparse_t* h = state->alloc(sizeof *h);
	if (!h) return -1;
	memset(h, 0, sizeof *h);
	h->state = state;
	h->P = P;
	h->nn = nn;
	h->rp = state->alloc((nn + 1) * sizeof *h->rp);
	h->cols = state->alloc((size_t) nb * sizeof *h->cols + 1);
	h->vals = state->alloc((size_t) nb * 4 * sizeof *h->vals + 1);
	if (!h->rp || !h->cols || !h->vals || bfm_gpu_problem_download(P, h->rp, h->cols, h->vals, b) < 0) {
		if (h->rp) state->free(h->rp);
		if (h->cols) state->free(h->cols);
		if (h->vals) state->free(h->vals);
		state->free(h);
		return -1;
	}
	memset(A, 0, sizeof *A);
	A->state = state;
	A->kind = BFM_MATRIX_KIND_SPARSE;
	A->major = BFM_MATRIX_MAJOR_ROW;
	A->m = 2 * nn;
	A->sparse.handle = h;
	A->sparse.nnz = 4 * (size_t) nb;
	return 0;
}

int bfmi_sparse_destroy(bfm_matrix_t* A) {
	sparse_t* h = handle_of(A);
	if (!h) return 0;
	bfm_gpu_problem_destroy(h->P);
	h->state->free(h->rp);
	h->state->free(h->cols);
	h->state->free(h->vals);
	h->state->free(h);
	A->sparse.handle = NULL;
	return 0;
}

/* entry (i, j) of the caller-order matrix; 0 outside the pattern */
static double entry(sparse_t const* h, size_t i, size_t j) {
	size_t const r = i / 2, c = j / 2;
	int32_t lo = h->rp[r], hi = h->rp[r + 1] - 1;
	while (lo <= hi) {  // columns ascend within a row
		int32_t const mid = lo + (hi - lo) / 2;
		if ((size_t) h->cols[mid] == c) return h->vals[4l * mid + 2 * (i % 2) + (j % 2)];
		if ((size_t) h->cols[mid] < c) lo = mid + 1;
		else hi = mid - 1;
	}
	return 0.0;
}

/* entry (i, j) of the system's matrix: P A P^T once renumbered */
double bfmi_sparse_get(bfm_matrix_t* A, size_t i, size_t j) {
	sparse_t const* h = handle_of(A);
	if (h->inv) {
		i = h->inv[i];
		j = h->inv[j];
	}
	return entry(h, i, j);
}

/* largest |i - j| over the nonzeros of the (renumbered) matrix */
size_t bfmi_sparse_bandwidth(bfm_matrix_t* A) {
	sparse_t const* h = handle_of(A);
	size_t k = 0;
	for (size_t r = 0; r < h->nn; r++)
		for (int32_t e = h->rp[r]; e < h->rp[r + 1]; e++)
			for (int t = 0; t < 4; t++) {
				if (h->vals[4l * e + t] == 0.0) continue;
				size_t i = 2 * r + t / 2, j = 2 * (size_t) h->cols[e] + t % 2;
				if (h->perm) {
					i = h->perm[i];
					j = h->perm[j];
				}
				size_t const d = i > j ? i - j : j - i;
				if (d > k) k = d;
			}
	return k;
}

/* The reference's RCM (perm.c:117-331) of the matrix's numeric nonzeros,
 * from the scalar rows of the block CSR (the sparse, bit-exact restatement
 * bfm_gpu_rcm_csr). */
int bfmi_sparse_rcm(bfm_perm_t* perm, bfm_matrix_t* A) {
	sparse_t const* h = handle_of(A);
	bfm_state_t* const st = perm->state;
	size_t const m = A->m;
	if (perm->m != m) return -1;
	size_t const nnz = A->sparse.nnz;
	int64_t* rp = st->alloc((m + 1) * sizeof *rp);
	int64_t* cols = st->alloc(nnz * sizeof *cols + 1);
	double* vals = st->alloc(nnz * sizeof *vals + 1);
	int64_t* p64 = st->alloc(m * sizeof *p64 + 1);
	int64_t* i64 = st->alloc(m * sizeof *i64 + 1);
	size_t* np = st->alloc(m * sizeof *np + 1);
	size_t* ni = st->alloc(m * sizeof *ni + 1);
	int rv = -1;
	if (rp && cols && vals && p64 && i64 && np && ni) {
		size_t t = 0;
		rp[0] = 0;
		for (size_t i = 0; i < m; i++) {
			size_t const r = i / 2, u = i % 2;
			for (int32_t e = h->rp[r]; e < h->rp[r + 1]; e++)
				for (int v = 0; v < 2; v++) {
					cols[t] = 2 * (int64_t) h->cols[e] + v;
					vals[t] = h->vals[4l * e + 2 * u + v];
					t++;
				}
			rp[i + 1] = (int64_t) t;
		}
		if (bfm_gpu_rcm_csr((int64_t) m, rp, cols, vals, p64, i64) == 0) {
			for (size_t i = 0; i < m; i++) {
				np[i] = (size_t) p64[i];
				ni[i] = (size_t) i64[i];
			}
			bfm_perm_destroy(perm);
			perm->perm = np;
			perm->inv_perm = ni;
			perm->has_perm = true;
			np = ni = NULL;
			rv = 0;
		}
	}
	if (rp) st->free(rp);
	if (cols) st->free(cols);
	if (vals) st->free(vals);
	if (p64) st->free(p64);
	if (i64) st->free(i64);
	if (np) st->free(np);
	if (ni) st->free(ni);
	return rv;
}

/* Renumbering a sparse matrix records the permutation (new = perm[old]); the
 * storage stays in the caller's order.  One renumbering at a time, forward. */
int bfmi_sparse_permute(bfm_perm_t* perm, bfm_matrix_t* A, bool inv) {
	sparse_t* h = handle_of(A);
	if (inv || !perm->has_perm || perm->m != A->m || h->perm) return -1;
	h->perm = perm->perm;
	h->inv = perm->inv_perm;
	return 0;
}

/* y <- A^-1 y with the GPU PCG (the options of bfm_gpu_get_opts; FP64);
 * y in the system's (renumbered) order. */
int bfmi_sparse_solve(bfm_matrix_t* A, bfm_vec_t* y) {
	sparse_t const* h = handle_of(A);
	bfm_state_t* const st = h->state;
	size_t const m = A->m;
	if (y->n != m) return -1;
	double* b = st->alloc(m * sizeof *b + 1);
	double* x = st->alloc(m * sizeof *x + 1);
	int rv = -1;
	if (b && x) {
		for (size_t i = 0; i < m; i++) b[i] = h->perm ? y->data[h->perm[i]] : y->data[i];
		bfm_gpu_opts_t o;
		bfm_gpu_get_opts(&o);
		int status = -1, iters = 0;
		double res = 0.0;
		if (bfmi_solve_rhs(h->P, b, x, &o, &status, &iters, &res) == 0) {
			// BFM_GPU_STAGNATED: the roundoff floor above rtol, the solution is usable
			if (status == BFM_GPU_OK || status == BFM_GPU_STAGNATED) {
				for (size_t i = 0; i < m; i++) {
					if (h->perm) y->data[h->perm[i]] = x[i];
					else y->data[i] = x[i];
				}
				rv = 0;
			}
			else {
				char msg[160];
				snprintf(msg, sizeof msg, "sparse solve: status %d after %d iterations (relative residual %g)", status,
				         iters, res);
				bfm_gpu_set_last_error(msg);
			}
		}
	}
	if (b) st->free(b);
	if (x) st->free(x);
	return rv;
}
