/* Dense and band matrices, LU without pivoting, permutations and RCM: the
 * host-side linear-algebra utilities of libbfm's public API
 * (libbfm/src/matrix.c, perm.c).  They serve small dense systems returned by
 * the bfm_system_* creators; the GPU hot path never goes through them.
 *
 * Storage formats are part of the ABI (callers may read `data` directly) and
 * are kept as the reference defines them:
 *   full: row-major i*m+j, column-major i+j*m          (matrix.c:30)
 *   band: row-major j+i*2k, column-major i+j*2k        (matrix.c:208)
 */
#include <stdint.h>
#include <string.h>

#include <bfm/gpu.h>
#include <bfm/matrix.h>
#include <bfm/perm.h>

#include "internal.h"

static double* zalloc_d(bfm_state_t* state, size_t n) {
	double* p = state->alloc(n * sizeof *p);
	if (p) memset(p, 0, n * sizeof *p);
	return p;
}

static int in_band(bfm_matrix_t const* A, size_t i, size_t j) {
	size_t const d = i > j ? i - j : j - i;
	return d <= A->band.k;
}

static size_t full_index(bfm_matrix_t const* A, size_t i, size_t j) {
	return A->major == BFM_MATRIX_MAJOR_ROW ? i * A->m + j : i + j * A->m;
}

static size_t band_index(bfm_matrix_t const* A, size_t i, size_t j) {
	size_t const k2 = 2 * A->band.k;
	return A->major == BFM_MATRIX_MAJOR_ROW ? j + i * k2 : i + j * k2;
}

int bfm_matrix_full_create(bfm_matrix_t* A, bfm_state_t* state, bfm_matrix_major_t major, size_t m) {
	A->state = state;
	A->kind = BFM_MATRIX_KIND_FULL;
	A->major = major;
	A->m = m;
	A->full.data = zalloc_d(state, m * m);
	return A->full.data ? 0 : -1;
}

int bfm_matrix_band_create(bfm_matrix_t* A, bfm_state_t* state, bfm_matrix_major_t major, size_t m, size_t k) {
	A->state = state;
	A->kind = BFM_MATRIX_KIND_BAND;
	A->major = major;
	A->m = m;
	A->band.k = k;
	A->band.data = zalloc_d(state, m * (2 * k + 1));
	return A->band.data ? 0 : -1;
}

int bfm_matrix_destroy(bfm_matrix_t* A) {
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_destroy(A);
	if (A->kind == BFM_MATRIX_KIND_FULL) {
		A->state->free(A->full.data);
		A->full.data = NULL;
		return 0;
	}
	if (A->kind == BFM_MATRIX_KIND_BAND) {
		A->state->free(A->band.data);
		A->band.data = NULL;
		return 0;
	}
	return -1;
}

double bfm_matrix_get(bfm_matrix_t* A, size_t i, size_t j) {
	if (i >= A->m || j >= A->m) return BFM_NAN;
	if (A->kind == BFM_MATRIX_KIND_FULL) return A->full.data[full_index(A, i, j)];
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_get(A, i, j);
	if (A->kind == BFM_MATRIX_KIND_BAND) return in_band(A, i, j) ? A->band.data[band_index(A, i, j)] : 0.0;
	return -1;
}

int bfm_matrix_set(bfm_matrix_t* A, size_t i, size_t j, double v) {
	if (i >= A->m || j >= A->m) return -1;
	if (A->kind == BFM_MATRIX_KIND_FULL) {
		A->full.data[full_index(A, i, j)] = v;
		return 0;
	}
	if (A->kind == BFM_MATRIX_KIND_BAND) {
		if (!in_band(A, i, j)) return fabs(v) < BFM_PIVOT_EPS ? 0 : -1;
		A->band.data[band_index(A, i, j)] = v;
		return 0;
	}
	return -1;
}

int bfm_matrix_add(bfm_matrix_t* A, size_t i, size_t j, double v) {
	if (i >= A->m || j >= A->m) return -1;
	if (A->kind == BFM_MATRIX_KIND_FULL) {
		A->full.data[full_index(A, i, j)] += v;
		return 0;
	}
	if (A->kind == BFM_MATRIX_KIND_BAND) {
		if (!in_band(A, i, j)) return fabs(v) < BFM_PIVOT_EPS ? 0 : -1;
		A->band.data[band_index(A, i, j)] += v;
		return 0;
	}
	return -1;
}

size_t bfm_matrix_bandwidth(bfm_matrix_t* A) {
	if (A->kind == BFM_MATRIX_KIND_BAND) return A->band.k;
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_bandwidth(A);
	if (A->kind != BFM_MATRIX_KIND_FULL) return (size_t) -1;
	size_t k = 0;
	for (size_t i = 0; i < A->m; i++)
		for (size_t j = 0; j < A->m; j++) {
			size_t const d = i > j ? i - j : j - i;
			if (d > k && A->full.data[full_index(A, i, j)] != 0) k = d;
		}
	return k;
}

int bfm_matrix_copy(bfm_matrix_t* A, bfm_matrix_t* src) {
	if (A->m != src->m || A->kind == BFM_MATRIX_KIND_SPARSE) return -1;  // sparse matrices are read-only
	if (A->kind == BFM_MATRIX_KIND_FULL && src->kind == BFM_MATRIX_KIND_FULL) {
		memcpy(A->full.data, src->full.data, src->m * src->m * sizeof(double));
		return 0;
	}
	if (A->kind == BFM_MATRIX_KIND_BAND && src->kind == BFM_MATRIX_KIND_BAND) {
		if (A->band.k != src->band.k) return -1;
		memcpy(A->band.data, src->band.data, src->m * (2 * src->band.k + 1) * sizeof(double));
		return 0;
	}
	for (size_t i = 0; i < A->m; i++)
		for (size_t j = 0; j < A->m; j++) {
			double const v = bfm_matrix_get(src, i, j);
			if (BFM_IS_NAN(v) || bfm_matrix_set(A, i, j, v) < 0) return -1;
		}
	return 0;
}

/* In-place Doolittle LU without pivoting (ref matrix.c:73-121, 253-302): the
 * multipliers replace the strict lower part; fails on a pivot below 1e-20.
 * The band form restricts every row operation to the band. */
int bfm_matrix_lu(bfm_matrix_t* A) {
	size_t const m = A->m;
	size_t const k = A->kind == BFM_MATRIX_KIND_BAND ? A->band.k : m;
	if (A->kind != BFM_MATRIX_KIND_FULL && A->kind != BFM_MATRIX_KIND_BAND) return -1;
	for (size_t p = 0; p + 1 < m; p++) {
		double const piv = bfm_matrix_get(A, p, p);
		if (BFM_IS_NAN(piv) || fabs(piv) < BFM_PIVOT_EPS) return -1;
		size_t const end = p + k + 1 < m ? p + k + 1 : m;
		for (size_t i = p + 1; i < end; i++) {
			double const below = bfm_matrix_get(A, i, p);
			if (BFM_IS_NAN(below)) return -1;
			double const f = below / piv;
			if (bfm_matrix_set(A, i, p, f) < 0) return -1;
			for (size_t j = p + 1; j < end; j++) {
				double const u = bfm_matrix_get(A, p, j);
				if (BFM_IS_NAN(u) || bfm_matrix_add(A, i, j, -f * u) < 0) return -1;
			}
		}
	}
	return 0;
}

/* Forward (unit lower) then backward substitution, in place
 * (ref matrix.c:123-174, 351-404). */
int bfm_matrix_lu_solve(bfm_matrix_t* A, bfm_vec_t* y) {
	if (A->m != y->n) return -1;
	if (A->kind != BFM_MATRIX_KIND_FULL && A->kind != BFM_MATRIX_KIND_BAND) return -1;
	size_t const m = A->m;
	size_t const k = A->kind == BFM_MATRIX_KIND_BAND ? A->band.k : m;
	double* const v = y->data;
	for (size_t p = 0; p < m; p++) {
		size_t const lo = p > k ? p - k : 0;
		for (size_t i = lo; i < p; i++) {
			double const l = bfm_matrix_get(A, p, i);
			if (BFM_IS_NAN(l)) return -1;
			v[p] -= l * v[i];
		}
	}
	for (size_t pp = m; pp-- > 0;) {
		size_t const hi = pp + k + 1 < m ? pp + k + 1 : m;
		for (size_t i = pp + 1; i < hi; i++) {
			double const u = bfm_matrix_get(A, pp, i);
			if (BFM_IS_NAN(u)) return -1;
			v[pp] -= v[i] * u;
		}
		double const piv = bfm_matrix_get(A, pp, pp);
		if (BFM_IS_NAN(piv) || piv == 0) return -1;
		v[pp] /= piv;
	}
	return 0;
}

int bfm_matrix_solve(bfm_matrix_t* A, bfm_vec_t* y) {
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_solve(A, y);  // the GPU PCG, not a factorization
	if (bfm_matrix_lu(A) < 0) return -1;
	return bfm_matrix_lu_solve(A, y);
}

/* ---------------------------------------------------------------- permutations (ref perm.c) */

int bfm_perm_create(bfm_perm_t* perm, bfm_state_t* state, size_t m) {
	memset(perm, 0, sizeof *perm);
	perm->state = state;
	perm->m = m;
	return 0;
}

int bfm_perm_destroy(bfm_perm_t* perm) {
	if (perm->has_perm) {
		perm->state->free(perm->perm);
		perm->state->free(perm->inv_perm);
	}
	perm->has_perm = false;
	perm->perm = perm->inv_perm = NULL;
	return 0;
}

/* new[p[i]][p[j]] = old[i][j] with p = perm (or inv_perm) */
int bfm_perm_perm_matrix(bfm_perm_t* perm, bfm_matrix_t* A, bool inv) {
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_permute(perm, A, inv);
	if (!perm->has_perm || A->m != perm->m || A->kind != BFM_MATRIX_KIND_FULL) return -1;
	size_t const m = A->m;
	size_t const* p = inv ? perm->inv_perm : perm->perm;
	double* old = perm->state->alloc(m * m * sizeof *old + 1);
	if (!old) return -1;
	memcpy(old, A->full.data, m * m * sizeof *old);
	for (size_t i = 0; i < m; i++)
		for (size_t j = 0; j < m; j++) A->full.data[full_index(A, p[i], p[j])] = old[full_index(A, i, j)];
	perm->state->free(old);
	return 0;
}

/* new[p[i]] = old[i] */
int bfm_perm_perm_vec(bfm_perm_t* perm, bfm_vec_t* vec, bool inv) {
	if (!perm->has_perm || vec->n != perm->m) return -1;
	size_t const m = vec->n;
	size_t const* p = inv ? perm->inv_perm : perm->perm;
	double* old = perm->state->alloc(m * sizeof *old + 1);
	if (!old) return -1;
	memcpy(old, vec->data, m * sizeof *old);
	for (size_t i = 0; i < m; i++) vec->data[p[i]] = old[i];
	perm->state->free(old);
	return 0;
}

/* RCM of a full or band matrix: its numeric nonzeros go to CSR (one O(m^2)
 * scan, unavoidable for dense input), then the sparse bit-exact RCM. */
int bfm_perm_rcm(bfm_perm_t* perm, bfm_matrix_t* A) {
	if (A->kind == BFM_MATRIX_KIND_SPARSE) return bfmi_sparse_rcm(perm, A);
	size_t const m = A->m;
	if (perm->m != m) return -1;
	bfm_state_t* const state = perm->state;
	int64_t* row_ptr = state->alloc((m + 1) * sizeof *row_ptr);
	if (!row_ptr) return -1;
	size_t nnz = 0;
	row_ptr[0] = 0;
	for (size_t i = 0; i < m; i++) {
		size_t const lo = A->kind == BFM_MATRIX_KIND_BAND && i > A->band.k ? i - A->band.k : 0;
		size_t const hi = A->kind == BFM_MATRIX_KIND_BAND && i + A->band.k + 1 < m ? i + A->band.k + 1 : m;
		for (size_t j = lo; j < hi; j++) nnz += bfm_matrix_get(A, i, j) != 0;
		row_ptr[i + 1] = (int64_t) nnz;
	}
	int64_t* cols = state->alloc(nnz * sizeof *cols + 1);
	double* vals = state->alloc(nnz * sizeof *vals + 1);
	size_t* np = state->alloc(m * sizeof *np + 1);
	size_t* ni = state->alloc(m * sizeof *ni + 1);
	int64_t* p64 = state->alloc(m * sizeof *p64 + 1);
	int64_t* i64 = state->alloc(m * sizeof *i64 + 1);
	int rv = -1;
	if (cols && vals && np && ni && p64 && i64) {
		size_t t = 0;
		for (size_t i = 0; i < m; i++) {
			size_t const lo = A->kind == BFM_MATRIX_KIND_BAND && i > A->band.k ? i - A->band.k : 0;
			size_t const hi = A->kind == BFM_MATRIX_KIND_BAND && i + A->band.k + 1 < m ? i + A->band.k + 1 : m;
			for (size_t j = lo; j < hi; j++) {
				double const v = bfm_matrix_get(A, i, j);
				if (v != 0) {
					cols[t] = (int64_t) j;
					vals[t] = v;
					t++;
				}
			}
		}
		if (bfm_gpu_rcm_csr((int64_t) m, row_ptr, cols, vals, p64, i64) == 0) {
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
	state->free(row_ptr);
	if (cols) state->free(cols);
	if (vals) state->free(vals);
	if (np) state->free(np);
	if (ni) state->free(ni);
	if (p64) state->free(p64);
	if (i64) state->free(i64);
	return rv;
}
