/* Dense and band matrices (host); ABI-identical to the reference's
 * libbfm/src/bfm/matrix.h:10-127.  These stay host-side utilities: the GPU
 * hot path stores its stiffness matrix as 2x2-block CSR on the device. */
#pragma once

#include <math.h>
#include <stdbool.h>
#include <sys/types.h>

#include <bfm/bfm.h>
#include <bfm/math.h>

typedef enum {
	BFM_MATRIX_KIND_FULL,
	BFM_MATRIX_KIND_BAND,
	/* Additive (not in the reference): the stiffness matrix of a
	 * bfm_system_create_planar_* system kept sparse -- 2x2-block CSR in GPU
	 * memory with a host copy, O(nnz) storage where FULL needs n^2.  Read-only
	 * (bfm_matrix_set/add return -1); bfm_matrix_solve solves it with the GPU
	 * PCG (bfm_gpu_get_opts: rtol, preconditioner) instead of a band LU. */
	BFM_MATRIX_KIND_SPARSE,
} bfm_matrix_kind_t;

typedef enum {
	BFM_MATRIX_MAJOR_ROW,
	BFM_MATRIX_MAJOR_COLUMN,
} bfm_matrix_major_t;

typedef struct {
	double* data;
} bfm_matrix_full_t;

typedef struct {
	size_t k; /* half bandwidth */
	double* data;
} bfm_matrix_band_t;

typedef struct {
	void* handle; /* the library's sparse matrix object           */
	size_t nnz;   /* stored scalar entries (4 per 2x2 block)       */
} bfm_matrix_sparse_t;

typedef struct {
	bfm_state_t* state;
	bfm_matrix_kind_t kind;
	bfm_matrix_major_t major;
	size_t m;
	union {
		bfm_matrix_full_t full;
		bfm_matrix_band_t band;
		bfm_matrix_sparse_t sparse; /* same size as band: the struct keeps its layout */
	};
} bfm_matrix_t;

int bfm_matrix_full_create(bfm_matrix_t* matrix, bfm_state_t* state, bfm_matrix_major_t major, size_t m);           /* ref matrix.c:555-568 */
int bfm_matrix_band_create(bfm_matrix_t* matrix, bfm_state_t* state, bfm_matrix_major_t major, size_t m, size_t k); /* ref matrix.c:570-584 */
int bfm_matrix_copy(bfm_matrix_t* matrix, bfm_matrix_t* src);          /* ref matrix.c:408-441 */
int bfm_matrix_destroy(bfm_matrix_t* matrix);                          /* ref matrix.c:443-453 */
double bfm_matrix_get(bfm_matrix_t* matrix, size_t i, size_t j);       /* ref matrix.c:455-465; NaN out of range */
int bfm_matrix_set(bfm_matrix_t* matrix, size_t i, size_t j, double val); /* ref matrix.c:467-477 */
int bfm_matrix_add(bfm_matrix_t* matrix, size_t i, size_t j, double val); /* ref matrix.c:479-489 */
size_t bfm_matrix_bandwidth(bfm_matrix_t* matrix);                     /* ref matrix.c:491-501 */
int bfm_matrix_lu(bfm_matrix_t* matrix);                               /* ref matrix.c:503-513; no pivoting */
int bfm_matrix_lu_solve(bfm_matrix_t* matrix, bfm_vec_t* y);           /* ref matrix.c:515-529 */
int bfm_matrix_solve(bfm_matrix_t* matrix, bfm_vec_t* y);              /* ref matrix.c:531-541 */
