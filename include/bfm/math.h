/* Small vector type and numeric helpers; ABI-identical to the reference's
 * libbfm/src/bfm/math.h:5-23. */
#pragma once

#include <bfm/bfm.h>

#define BFM_NAN (0. / 0.)
#define BFM_IS_NAN(x) ((x) != (x))
#define BFM_PIVOT_EPS 1e-20

#define BFM_MAX(a, b) ((a) > (b) ? (a) : (b))
#define BFM_MIN(a, b) ((a) < (b) ? (a) : (b))
#define BFM_ABS(a) ((a) < 0 ? -(a) : (a))

typedef struct {
	bfm_state_t* state;
	size_t n;
	double* data;
} bfm_vec_t;

int bfm_vec_create(bfm_vec_t* vec, bfm_state_t* state, size_t n); /* ref vec.c:5-18  */
int bfm_vec_copy(bfm_vec_t* vec, bfm_vec_t* src);                 /* ref vec.c:20-23 */
int bfm_vec_destroy(bfm_vec_t* vec);                              /* ref vec.c:25-32 */
