/* Permutations and RCM renumbering; ABI-identical to the reference's
 * libbfm/src/bfm/perm.h:6-22.  bfm_perm_rcm produces the reference's exact
 * permutation (bit-exact integer parity). */
#pragma once

#include <bfm/math.h>
#include <bfm/matrix.h>

typedef struct {
	bfm_state_t* state;
	size_t m;
	bool has_perm;
	size_t* perm;     /* new position of old index i */
	size_t* inv_perm; /* old index at new position p */
} bfm_perm_t;

int bfm_perm_create(bfm_perm_t* perm, bfm_state_t* state, size_t m);        /* ref perm.c:5-13    */
int bfm_perm_destroy(bfm_perm_t* perm);                                    /* ref perm.c:15-24   */
int bfm_perm_perm_matrix(bfm_perm_t* perm, bfm_matrix_t* matrix, bool inv); /* ref perm.c:26-68   */
int bfm_perm_perm_vec(bfm_perm_t* perm, bfm_vec_t* vec, bool inv);          /* ref perm.c:70-103  */
int bfm_perm_rcm(bfm_perm_t* perm, bfm_matrix_t* mat);                      /* ref perm.c:117-331 */
