/* Integration rules; ABI-identical to the reference's libbfm/src/bfm/rule.h:6-24. */
#pragma once

#include <bfm/mesh.h>
#include <bfm/shape.h>

typedef struct {
	bfm_state_t* state;
	size_t dim;
	bfm_elem_kind_t kind;
	size_t n_points;
	double* weights;
	double** points; /* points[q][d] */
	bfm_shape_t shape;
} bfm_rule_t;

int bfm_rule_create(bfm_rule_t* rule, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind, size_t n_points); /* ref rule.c:5-71    */
int bfm_rule_destroy(bfm_rule_t* rule);                                                                      /* ref rule.c:73-86   */
int bfm_rule_create_gauss_legendre(bfm_rule_t* rule, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind);  /* ref rule.c:113-151 */
