/* Isotropic material; ABI-identical to the reference's
 * libbfm/src/bfm/material.h:5-26. */
#pragma once

#include <bfm/bfm.h>

typedef struct {
	double r;
	double g;
	double b;
	double a;
} bfm_colour_t;

typedef struct {
	bfm_state_t* state;
	char* name;
	bfm_colour_t colour;
	double rho; /* density          */
	double E;   /* Young's modulus  */
	double nu;  /* Poisson's ratio  */
} bfm_material_t;

int bfm_material_create(bfm_material_t* material, bfm_state_t* state, char* name, double rho, double E, double nu); /* ref material.c:5-23  */
int bfm_material_destroy(bfm_material_t* material);                                                                  /* ref material.c:25-31 */
int bfm_material_set_colour(bfm_material_t* material, double r, double g, double b, double a);                      /* ref material.c:33-40 */
