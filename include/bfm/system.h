/* Assembled linear systems; ABI-identical to the reference's
 * libbfm/src/bfm/system.h:9-28.  The planar creators assemble on the GPU and
 * hand back the dense host matrix this struct can hold (small n only). */
#pragma once

#include <bfm/force.h>
#include <bfm/instance.h>
#include <bfm/math.h>
#include <bfm/matrix.h>
#include <bfm/perm.h>

typedef struct {
	bfm_state_t* state;
	size_t n;
	bfm_perm_t perm;
	bfm_matrix_t A;
	bfm_vec_t b;
} bfm_system_t;

int bfm_system_create(bfm_system_t* system, bfm_state_t* state, size_t n);  /* ref system.c:5-34  */
int bfm_system_destroy(bfm_system_t* system);                              /* ref system.c:36-42 */
int bfm_system_renumber(bfm_system_t* system);                             /* ref system.c:44-81 */
int bfm_system_create_planar_strain(bfm_system_t* system, bfm_instance_t* instance, size_t n_forces, bfm_force_t** forces);       /* ref system.c:531-533 */
int bfm_system_create_planar_stress(bfm_system_t* system, bfm_instance_t* instance, size_t n_forces, bfm_force_t** forces);       /* ref system.c:535-537 */
int bfm_system_create_axisymmetric_strain(bfm_system_t* system, bfm_instance_t* instance, size_t n_forces, bfm_force_t** forces); /* ref system.c:539-622 */
