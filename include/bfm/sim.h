/* Simulation driver; ABI-identical to the reference's libbfm/src/bfm/sim.h:6-33.
 * bfm_sim_run is the hot entry: here it assembles and solves every instance on
 * the GPU (2x2-block CSR, Dirichlet elimination, preconditioned CG) and copies
 * the displacements into instance->effects.  There is no CPU fallback: without
 * a usable GPU it returns -1 and fills state->err. */
#pragma once

#include <bfm/force.h>
#include <bfm/instance.h>

typedef enum {
	BFM_SIM_KIND_NONE = 0,
	BFM_SIM_KIND_PLANAR_STRAIN = 1,
	BFM_SIM_KIND_PLANAR_STRESS = 2,
	BFM_SIM_KIND_AXISYMMETRIC_STRAIN = 3,
} bfm_sim_kind_t;

typedef struct {
	bfm_state_t* state;
	bfm_sim_kind_t kind;
	size_t n_instances;
	bfm_instance_t** instances;
	size_t n_forces;
	bfm_force_t** forces;
} bfm_sim_t;

int bfm_sim_create(bfm_sim_t* sim, bfm_state_t* state, bfm_sim_kind_t kind); /* ref sim.c:8-15    */
int bfm_sim_destroy(bfm_sim_t* sim);                                        /* ref sim.c:17-29   */
int bfm_sim_set_n_instances(bfm_sim_t* sim, size_t n_instances);            /* ref sim.c:31-49   */
int bfm_sim_add_instance(bfm_sim_t* sim, bfm_instance_t* instance);         /* ref sim.c:51-63   */
int bfm_sim_set_n_forces(bfm_sim_t* sim, size_t n_forces);                  /* ref sim.c:65-83   */
int bfm_sim_add_force(bfm_sim_t* sim, bfm_force_t* force);                  /* ref sim.c:85-97   */
int bfm_sim_run(bfm_sim_t* sim);                                            /* ref sim.c:137-155 */
