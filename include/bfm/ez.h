/* LEPL1110 problem-file front end; ABI-identical to the reference's
 * libbfm/src/bfm/ez.h:11-29. */
#pragma once

#include <bfm/condition.h>
#include <bfm/instance.h>
#include <bfm/material.h>
#include <bfm/mesh.h>
#include <bfm/obj.h>
#include <bfm/rule.h>
#include <bfm/sim.h>

typedef struct {
	bfm_state_t* state;
	bfm_mesh_t* mesh;
	size_t n_conditions;
	bfm_condition_t* conditions;
	bfm_force_t gravity;
	bfm_material_t material;
	bfm_rule_t rule;
	bfm_obj_t obj;
	bfm_instance_t instance;
	bfm_sim_t sim;
} bfm_ez_lepl1110_t;

int bfm_ez_lepl1110_create(bfm_ez_lepl1110_t* ez, bfm_state_t* state, bfm_mesh_t* mesh, char* name); /* ref ez.c:6-189   */
int bfm_ez_lepl1110_destroy(bfm_ez_lepl1110_t* ez);                                                 /* ref ez.c:191-209 */
int bfm_ez_lepl1110_write(bfm_ez_lepl1110_t* ez, size_t shift, char const* filename);               /* ref ez.c:211-229 */
