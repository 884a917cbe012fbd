/* Instance = object + conditions + result; ABI-identical to the reference's
 * libbfm/src/bfm/instance.h:6-23.  `effects` holds u,v per node (host FP64). */
#pragma once

#include <bfm/condition.h>
#include <bfm/obj.h>

typedef struct {
	bfm_state_t* state;
	bfm_obj_t* obj;
	size_t n_effects;
	double* effects;
	size_t n_conditions;
	bfm_condition_t** conditions;
} bfm_instance_t;

int bfm_instance_create(bfm_instance_t* instance, bfm_state_t* state, bfm_obj_t* obj);      /* ref instance.c:6-25  */
int bfm_instance_destroy(bfm_instance_t* instance);                                       /* ref instance.c:27-39 */
int bfm_instance_set_n_conditions(bfm_instance_t* instance, size_t n_conditions);         /* ref instance.c:41-59 */
int bfm_instance_add_condition(bfm_instance_t* instance, bfm_condition_t* condition);     /* ref instance.c:61-73 */
