/* libbfm's small host-side objects: state, vectors, materials, shapes,
 * integration rules, forces, conditions, objects, instances, simulations and
 * meshes.  Written from the public header contracts (include/bfm/*.h, which
 * are ABI-identical to the reference's libbfm/src/bfm/*.h); each function
 * cites the reference function whose behaviour it keeps.
 *
 * All host buffers come from state->alloc/realloc/free, as in the reference.
 */
#include <stdio.h>
#include <string.h>

#include <bfm/bfm.h>
#include <bfm/condition.h>
#include <bfm/force.h>
#include <bfm/instance.h>
#include <bfm/material.h>
#include <bfm/math.h>
#include <bfm/mesh.h>
#include <bfm/obj.h>
#include <bfm/rule.h>
#include <bfm/shape.h>
#include <bfm/sim.h>

/* ---------------------------------------------------------------- state (ref state.c) */

int bfm_state_create(bfm_state_t* state) {
	memset(state, 0, sizeof *state);
	state->alloc = malloc;
	state->realloc = realloc;
	state->free = free;
	return 0;
}

int bfm_state_destroy(bfm_state_t* state) {
	(void) state;
	return 0;
}

int bfm_set_alloc(bfm_state_t* state, bfm_alloc_t alloc) {
	state->alloc = alloc;
	return 0;
}

int bfm_set_realloc(bfm_state_t* state, bfm_realloc_t re) {
	state->realloc = re;
	return 0;
}

int bfm_set_free(bfm_state_t* state, bfm_free_t fr) {
	state->free = fr;
	return 0;
}

int bfm_err_print(bfm_state_t* state) {
	bfm_err_t const* e = &state->err;
	if (e->has) printf("[BFM %s:%zu (%s)] %s\n", e->file, e->line, e->func, e->msg);
	return 0;
}

/* ---------------------------------------------------------------- vec (ref vec.c) */

static void* zalloc(bfm_state_t* state, size_t size) {
	void* p = state->alloc(size);
	if (p) memset(p, 0, size);
	return p;
}

int bfm_vec_create(bfm_vec_t* vec, bfm_state_t* state, size_t n) {
	vec->state = state;
	vec->n = n;
	vec->data = zalloc(state, n * sizeof *vec->data);
	return vec->data ? 0 : -1;
}

int bfm_vec_copy(bfm_vec_t* vec, bfm_vec_t* src) {
	memcpy(vec->data, src->data, src->n * sizeof *vec->data);
	return 0;
}

int bfm_vec_destroy(bfm_vec_t* vec) {
	vec->state->free(vec->data);
	vec->data = NULL;
	return 0;
}

/* ---------------------------------------------------------------- material (ref material.c) */

int bfm_material_create(bfm_material_t* m, bfm_state_t* state, char* name, double rho, double E, double nu) {
	memset(m, 0, sizeof *m);
	m->state = state;
	size_t const len = strlen(name) + 1;
	/* the reference strdup()s the name but frees it through state->free; take it from state->alloc */
	m->name = state->alloc(len);
	if (!m->name) return -1;
	memcpy(m->name, name, len);
	m->rho = rho;
	m->E = E;
	m->nu = nu;
	return 0;
}

int bfm_material_destroy(bfm_material_t* m) {
	m->state->free(m->name);
	m->name = NULL;
	return 0;
}

int bfm_material_set_colour(bfm_material_t* m, double r, double g, double b, double a) {
	m->colour.r = r;
	m->colour.g = g;
	m->colour.b = b;
	m->colour.a = a;
	return 0;
}

/* ---------------------------------------------------------------- shape (ref shape.c:3-105) */

/* Linear triangle on the reference triangle (0,0),(1,0),(0,1); bilinear quad
 * on [-1,1]^2 with local nodes (+,+), (-,+), (-,-), (+,-). */
static int lagrange_phi(bfm_shape_t* shape, double* pt, double* phi) {
	if (shape->dim != 2) return -1;
	double const u = pt[0], v = pt[1];
	switch (shape->kind) {
	case BFM_ELEM_KIND_SIMPLEX:
		phi[0] = 1 - u - v;
		phi[1] = u;
		phi[2] = v;
		return 0;
	case BFM_ELEM_KIND_QUAD:
		phi[0] = (1 + u) * (1 + v) / 4;
		phi[1] = (1 - u) * (1 + v) / 4;
		phi[2] = (1 - u) * (1 - v) / 4;
		phi[3] = (1 + u) * (1 - v) / 4;
		return 0;
	case BFM_ELEM_KIND_QUADRATIC_TRIANGLE:
		/* values are given, but the element is unsupported (as in the reference) */
		phi[0] = 1 - 3 * (u + v) + 2 * (u + v) * (u + v);
		phi[1] = u * (2 * u - 1);
		phi[2] = v * (2 * v - 1);
		phi[3] = 4 * u * (1 - u - v);
		phi[4] = 4 * u * v;
		phi[5] = 4 * v * (1 - u - v);
		return -1;
	}
	return -1;
}

static int lagrange_dphi(bfm_shape_t* shape, size_t wrt, double* pt, double* d) {
	if (shape->dim != 2) return -1;
	double const u = pt[0], v = pt[1];
	switch (shape->kind) {
	case BFM_ELEM_KIND_SIMPLEX:
		d[0] = -1;
		d[1] = wrt == 0 ? 1 : 0;
		d[2] = wrt == 0 ? 0 : 1;
		return 0;
	case BFM_ELEM_KIND_QUAD:
		if (wrt == 0) {
			d[0] = (1 + v) / 4;
			d[1] = (-1 - v) / 4;
			d[2] = (-1 + v) / 4;
			d[3] = (1 - v) / 4;
		}
		else {
			d[0] = (1 + u) / 4;
			d[1] = (1 - u) / 4;
			d[2] = (-1 + u) / 4;
			d[3] = (-1 - u) / 4;
		}
		return 0;
	case BFM_ELEM_KIND_QUADRATIC_TRIANGLE:
		return -1;
	}
	return -1;
}

int bfm_shape_create(bfm_shape_t* shape, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind) {
	shape->state = state;
	shape->dim = dim;
	shape->kind = kind;
	shape->phi = lagrange_phi;
	shape->dphi = lagrange_dphi;
	return 0;
}

int bfm_shape_destroy(bfm_shape_t* shape) {
	(void) shape;
	return 0;
}

/* ---------------------------------------------------------------- rule (ref rule.c) */

int bfm_rule_create(bfm_rule_t* rule, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind, size_t n_points) {
	memset(rule, 0, sizeof *rule);
	rule->state = state;
	rule->dim = dim;
	rule->kind = kind;
	rule->n_points = n_points;
	rule->weights = zalloc(state, n_points * sizeof *rule->weights);
	rule->points = zalloc(state, n_points * sizeof *rule->points);
	if (!rule->weights || !rule->points) goto fail;
	for (size_t q = 0; q < n_points; q++) {
		rule->points[q] = zalloc(state, dim * sizeof **rule->points);
		if (!rule->points[q]) goto fail;
	}
	if (bfm_shape_create(&rule->shape, state, dim, kind) < 0) goto fail;
	return 0;
fail:
	if (rule->points)
		for (size_t q = 0; q < n_points; q++)
			if (rule->points[q]) state->free(rule->points[q]);
	if (rule->points) state->free(rule->points);
	if (rule->weights) state->free(rule->weights);
	rule->points = NULL;
	rule->weights = NULL;
	return -1;
}

int bfm_rule_destroy(bfm_rule_t* rule) {
	bfm_state_t* const state = rule->state;
	if (rule->points) {
		for (size_t q = 0; q < rule->n_points; q++) state->free(rule->points[q]);
		state->free(rule->points);
	}
	state->free(rule->weights);
	rule->points = NULL;
	rule->weights = NULL;
	bfm_shape_destroy(&rule->shape);
	return 0;
}

/* Gauss points and weights: the numbers of the reference's tables
 * (rule.c:90-111), including its 15-digit literal for 1/sqrt(3), so that
 * results agree with it to the last bit. */
int bfm_rule_create_gauss_legendre(bfm_rule_t* rule, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind) {
	if (dim != 2 || (kind != BFM_ELEM_KIND_SIMPLEX && kind != BFM_ELEM_KIND_QUAD)) return -1;
	size_t const nq = (size_t) kind;
	if (bfm_rule_create(rule, state, dim, kind, nq) < 0) return -1;
	if (kind == BFM_ELEM_KIND_SIMPLEX) {
		double const a = 1. / 6, b = 1 - 1. / 3;
		double const xy[3][2] = {{a, a}, {b, a}, {a, b}};
		for (size_t q = 0; q < 3; q++) {
			rule->weights[q] = a;
			rule->points[q][0] = xy[q][0];
			rule->points[q][1] = xy[q][1];
		}
	}
	else {
		double const g = 0.577350269189626;
		double const xy[4][2] = {{-g, g}, {-g, -g}, {g, -g}, {g, g}};
		for (size_t q = 0; q < 4; q++) {
			rule->weights[q] = 1;
			rule->points[q][0] = xy[q][0];
			rule->points[q][1] = xy[q][1];
		}
	}
	return 0;
}

/* ---------------------------------------------------------------- force (ref force.c) */

int bfm_force_create(bfm_force_t* force, bfm_state_t* state, size_t dim) {
	memset(force, 0, sizeof *force);
	force->state = state;
	force->dim = dim;
	return 0;
}

int bfm_force_destroy(bfm_force_t* force) {
	if (force->kind == BFM_FORCE_KIND_LINEAR && force->linear.force.data) bfm_vec_destroy(&force->linear.force);
	return 0;
}

int bfm_force_set_none(bfm_force_t* force) {
	force->kind = BFM_FORCE_KIND_NONE;
	return 0;
}

int bfm_force_set_linear(bfm_force_t* force, bfm_vec_t* vec) {
	force->kind = BFM_FORCE_KIND_LINEAR;
	if (vec->n != force->dim) return -1;
	if (bfm_vec_create(&force->linear.force, vec->state, vec->n) < 0) return -1;
	return bfm_vec_copy(&force->linear.force, vec);
}

int bfm_force_set_funky(bfm_force_t* force, bfm_force_funky_func_t func, void* data) {
	force->kind = BFM_FORCE_KIND_FUNKY;
	force->funky.func = func;
	force->funky.data = data;
	return 0;
}

/* Value of a force at a position (ref force.c:79-99).  The reference's linear
 * case copies the value and then returns -1; here it returns 0. */
int bfm_force_eval(bfm_force_t* force, bfm_vec_t* pos, bfm_vec_t* out) {
	if (out->n != force->dim) return -1;
	switch (force->kind) {
	case BFM_FORCE_KIND_NONE:
		memset(out->data, 0, out->n * sizeof *out->data);
		return 0;
	case BFM_FORCE_KIND_LINEAR:
		return bfm_vec_copy(out, &force->linear.force);
	case BFM_FORCE_KIND_FUNKY:
		return force->funky.func(force, pos, out, force->funky.data);
	}
	return -1;
}

/* ---------------------------------------------------------------- condition (ref condition.c) */

int bfm_condition_create(bfm_condition_t* c, bfm_state_t* state, bfm_mesh_t* mesh, bfm_condition_kind_t kind) {
	c->state = state;
	c->mesh = mesh;
	c->kind = kind;
	c->value = 0;
	c->nodes = zalloc(state, mesh->n_nodes * sizeof *c->nodes);
	return c->nodes || !mesh->n_nodes ? 0 : -1;
}

int bfm_condition_destroy(bfm_condition_t* c) {
	c->state->free(c->nodes);
	c->nodes = NULL;
	return 0;
}

/* ---------------------------------------------------------------- obj, instance (ref obj.c, instance.c) */

int bfm_obj_create(bfm_obj_t* obj, bfm_state_t* state, bfm_mesh_t* mesh, bfm_material_t* material, bfm_rule_t* rule) {
	obj->state = state;
	obj->mesh = mesh;
	obj->material = material;
	obj->rule = rule;
	return 0;
}

int bfm_obj_destroy(bfm_obj_t* obj) {
	(void) obj;
	return 0;
}

int bfm_instance_create(bfm_instance_t* inst, bfm_state_t* state, bfm_obj_t* obj) {
	memset(inst, 0, sizeof *inst);
	inst->state = state;
	inst->obj = obj;
	inst->n_effects = obj->mesh->n_nodes * obj->mesh->dim;
	inst->effects = zalloc(state, inst->n_effects * sizeof *inst->effects);
	return inst->effects || !inst->n_effects ? 0 : -1;
}

int bfm_instance_destroy(bfm_instance_t* inst) {
	bfm_state_t* const state = inst->state;
	if (inst->effects) state->free(inst->effects);
	if (inst->conditions) state->free(inst->conditions);
	inst->effects = NULL;
	inst->conditions = NULL;
	return 0;
}

int bfm_instance_set_n_conditions(bfm_instance_t* inst, size_t n) {
	bfm_state_t* const state = inst->state;
	if (inst->conditions) state->free(inst->conditions);
	inst->n_conditions = n;
	inst->conditions = zalloc(state, n * sizeof *inst->conditions);
	return inst->conditions ? 0 : -1;
}

int bfm_instance_add_condition(bfm_instance_t* inst, bfm_condition_t* c) {
	bfm_condition_t** grown = inst->state->realloc(inst->conditions, (inst->n_conditions + 1) * sizeof *grown);
	if (!grown) return -1;
	inst->conditions = grown;
	inst->conditions[inst->n_conditions++] = c;
	return 0;
}

/* ---------------------------------------------------------------- sim bookkeeping (ref sim.c:8-97) */

int bfm_sim_create(bfm_sim_t* sim, bfm_state_t* state, bfm_sim_kind_t kind) {
	memset(sim, 0, sizeof *sim);
	sim->state = state;
	sim->kind = kind;
	return 0;
}

int bfm_sim_destroy(bfm_sim_t* sim) {
	bfm_state_t* const state = sim->state;
	if (sim->instances) state->free(sim->instances);
	if (sim->forces) state->free(sim->forces);
	sim->instances = NULL;
	sim->forces = NULL;
	return 0;
}

int bfm_sim_set_n_instances(bfm_sim_t* sim, size_t n) {
	bfm_state_t* const state = sim->state;
	if (sim->instances) state->free(sim->instances);
	sim->n_instances = n;
	sim->instances = zalloc(state, n * sizeof *sim->instances);
	return sim->instances ? 0 : -1;
}

int bfm_sim_add_instance(bfm_sim_t* sim, bfm_instance_t* inst) {
	bfm_instance_t** grown = sim->state->realloc(sim->instances, (sim->n_instances + 1) * sizeof *grown);
	if (!grown) return -1;
	sim->instances = grown;
	sim->instances[sim->n_instances++] = inst;
	return 0;
}

int bfm_sim_set_n_forces(bfm_sim_t* sim, size_t n) {
	bfm_state_t* const state = sim->state;
	if (sim->forces) state->free(sim->forces);
	sim->n_forces = n;
	sim->forces = zalloc(state, n * sizeof *sim->forces);
	return sim->forces ? 0 : -1;
}

int bfm_sim_add_force(bfm_sim_t* sim, bfm_force_t* force) {
	bfm_force_t** grown = sim->state->realloc(sim->forces, (sim->n_forces + 1) * sizeof *grown);
	if (!grown) return -1;
	sim->forces = grown;
	sim->forces[sim->n_forces++] = force;
	return 0;
}

/* ---------------------------------------------------------------- mesh lifetime (ref mesh.c:6-30) */

int bfm_mesh_create(bfm_mesh_t* mesh, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind) {
	memset(mesh, 0, sizeof *mesh);
	mesh->state = state;
	mesh->dim = dim;
	mesh->kind = kind;
	return 0;
}

int bfm_mesh_destroy(bfm_mesh_t* mesh) {
	bfm_state_t* const state = mesh->state;
	state->free(mesh->coords);
	state->free(mesh->elems);
	state->free(mesh->edges);
	if (mesh->domains)
		for (size_t i = 0; i < mesh->n_domains; i++) state->free(mesh->domains[i].elements);
	state->free(mesh->domains);
	mesh->coords = NULL;
	mesh->elems = NULL;
	mesh->edges = NULL;
	mesh->domains = NULL;
	return 0;
}
