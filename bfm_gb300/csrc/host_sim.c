/* The hot entry of libbfm on the GPU: bfm_sim_run (reference sim.c:103-155)
 * and the planar bfm_system_* creators (system.c:427-538), both driven
 * through the device-problem API of include/bfm/gpu.h.
 *
 * Per instance the host only gathers what the GPU needs from the libbfm
 * structures (int32 connectivity, shape values sampled at the rule's points,
 * constant or per-node forces, condition masks, edges); pattern, element
 * loop, conditions and the solve all run on the device.  There is no CPU
 * fallback: without a GPU, bfm_sim_run returns -1 and fills state->err.
 */
#include <limits.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <bfm/gpu.h>
#include <bfm/sim.h>
#include <bfm/system.h>

#include "internal.h"
#include "trace.h"

/* ---------------------------------------------------------------- errors and options */

static _Thread_local char t_msg[512];
static _Thread_local bfm_gpu_opts_t t_opts;
static _Thread_local int t_opts_set;
static _Thread_local bfm_gpu_stats_t t_stats;
static _Thread_local int t_storage = -1;  /* system matrix storage: -1 = not set (environment) */

int bfm_gpu_set_system_storage(int kind) {
	if (kind != BFM_MATRIX_KIND_FULL && kind != BFM_MATRIX_KIND_SPARSE) return -1;
	t_storage = kind;
	return 0;
}

/* sparse storage: asked for, or a dense n x n matrix above 16 GB */
static int sparse_system(size_t n) {
	int kind = t_storage;
	if (kind < 0) {
		char const* e = getenv("BFM_GPU_SYSTEM_STORAGE");
		kind = e && !strcmp(e, "sparse") ? BFM_MATRIX_KIND_SPARSE : BFM_MATRIX_KIND_FULL;
	}
	return kind == BFM_MATRIX_KIND_SPARSE || (double) n * (double) n * sizeof(double) > 16e9;
}

static int report(bfm_state_t* state, char const* func, int line, char const* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(t_msg, sizeof t_msg, fmt, ap);
	va_end(ap);
	if (state) {
		state->err.has = true;
		state->err.msg = t_msg;
		state->err.file = __FILE__;
		state->err.func = func;
		state->err.line = (size_t) line;
	}
	return -1;
}

#define REPORT(state, ...) report(state, __func__, __LINE__, __VA_ARGS__)

static bfm_gpu_opts_t current_opts(void) {
	if (!t_opts_set) {
		bfm_gpu_default_opts(&t_opts);
		char const* p = getenv("BFM_GPU_PRECISION");
		if (p && (!strcmp(p, "mixed") || !strcmp(p, "1"))) t_opts.precision = BFM_GPU_MIXED;
		if (p && (!strcmp(p, "mixed_exact") || !strcmp(p, "2"))) t_opts.precision = BFM_GPU_MIXED_EXACT;
		if (p && (!strcmp(p, "df") || !strcmp(p, "3"))) t_opts.precision = BFM_GPU_FP64_DF;
		char const* r = getenv("BFM_GPU_RTOL");
		if (r) t_opts.rtol = strtod(r, NULL);
		char const* pc = getenv("BFM_GPU_PRECOND");
		if (pc && (!strcmp(pc, "block") || !strcmp(pc, "1"))) t_opts.precond = BFM_GPU_PC_BLOCK_JACOBI;
		if (pc && (!strcmp(pc, "learned") || !strcmp(pc, "2"))) t_opts.precond = BFM_GPU_PC_LEARNED;
		if (pc && (!strcmp(pc, "ssor") || !strcmp(pc, "3"))) t_opts.precond = BFM_GPU_PC_SSOR;
		if (pc && (!strcmp(pc, "learned_ssor") || !strcmp(pc, "4"))) t_opts.precond = BFM_GPU_PC_LEARNED_SSOR;
		if (pc && (!strcmp(pc, "ssor2") || !strcmp(pc, "5"))) t_opts.precond = BFM_GPU_PC_SSOR2;
		if (pc && (!strcmp(pc, "learned_ssor2") || !strcmp(pc, "6"))) t_opts.precond = BFM_GPU_PC_LEARNED_SSOR2;
		t_opts_set = 1;
	}
	return t_opts;
}

int bfm_gpu_set_opts(const bfm_gpu_opts_t* opts) {
	t_opts = *opts;
	t_opts_set = 1;
	return 0;
}

int bfm_gpu_get_opts(bfm_gpu_opts_t* opts) {
	*opts = current_opts();
	return 0;
}

int bfm_gpu_last_stats(bfm_gpu_stats_t* stats) {
	*stats = t_stats;
	return 0;
}

/* ---------------------------------------------------------------- per-element material registry */

typedef struct {
	bfm_instance_t* inst;
	const double* E;
	const double* nu;
} elem_mat_t;

static elem_mat_t g_elem_mat[64];
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

int bfm_gpu_instance_set_elem_material(bfm_instance_t* inst, const double* E, const double* nu) {
	pthread_mutex_lock(&g_lock);
	int rv = -1;
	for (int i = 0; i < 64; i++)
		if (g_elem_mat[i].inst == inst) g_elem_mat[i].inst = NULL;
	if (!E && !nu) rv = 0;
	else
		for (int i = 0; i < 64; i++)
			if (!g_elem_mat[i].inst) {
				g_elem_mat[i] = (elem_mat_t){inst, E, nu};
				rv = 0;
				break;
			}
	pthread_mutex_unlock(&g_lock);
	return rv;
}

static elem_mat_t elem_mat_of(bfm_instance_t* inst) {
	elem_mat_t r = {inst, NULL, NULL};
	pthread_mutex_lock(&g_lock);
	for (int i = 0; i < 64; i++)
		if (g_elem_mat[i].inst == inst) r = g_elem_mat[i];
	pthread_mutex_unlock(&g_lock);
	return r;
}

/* ---------------------------------------------------------------- device problem cache */

/* Device storage is kept per instance between runs (cudaMalloc is slow);
 * every run uploads all inputs again, so edits to the instance are seen. */
typedef struct {
	bfm_instance_t* inst;
	int kind, N, E, n_edges, n_conds;
	bfm_gpu_problem_t* P;
	unsigned long stamp;
} cache_t;

static cache_t g_cache[8];
static unsigned long g_clock;

static bfm_gpu_problem_t* problem_for(bfm_instance_t* inst, int kind, int N, int E, int n_edges, int n_conds) {
	cache_t* slot = NULL;
	for (int i = 0; i < 8; i++) {
		cache_t* c = &g_cache[i];
		if (c->P && c->inst == inst && c->kind == kind && c->N == N && c->E == E && c->n_edges >= n_edges &&
		    c->n_conds >= n_conds) {
			c->stamp = ++g_clock;
			return c->P;
		}
	}
	for (int i = 0; i < 8; i++)
		if (!slot || !g_cache[i].P || g_cache[i].stamp < slot->stamp) {
			slot = &g_cache[i];
			if (!slot->P) break;
		}
	if (slot->P) bfm_gpu_problem_destroy(slot->P);
	memset(slot, 0, sizeof *slot);
	bfm_gpu_problem_t* P = NULL;
	if (bfm_gpu_problem_create(&P, kind, N, E, n_edges, n_conds, NULL) < 0) return NULL;
	*slot = (cache_t){inst, kind, N, E, n_edges, n_conds, P, ++g_clock};
	return P;
}

/* ---------------------------------------------------------------- gathering the inputs */

typedef struct {
	int32_t* elems;
	double weights[16], phi[64], dxi[64], deta[64];
	int nq;
	int nf;
	double fval[16];
	double* fields[8];
	int nc;
	int kinds[16];
	double values[16];
	uint8_t* masks;
	int n_edges;
	int32_t* edges;
	uint8_t* eboundary;
} gathered_t;

static void release(gathered_t* g) {
	free(g->elems);
	free(g->masks);
	free(g->edges);
	free(g->eboundary);
	for (int i = 0; i < 8; i++) free(g->fields[i]);
}

static int gather(bfm_state_t* st, bfm_sim_t* sim, bfm_instance_t* inst, gathered_t* g) {
	memset(g, 0, sizeof *g);
	bfm_mesh_t* const mesh = inst->obj->mesh;
	bfm_rule_t* const rule = inst->obj->rule;
	size_t const N = mesh->n_nodes, E = mesh->n_elems, kind = (size_t) mesh->kind;
	if (mesh->dim != 2) return REPORT(st, "only 2D meshes are supported (dim = %zu)", mesh->dim);
	if (kind != BFM_ELEM_KIND_SIMPLEX && kind != BFM_ELEM_KIND_QUAD)
		return REPORT(st, "only linear triangles and bilinear quads are supported (kind = %zu)", kind);
	if (N > INT_MAX / 2 || E * kind > INT_MAX) return REPORT(st, "mesh too large for 32-bit indices");
	/* connectivity: 64-bit ids go to the device as they are (narrowed and
	 * checked there); other widths are converted here */
	if (sizeof(size_t) != sizeof(uint64_t)) {
		g->elems = malloc(E * kind * sizeof *g->elems + 1);
		if (!g->elems) return REPORT(st, "out of host memory");
		for (size_t i = 0; i < E * kind; i++) {
			if (mesh->elems[i] >= N) return REPORT(st, "element %zu refers to node %zu of %zu", i / kind, mesh->elems[i], N);
			g->elems[i] = (int32_t) mesh->elems[i];
		}
	}
	/* shape functions sampled at the integration points through the rule's own pointers */
	if (rule->n_points > 16) return REPORT(st, "integration rules of at most 16 points are supported");
	g->nq = (int) rule->n_points;
	for (int q = 0; q < g->nq; q++) {
		double ph[8] = {0}, dx[8] = {0}, de[8] = {0};
		bfm_shape_t* const sh = &rule->shape;
		sh->phi(sh, rule->points[q], ph);
		sh->dphi(sh, 0, rule->points[q], dx);
		sh->dphi(sh, 1, rule->points[q], de);
		g->weights[q] = rule->weights[q];
		for (size_t j = 0; j < kind; j++) {
			g->phi[q * kind + j] = ph[j];
			g->dxi[q * kind + j] = dx[j];
			g->deta[q * kind + j] = de[j];
		}
	}
	/* body forces: constants, or per-node values of a callback (evaluated at
	 * the node, as the reference does, system.c:190-203) */
	if (sim->n_forces > 8) return REPORT(st, "at most 8 body forces are supported");
	g->nf = (int) sim->n_forces;
	for (int f = 0; f < g->nf; f++) {
		bfm_force_t* const F = sim->forces[f];
		if (F->dim != 2) return REPORT(st, "body force %d has dimension %zu, expected 2", f, F->dim);
		if (F->kind == BFM_FORCE_KIND_LINEAR) {
			g->fval[2 * f] = F->linear.force.data[0];
			g->fval[2 * f + 1] = F->linear.force.data[1];
		}
		else if (F->kind == BFM_FORCE_KIND_FUNKY) {
			g->fields[f] = malloc(2 * N * sizeof(double) + 1);
			if (!g->fields[f]) return REPORT(st, "out of host memory");
			double pos_d[2], out_d[2];
			bfm_vec_t pos = {st, 2, pos_d}, out = {st, 2, out_d};
			for (size_t i = 0; i < N; i++) {
				pos_d[0] = mesh->coords[2 * i];
				pos_d[1] = mesh->coords[2 * i + 1];
				out_d[0] = out_d[1] = 0;
				bfm_force_eval(F, &pos, &out);
				g->fields[f][2 * i] = out_d[0];
				g->fields[f][2 * i + 1] = out_d[1];
			}
		}
	}
	/* conditions, in the instance's order */
	if (inst->n_conditions > 16) return REPORT(st, "at most 16 conditions per instance are supported");
	g->nc = (int) inst->n_conditions;
	g->masks = malloc((size_t) g->nc * N + 1);
	if (!g->masks) return REPORT(st, "out of host memory");
	int need_edges = 0;
	for (int c = 0; c < g->nc; c++) {
		bfm_condition_t* const C = inst->conditions[c];
		int const k = C->kind;
		if (k < BFM_CONDITION_KIND_DIRICHLET_X || k > BFM_CONDITION_KIND_DIRICHLET_TANGENT)
			return REPORT(st, "unknown condition kind %d", k);
		need_edges |= k != BFM_CONDITION_KIND_DIRICHLET_X && k != BFM_CONDITION_KIND_DIRICHLET_Y;
		g->kinds[c] = k;
		g->values[c] = C->value;
		/* a C bool is one byte holding 0 or 1: the mask's own layout */
		_Static_assert(sizeof(bool) == 1, "one-byte bool");
		memcpy(g->masks + (size_t) c * N, C->nodes, N);
	}
	if (need_edges && mesh->n_edges) {
		if (mesh->n_edges > INT_MAX / 2) return REPORT(st, "too many edges");
		g->n_edges = (int) mesh->n_edges;
		g->edges = malloc(2 * mesh->n_edges * sizeof *g->edges + 1);
		g->eboundary = malloc(mesh->n_edges + 1);
		if (!g->edges || !g->eboundary) return REPORT(st, "out of host memory");
		for (size_t e = 0; e < mesh->n_edges; e++) {
			for (int k = 0; k < 2; k++) {
				size_t const nd = mesh->edges[e].nodes[k];
				if (nd >= N) return REPORT(st, "edge %zu refers to node %zu of %zu", e, nd, N);
				g->edges[2 * e + k] = (int32_t) nd;
			}
			/* the normal/tangent Dirichlet condition sums over edges with one element (system.c:396) */
			g->eboundary[e] = mesh->edges[e].elems[1] == -1;
		}
	}
	return 0;
}

/* Upload one instance and assemble it in `precision`. */
static bfm_gpu_problem_t* upload_and_assemble(bfm_state_t* st, bfm_sim_t* sim, bfm_instance_t* inst, int stress, int precision,
                                              int precond, int dedicated) {
	gathered_t g;
	if (gather(st, sim, inst, &g) < 0) {
		release(&g);
		return NULL;
	}
	bfm_mesh_t* const mesh = inst->obj->mesh;
	bfm_material_t* const mat = inst->obj->material;
	elem_mat_t const em = elem_mat_of(inst);
	/* a dedicated problem (owned by the caller, e.g. a sparse system matrix) or the instance's cached one */
	bfm_gpu_problem_t* P = NULL;
	if (dedicated) {
		if (bfm_gpu_problem_create(&P, (int) mesh->kind, (int) mesh->n_nodes, (int) mesh->n_elems, g.n_edges, g.nc, NULL) < 0)
			P = NULL;
	}
	else {
		P = problem_for(inst, (int) mesh->kind, (int) mesh->n_nodes, (int) mesh->n_elems, g.n_edges, g.nc);
	}
	int ok = P != NULL;
	const double* fields[8];
	for (int f = 0; f < 8; f++) fields[f] = g.fields[f];
	if (ok && g.elems) ok = bfm_gpu_problem_set_geometry(P, mesh->coords, g.elems, BFM_GPU_HOST) == 0;
	else if (ok) {
		long bad = -1;
		ok = bfmi_set_geometry_u64(P, mesh->coords, (const uint64_t*) mesh->elems, &bad) == 0;
		if (ok && bad >= 0) {
			REPORT(st, "element %zu refers to node %zu of %zu", (size_t) bad / (size_t) mesh->kind, mesh->elems[bad],
			       mesh->n_nodes);
			if (dedicated) bfm_gpu_problem_destroy(P);
			release(&g);
			return NULL;
		}
	}
	ok = ok && bfm_gpu_problem_set_material(P, mat->E, mat->nu, mat->rho, stress, em.E, em.nu, BFM_GPU_HOST) == 0;
	ok = ok && bfm_gpu_problem_set_rule(P, g.nq, g.weights, g.phi, g.dxi, g.deta) == 0;
	ok = ok && bfm_gpu_problem_set_forces(P, g.nf, g.fval, fields, BFM_GPU_HOST) == 0;
	ok = ok && bfm_gpu_problem_set_conditions(P, g.nc, g.kinds, g.values, g.masks, g.n_edges, g.edges, BFM_GPU_HOST) == 0;
	if (g.n_edges) ok = ok && bfm_gpu_problem_set_edge_boundary(P, g.eboundary, BFM_GPU_HOST) == 0;
	(void) precond;
	ok = ok && bfm_gpu_problem_assemble(P, precision) == 0;
	release(&g);
	if (!ok) {
		REPORT(st, "%s", bfm_gpu_last_error());
		if (dedicated && P) bfm_gpu_problem_destroy(P);
		return NULL;
	}
	return P;
}

/* The network the environment names (BFM_GPU_MPNN = weights file), loaded
 * once and selected when a run asks for the learned preconditioner, so that
 * unchanged callers can use it through environment variables alone. */
static bfm_gpu_mpnn_t* g_env_net;

static int env_network(bfm_state_t* st) {
	char const* path = getenv("BFM_GPU_MPNN");
	if (!path || g_env_net) return 0;
	if (bfm_gpu_mpnn_create(&g_env_net, 0) < 0) return REPORT(st, "%s", bfm_gpu_last_error());
	if (bfm_gpu_mpnn_load(g_env_net, path) < 0) {
		REPORT(st, "%s", bfm_gpu_last_error());
		bfm_gpu_mpnn_destroy(g_env_net);
		g_env_net = NULL;
		return -1;
	}
	return bfm_gpu_mpnn_use(g_env_net);
}

static int run_instance(bfm_sim_t* sim, bfm_instance_t* inst, int stress) {
	bfm_state_t* const st = sim->state;
	bfm_gpu_opts_t const o = current_opts();
	if ((o.precond == BFM_GPU_PC_LEARNED || o.precond == BFM_GPU_PC_LEARNED_SSOR || o.precond == BFM_GPU_PC_LEARNED_SSOR2) &&
	    env_network(st) < 0)
		return -1;
	bfm_gpu_problem_t* P = upload_and_assemble(st, sim, inst, stress, o.precision, o.precond, 0);
	if (!P) return -1;
	if (bfm_gpu_problem_solve(P, &o) < 0) return REPORT(st, "%s", bfm_gpu_last_error());
	bfm_gpu_stats_t s;
	if (bfm_gpu_problem_stats(P, &s) < 0) return REPORT(st, "%s", bfm_gpu_last_error());
	t_stats = s;
	if (s.status == BFM_GPU_BAD_MESH) return REPORT(st, "%s", bfm_gpu_last_error());
	if (bfm_gpu_problem_solution(P, inst->effects, BFM_GPU_HOST) < 0) return REPORT(st, "%s", bfm_gpu_last_error());
	/* BFM_GPU_STAGNATED: the residual reached the roundoff floor above rtol; x is usable */
	if (s.status == BFM_GPU_NOT_CONVERGED)
		return REPORT(st, "CG did not reach rtol %g in %d iterations (relative residual %g)", o.rtol, s.iterations, s.rel_residual);
	if (s.status == BFM_GPU_BREAKDOWN)
		return REPORT(st, "CG broke down after %d iterations: the system is not positive definite (missing constraints?)",
		              s.iterations);
	if (s.status == BFM_GPU_TIMEOUT)
		return REPORT(st, "a grid barrier of the solver timed out after %d iterations (barrier_polls %lld)", s.iterations,
		              (long long) o.barrier_polls);
	return 0;
}

/* Element mode of the axisymmetric system: 2 (the plane-strain constant a,
 * the radius on every stiffness term, consistent edge loads) unless
 * BFM_GPU_AXISYM_REFERENCE=1 asks for 3, the reference's own formulas
 * (system.c:241, 337, 591-601), which make K indefinite for usual nu. */
static int axisym_mode(void) {
	char const* e = getenv("BFM_GPU_AXISYM_REFERENCE");
	return e && e[0] == '1' ? 3 : 2;
}

int bfm_sim_run(bfm_sim_t* sim) {
	if (sim->kind == BFM_SIM_KIND_NONE) return 0;
	if (sim->kind != BFM_SIM_KIND_PLANAR_STRAIN && sim->kind != BFM_SIM_KIND_PLANAR_STRESS &&
	    sim->kind != BFM_SIM_KIND_AXISYMMETRIC_STRAIN)
		return -1;
	int const stress = sim->kind == BFM_SIM_KIND_AXISYMMETRIC_STRAIN ? axisym_mode()
	                                                                 : sim->kind == BFM_SIM_KIND_PLANAR_STRESS;
	int rc = 0;
	BFM_RANGE_PUSH("bfm_sim_run");
	for (size_t i = 0; i < sim->n_instances && rc == 0; i++)
		if (run_instance(sim, sim->instances[i], stress) < 0) rc = -1;
	BFM_RANGE_POP();
	return rc;
}

/* ---------------------------------------------------------------- dense systems (ref system.c) */

int bfm_system_create(bfm_system_t* s, bfm_state_t* state, size_t n) {
	s->state = state;
	s->n = n;
	if (bfm_perm_create(&s->perm, state, n) < 0) return -1;
	if (bfm_matrix_full_create(&s->A, state, BFM_MATRIX_MAJOR_ROW, n) < 0) return -1;
	if (bfm_vec_create(&s->b, state, n) < 0) {
		bfm_matrix_destroy(&s->A);
		return -1;
	}
	return 0;
}

int bfm_system_destroy(bfm_system_t* s) {
	bfm_perm_destroy(&s->perm);
	bfm_matrix_destroy(&s->A);
	bfm_vec_destroy(&s->b);
	return 0;
}

/* RCM renumbering, then conversion to band storage (ref system.c:44-81). */
int bfm_system_renumber(bfm_system_t* s) {
	if (s->A.kind == BFM_MATRIX_KIND_SPARSE) {
		/* the reference's permutation and permuted right-hand side; the sparse
		 * matrix records the permutation and keeps its storage */
		if (bfm_perm_rcm(&s->perm, &s->A) < 0) return -1;
		if (bfm_perm_perm_vec(&s->perm, &s->b, false) < 0) return -1;
		return bfm_perm_perm_matrix(&s->perm, &s->A, false);
	}
	if (bfm_perm_rcm(&s->perm, &s->A) < 0) return -1;
	if (bfm_perm_perm_matrix(&s->perm, &s->A, false) < 0) return -1;
	if (bfm_perm_perm_vec(&s->perm, &s->b, false) < 0) return -1;
	size_t const k = bfm_matrix_bandwidth(&s->A);
	bfm_matrix_t band;
	if (bfm_matrix_band_create(&band, s->state, s->A.major, s->A.m, k) < 0) return -1;
	if (bfm_matrix_copy(&band, &s->A) < 0) {
		bfm_matrix_destroy(&band);
		return -1;
	}
	bfm_matrix_destroy(&s->A);
	s->A = band;
	return 0;
}

/* Assemble on the GPU (FP64, the reference's operation order) and expand the
 * 2x2-block matrix into the dense system this struct holds. */
static int create_planar(bfm_system_t* s, bfm_instance_t* inst, size_t n_forces, bfm_force_t** forces, int stress) {
	bfm_state_t* const st = inst->state;
	bfm_mesh_t* const mesh = inst->obj->mesh;
	if (mesh->dim != 2 || (mesh->kind != BFM_ELEM_KIND_SIMPLEX && mesh->kind != BFM_ELEM_KIND_QUAD)) return -1;
	size_t const n = mesh->n_nodes * 2;
	bfm_sim_t tmp;
	memset(&tmp, 0, sizeof tmp);
	tmp.state = st;
	tmp.n_forces = n_forces;
	tmp.forces = forces;
	if (sparse_system(n)) {
		/* O(nnz): the device problem stays (the matrix owns it), a host copy of
		 * its 2x2-block CSR for reads; no n x n storage anywhere */
		s->state = st;
		s->n = n;
		if (bfm_perm_create(&s->perm, st, n) < 0) return -1;
		if (bfm_vec_create(&s->b, st, n) < 0) return -1;
		bfm_gpu_problem_t* P = upload_and_assemble(st, &tmp, inst, stress, BFM_GPU_FP64, BFM_GPU_PC_JACOBI, 1);
		if (!P) {
			bfm_vec_destroy(&s->b);
			return -1;
		}
		if (bfmi_sparse_wrap(&s->A, st, P, mesh->n_nodes, s->b.data) < 0) {
			bfm_gpu_problem_destroy(P);
			bfm_vec_destroy(&s->b);
			return REPORT(st, "%s", bfm_gpu_last_error());
		}
		return 0;
	}
	if (bfm_system_create(s, st, n) < 0) return -1;
	bfm_gpu_problem_t* P = upload_and_assemble(st, &tmp, inst, stress, BFM_GPU_FP64, BFM_GPU_PC_JACOBI, 0);
	if (!P) return -1;
	int64_t nb = 0;
	if (bfm_gpu_problem_n_blocks(P, &nb) < 0) return REPORT(st, "%s", bfm_gpu_last_error());
	int32_t* rp = malloc((mesh->n_nodes + 1) * sizeof *rp);
	int32_t* cols = malloc((size_t) nb * sizeof *cols + 1);
	double* vals = malloc((size_t) nb * 4 * sizeof *vals + 1);
	int rv = -1;
	if (rp && cols && vals && bfm_gpu_problem_download(P, rp, cols, vals, s->b.data) == 0) {
		for (size_t r = 0; r < mesh->n_nodes; r++)
			for (int32_t k = rp[r]; k < rp[r + 1]; k++) {
				size_t const c = (size_t) cols[k];
				double* const A = s->A.full.data;
				A[(2 * r) * n + 2 * c] = vals[4 * k];
				A[(2 * r) * n + 2 * c + 1] = vals[4 * k + 1];
				A[(2 * r + 1) * n + 2 * c] = vals[4 * k + 2];
				A[(2 * r + 1) * n + 2 * c + 1] = vals[4 * k + 3];
			}
		rv = 0;
	}
	else {
		REPORT(st, "%s", bfm_gpu_last_error());
	}
	free(rp);
	free(cols);
	free(vals);
	return rv;
}

int bfm_system_create_planar_strain(bfm_system_t* s, bfm_instance_t* inst, size_t n_forces, bfm_force_t** forces) {
	return create_planar(s, inst, n_forces, forces, 0);
}

int bfm_system_create_planar_stress(bfm_system_t* s, bfm_instance_t* inst, size_t n_forces, bfm_force_t** forces) {
	return create_planar(s, inst, n_forces, forces, 1);
}

int bfm_system_create_axisymmetric_strain(bfm_system_t* s, bfm_instance_t* inst, size_t n_forces, bfm_force_t** forces) {
	return create_planar(s, inst, n_forces, forces, axisym_mode());
}
