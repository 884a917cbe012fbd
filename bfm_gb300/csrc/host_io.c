/* File front ends of libbfm: the LEPL1110 mesh and problem formats, Wavefront
 * meshes and the U/V result writer (reference libbfm/src/mesh.c:52-279 and
 * ez.c:6-229).  Line-oriented parsers written for this library; they accept
 * everything the reference reads, and also LEPL1110 meshes without an edge
 * section (meshes/gear*.lepl1110), which the reference's reader crashes on.
 */
#include <ctype.h>
#include <stdio.h>
#include <string.h>
#include <strings.h>

#include <bfm/ez.h>
#include <bfm/mesh.h>

static void* zalloc(bfm_state_t* state, size_t size) {
	void* p = state->alloc(size ? size : 1);
	if (p) memset(p, 0, size ? size : 1);
	return p;
}

static char* trim(char* s) {
	while (*s && isspace((unsigned char) *s)) s++;
	char* e = s + strlen(s);
	while (e > s && isspace((unsigned char) e[-1])) *--e = 0;
	return s;
}

/* next line that is not blank (leftovers of fscanf included) */
static char* next_line(char* buf, int size, FILE* fp) {
	while (fgets(buf, size, fp)) {
		char* t = buf;
		while (*t && isspace((unsigned char) *t)) t++;
		if (*t) return buf;
	}
	return NULL;
}

/* case-insensitive prefix test on a trimmed line */
static int starts(char const* line, char const* key) { return strncasecmp(line, key, strlen(key)) == 0; }

/* ---------------------------------------------------------------- LEPL1110 mesh (ref mesh.c:104-201) */

int bfm_mesh_read_lepl1110(bfm_mesh_t* mesh, bfm_state_t* state, char const* name) {
	memset(mesh, 0, sizeof *mesh);
	mesh->state = state;
	mesh->dim = 2;
	FILE* fp = fopen(name, "r");
	if (!fp) return -1;
	char buf[4096];
	int rv = -1;
	size_t n;
	while (fgets(buf, sizeof buf, fp)) {
		char* line = trim(buf);
		if (!*line) continue;
		if (sscanf(line, "Number of nodes %zu", &n) == 1) {
			mesh->n_nodes = n;
			mesh->coords = zalloc(state, 2 * n * sizeof *mesh->coords);
			if (!mesh->coords) goto out;
			for (size_t i = 0; i < n; i++) {
				size_t id;
				if (!fgets(buf, sizeof buf, fp) ||
				    sscanf(buf, " %zu : %lf %lf", &id, &mesh->coords[2 * i], &mesh->coords[2 * i + 1]) != 3)
					goto out;
			}
		}
		else if (sscanf(line, "Number of edges %zu", &n) == 1) {
			mesh->n_edges = n;
			mesh->edges = zalloc(state, n * sizeof *mesh->edges);
			if (!mesh->edges) goto out;
			for (size_t i = 0; i < n; i++) {
				ssize_t id;
				if (!fgets(buf, sizeof buf, fp) ||
				    sscanf(buf, " %zd : %zu %zu", &id, &mesh->edges[i].nodes[0], &mesh->edges[i].nodes[1]) != 3)
					goto out;
				/* the reference keeps the file's edge number in elems[0] and marks every edge a border */
				mesh->edges[i].elems[0] = id;
				mesh->edges[i].elems[1] = -1;
			}
		}
		else if (starts(line, "Number of triangles") || starts(line, "Number of quads")) {
			mesh->kind = starts(line, "Number of triangles") ? BFM_ELEM_KIND_SIMPLEX : BFM_ELEM_KIND_QUAD;
			if (sscanf(strrchr(line, 's') + 1, "%zu", &n) != 1) goto out;
			mesh->n_elems = n;
			size_t const k = (size_t) mesh->kind;
			mesh->elems = zalloc(state, n * k * sizeof *mesh->elems);
			if (!mesh->elems) goto out;
			for (size_t i = 0; i < n; i++) {
				size_t id, *e = mesh->elems + i * k;
				if (!fgets(buf, sizeof buf, fp)) goto out;
				int const got = k == 3 ? sscanf(buf, " %zu : %zu %zu %zu", &id, e, e + 1, e + 2)
				                       : sscanf(buf, " %zu : %zu %zu %zu %zu", &id, e, e + 1, e + 2, e + 3);
				if (got != (int) k + 1) goto out;
			}
		}
		else if (sscanf(line, "Number of domains %zu", &n) == 1) {
			mesh->n_domains = n;
			mesh->domains = zalloc(state, n * sizeof *mesh->domains);
			if (!mesh->domains) goto out;
			for (size_t d = 0; d < n; d++) {
				size_t id = d, cnt = 0;
				bfm_domain_t tmp;
				memset(&tmp, 0, sizeof tmp);
				if (!next_line(buf, sizeof buf, fp) || sscanf(buf, " Domain : %zu", &id) != 1 || id >= n) goto out;
				if (!next_line(buf, sizeof buf, fp)) goto out;
				char* nm = strchr(buf, ':');
				if (!nm) goto out;
				nm++;
				while (*nm == ' ') nm++;
				nm[strcspn(nm, "\r\n")] = 0;
				strncpy(tmp.name, nm, sizeof tmp.name - 1);
				if (!next_line(buf, sizeof buf, fp) || sscanf(buf, " Number of elements : %zu", &cnt) != 1) goto out;
				tmp.n_elements = cnt;
				tmp.elements = zalloc(state, cnt * sizeof *tmp.elements);
				if (!tmp.elements) goto out;
				for (size_t j = 0; j < cnt; j++)
					if (fscanf(fp, "%zu", &tmp.elements[j]) != 1) {
						state->free(tmp.elements);
						goto out;
					}
				if (mesh->domains[id].elements) state->free(mesh->domains[id].elements);
				mesh->domains[id] = tmp;
			}
		}
	}
	rv = mesh->coords && mesh->elems ? 0 : -1;
out:
	fclose(fp);
	return rv;
}

/* ---------------------------------------------------------------- Wavefront (ref mesh.c:52-102, 203-279) */

typedef struct {
	size_t lo, hi;
	size_t a, b; /* endpoints in the order the element lists them */
	size_t elem;
} half_edge_t;

/* same ordering as the reference's edge list: smaller endpoint descending, then larger ascending */
static int cmp_half(void const* x, void const* y) {
	half_edge_t const* p = x;
	half_edge_t const* q = y;
	if (p->lo != q->lo) return p->lo > q->lo ? -1 : 1;
	if (p->hi != q->hi) return p->hi < q->hi ? -1 : 1;
	return p->elem < q->elem ? -1 : (p->elem > q->elem ? 1 : 0);
}

static int wavefront_edges(bfm_mesh_t* mesh) {
	bfm_state_t* const state = mesh->state;
	size_t const k = (size_t) mesh->kind, total = mesh->n_elems * k;
	half_edge_t* h = zalloc(state, total * sizeof *h);
	if (!h) return -1;
	for (size_t e = 0; e < mesh->n_elems; e++)
		for (size_t j = 0; j < k; j++) {
			half_edge_t* t = &h[e * k + j];
			t->a = mesh->elems[e * k + j];
			t->b = mesh->elems[e * k + (j + 1) % k];
			t->lo = t->a < t->b ? t->a : t->b;
			t->hi = t->a < t->b ? t->b : t->a;
			t->elem = e;
		}
	qsort(h, total, sizeof *h, cmp_half);
	mesh->edges = zalloc(state, total * sizeof *mesh->edges);
	if (!mesh->edges) {
		state->free(h);
		return -1;
	}
	/* Walk the sorted list as the reference does: a half-edge and the next one
	 * form an interior edge when they run in opposite directions; otherwise the
	 * half-edge is a boundary edge.  The last half-edge is looked at only as
	 * the second of a pair, so when it is unpaired it is left out (the
	 * reference's edge list ends the same way; kept for parity, since the
	 * edges feed the Neumann and normal/tangent conditions). */
	size_t cur = 0;
	for (size_t i = 1; i < total;) {
		bfm_edge_t* ed = &mesh->edges[cur++];
		half_edge_t const* p = &h[i - 1];
		ed->nodes[0] = p->a;
		ed->nodes[1] = p->b;
		ed->elems[0] = (ssize_t) p->elem;
		ed->elems[1] = -1;
		if (p->a == h[i].b && p->b == h[i].a) {
			ed->elems[1] = (ssize_t) h[i].elem;
			i += 2;
		}
		else {
			i += 1;
		}
	}
	state->free(h);
	mesh->n_edges = cur;
	return 0;
}

int bfm_mesh_read_wavefront(bfm_mesh_t* mesh, bfm_state_t* state, char const* name, bool full) {
	memset(mesh, 0, sizeof *mesh);
	mesh->state = state;
	mesh->dim = full ? 3 : 2;
	mesh->kind = BFM_ELEM_KIND_SIMPLEX;
	FILE* fp = fopen(name, "r");
	if (!fp) return -1;
	char buf[4096];
	size_t cap_n = 0, cap_e = 0;
	int rv = -1;
	while (fgets(buf, sizeof buf, fp)) {
		char* line = trim(buf);
		if (line[0] == 'v' && line[1] == ' ') {
			double x = 0, y = 0, z = 0;
			if (sscanf(line + 2, "%lf %lf %lf", &x, &y, &z) < 2) goto out;
			if (mesh->n_nodes == cap_n) {
				cap_n = cap_n ? 2 * cap_n : 256;
				double* c = state->realloc(mesh->coords, cap_n * mesh->dim * sizeof *c);
				if (!c) goto out;
				mesh->coords = c;
			}
			double* c = mesh->coords + mesh->n_nodes * mesh->dim;
			c[0] = x;
			c[1] = y;
			if (full) c[2] = z;
			mesh->n_nodes++;
		}
		else if (line[0] == 'f' && line[1] == ' ') {
			size_t v[3];
			char* p = line + 2;
			for (int j = 0; j < 3; j++) {
				char* end;
				unsigned long long const t = strtoull(p, &end, 10);
				if (end == p || t == 0) goto out;
				v[j] = (size_t) t - 1;
				p = end;
				while (*p && *p != ' ') p++; /* skip /vt/vn */
			}
			if (mesh->n_elems == cap_e) {
				cap_e = cap_e ? 2 * cap_e : 256;
				size_t* e = state->realloc(mesh->elems, cap_e * 3 * sizeof *e);
				if (!e) goto out;
				mesh->elems = e;
			}
			memcpy(mesh->elems + 3 * mesh->n_elems, v, sizeof v);
			mesh->n_elems++;
		}
	}
	rv = wavefront_edges(mesh);
out:
	fclose(fp);
	return rv;
}

/* ---------------------------------------------------------------- LEPL1110 problem (ref ez.c) */

static int condition_kind(char const* s, bfm_condition_kind_t* k) {
	static struct {
		char const* name;
		bfm_condition_kind_t kind;
	} const table[] = {
		{"Dirichlet-X", BFM_CONDITION_KIND_DIRICHLET_X},         {"Dirichlet-Y", BFM_CONDITION_KIND_DIRICHLET_Y},
		{"Neumann-X", BFM_CONDITION_KIND_NEUMANN_X},             {"Neumann-Y", BFM_CONDITION_KIND_NEUMANN_Y},
		{"Neumann-Tangent", BFM_CONDITION_KIND_NEUMANN_TANGENT}, {"Neumann-Normal", BFM_CONDITION_KIND_NEUMANN_NORMAL},
		{"Dirichlet-Normal", BFM_CONDITION_KIND_DIRICHLET_NORMAL}, {"Dirichlet-Tangent", BFM_CONDITION_KIND_DIRICHLET_TANGENT},
	};
	for (size_t i = 0; i < sizeof table / sizeof *table; i++)
		if (strcasecmp(s, table[i].name) == 0) {
			*k = table[i].kind;
			return 0;
		}
	return -1;
}

int bfm_ez_lepl1110_create(bfm_ez_lepl1110_t* ez, bfm_state_t* state, bfm_mesh_t* mesh, char* name) {
	memset(ez, 0, sizeof *ez);
	ez->state = state;
	ez->mesh = mesh;
	if (bfm_sim_create(&ez->sim, state, BFM_SIM_KIND_NONE) < 0) return -1;
	if (bfm_material_create(&ez->material, state, "lepl1110", 0, 0, 0) < 0) return -1;
	if (bfm_rule_create_gauss_legendre(&ez->rule, state, 2, mesh->kind) < 0) return -1;
	if (bfm_obj_create(&ez->obj, state, mesh, &ez->material, &ez->rule) < 0) return -1;
	if (bfm_instance_create(&ez->instance, state, &ez->obj) < 0) return -1;
	if (bfm_sim_add_instance(&ez->sim, &ez->instance) < 0) return -1;
	FILE* fp = fopen(name, "r");
	if (!fp) return -1;
	char buf[1024];
	int rv = 0;
	while (rv == 0 && fgets(buf, sizeof buf, fp)) {
		char* line = trim(buf);
		char* colon = strchr(line, ':');
		if (!colon) continue;
		*colon = 0;
		char* key = trim(line);
		char* val = trim(colon + 1);
		if (strcasecmp(key, "Type of problem") == 0) {
			if (strncasecmp(val, "Planar strain", 13) == 0) ez->sim.kind = BFM_SIM_KIND_PLANAR_STRAIN;
			else if (strncasecmp(val, "Planar stress", 13) == 0) ez->sim.kind = BFM_SIM_KIND_PLANAR_STRESS;
			else if (strncasecmp(val, "Axi-symetric", 12) == 0) ez->sim.kind = BFM_SIM_KIND_AXISYMMETRIC_STRAIN;
		}
		else if (strcasecmp(key, "Young modulus") == 0) {
			ez->material.E = strtod(val, NULL);
		}
		else if (strcasecmp(key, "Poisson ratio") == 0) {
			ez->material.nu = strtod(val, NULL);
		}
		else if (strcasecmp(key, "Mass density") == 0) {
			ez->material.rho = strtod(val, NULL);
		}
		else if (strcasecmp(key, "Gravity") == 0) {
			/* gravity g points down: the force is (0, -g), ref ez.c:75-104 */
			bfm_vec_t g;
			if (bfm_force_create(&ez->gravity, state, 2) < 0 || bfm_vec_create(&g, state, 2) < 0) {
				rv = -1;
				break;
			}
			g.data[1] = -strtod(val, NULL);
			bfm_force_set_linear(&ez->gravity, &g);
			bfm_vec_destroy(&g);
			if (bfm_sim_add_force(&ez->sim, &ez->gravity) < 0) rv = -1;
		}
		else if (strcasecmp(key, "Boundary condition") == 0) {
			/* "<kind> = <value>" before the colon we cut at, "<domain>" after the next one */
			char* dom = strchr(val, ':');
			char* eq = strchr(val, '=');
			if (!dom || !eq || eq > dom) {
				rv = -1;
				break;
			}
			*dom = 0;
			*eq = 0;
			bfm_condition_kind_t kind;
			if (condition_kind(trim(val), &kind) < 0) {
				rv = -1;
				break;
			}
			double const value = strtod(eq + 1, NULL);
			char* dname = trim(dom + 1);
			bfm_condition_t* grown = state->realloc(ez->conditions, (ez->n_conditions + 1) * sizeof *grown);
			if (!grown) {
				rv = -1;
				break;
			}
			ez->conditions = grown;
			bfm_condition_t* c = &ez->conditions[ez->n_conditions++];
			if (bfm_condition_create(c, state, mesh, kind) < 0) {
				rv = -1;
				break;
			}
			c->value = value;
			/* flag both ends of every edge of the first domain of that name (ref ez.c:158-173) */
			for (size_t d = 0; d < mesh->n_domains; d++) {
				char nm[sizeof mesh->domains[d].name + 1];
				memcpy(nm, mesh->domains[d].name, sizeof mesh->domains[d].name);
				nm[sizeof nm - 1] = 0;
				if (strncasecmp(trim(nm), dname, 25) != 0) continue;
				bfm_domain_t const* D = &mesh->domains[d];
				for (size_t j = 0; j < D->n_elements; j++) {
					size_t const e = D->elements[j];
					if (e >= mesh->n_edges) continue;
					for (int k = 0; k < 2; k++) {
						size_t const node = mesh->edges[e].nodes[k];
						if (node < mesh->n_nodes) c->nodes[node] = true;
					}
				}
				break;
			}
		}
	}
	fclose(fp);
	if (rv < 0) return -1;
	/* attach after parsing: the condition array may have moved while growing */
	for (size_t i = 0; i < ez->n_conditions; i++)
		if (bfm_instance_add_condition(&ez->instance, &ez->conditions[i]) < 0) return -1;
	return 0;
}

int bfm_ez_lepl1110_destroy(bfm_ez_lepl1110_t* ez) {
	for (size_t i = 0; i < ez->n_conditions; i++) bfm_condition_destroy(&ez->conditions[i]);
	if (ez->conditions) ez->state->free(ez->conditions);
	ez->conditions = NULL;
	bfm_force_destroy(&ez->gravity);
	bfm_material_destroy(&ez->material);
	bfm_rule_destroy(&ez->rule);
	bfm_obj_destroy(&ez->obj);
	bfm_instance_destroy(&ez->instance);
	bfm_sim_destroy(&ez->sim);
	return 0;
}

/* U or V (shift 0 or 1) as "%14.7e", three per line, byte-compatible with the
 * reference's writer (ez.c:211-229), including its line-break rule. */
int bfm_ez_lepl1110_write(bfm_ez_lepl1110_t* ez, size_t shift, char const* filename) {
	FILE* fp = fopen(filename, "w");
	if (!fp) return -1;
	size_t const n = ez->obj.mesh->n_nodes;
	fprintf(fp, "Number of nodes %zu\n", n);
	for (size_t i = 0; i < n; i++) {
		fprintf(fp, "%14.7e", ez->instance.effects[i * 2 + shift]);
		if (i + 1 != ez->instance.n_effects && (i + 1) % 3 == 0) fputc('\n', fp);
	}
	fputc('\n', fp);
	fclose(fp);
	return 0;
}
