/* 2D meshes; ABI-identical to the reference's libbfm/src/bfm/mesh.h:7-54.
 * Node coordinates are interleaved doubles, element connectivity size_t. */
#pragma once

#include <stdlib.h>

#include <bfm/matrix.h>

typedef enum {
	BFM_ELEM_KIND_SIMPLEX = 3,
	BFM_ELEM_KIND_QUAD = 4,
	BFM_ELEM_KIND_QUADRATIC_TRIANGLE = 6,
} bfm_elem_kind_t;

typedef enum {
	BFM_PLANAR_STRAINS,
} bfm_problem_type_t;

typedef struct {
	size_t nodes[2];  /* endpoints                                    */
	ssize_t elems[2]; /* adjacent elements, elems[1] == -1 on a border */
} bfm_edge_t;

typedef struct {
	char name[50];
	size_t n_elements; /* edge indices into bfm_mesh_t.edges */
	size_t* elements;
} bfm_domain_t;

typedef struct {
	bfm_state_t* state;
	size_t dim;
	bfm_elem_kind_t kind;
	size_t n_elems;
	size_t n_nodes;
	size_t n_edges;
	double* coords;
	size_t* elems;
	bfm_edge_t* edges;
	size_t n_domains;
	bfm_domain_t* domains;
} bfm_mesh_t;

int bfm_mesh_create(bfm_mesh_t* mesh, bfm_state_t* state, size_t dim, bfm_elem_kind_t kind);             /* ref mesh.c:6-14    */
int bfm_mesh_destroy(bfm_mesh_t* mesh);                                                                 /* ref mesh.c:16-30   */
int bfm_mesh_read_lepl1110(bfm_mesh_t* mesh, bfm_state_t* state, char const* name);                     /* ref mesh.c:104-201 */
int bfm_mesh_read_wavefront(bfm_mesh_t* mesh, bfm_state_t* state, char const* name, bool full);         /* ref mesh.c:203-279 */
