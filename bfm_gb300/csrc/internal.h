/* Library-internal helpers shared by the translation units (not exported). */
#pragma once

#include <bfm/gpu.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Set the message bfm_gpu_last_error() reports on this thread. */
__attribute__((visibility("hidden"))) void bfm_gpu_set_last_error(const char* msg);

struct bfm_gpu_problem;

/* Device buffers of an assembled problem, for the other translation units. */
typedef struct {
	int N, n_elems, kind, precision, precond, assembled, grid;
	const int* row_ptr;
	const int* cols;
	const float* vals32;
	const float* corr32;
	const double* vals64;     /* FP64 operator of the FP64 and MIXED_EXACT iterations */
	const double* vals64_any; /* FP64 values whenever this precision assembled them   */
	double* dinv64;           /* preconditioner arrays (layout: bfmi_set_precond_blocks) */
	float* dinv32;
	const double* b;
	double* x;
	void* vec[5];
	void* stream;
	/* colour-major order of the SSOR preconditioners (ncol = 0: caller's order):
	 * colour c holds the working rows [col_off[c], col_off[c + 1]), and every
	 * row's blocks before dpos[i] are lower-colour neighbours, after it the
	 * diagonal block and then higher-colour ones */
	int ncol;
	int col_off[65];
	const int* dpos;
	unsigned inputs_gen;  /* changes with every bfm_gpu_problem_set_* call */
} bfmi_buffers_t;

/* Mesh-side device arrays of a problem (read only). */
typedef struct {
	const double* coords;
	const int* inc_ptr;  /* node -> incident elements, ascending */
	const int* inc;
	const double* elemE; /* nullptr: uniform E */
	const double* elemNu;
	double E, nu;
	const int* last_ci;  /* per DOF: index of its last Dirichlet condition, -1 if free */
} bfmi_mesh_t;

__attribute__((visibility("hidden"))) int bfmi_mesh(struct bfm_gpu_problem* P, bfmi_mesh_t* out);

/* Preconditioner of the next solve from per-node 2x2 blocks (4 doubles per
 * node, device, on the problem's stream), stored in the layout of the
 * assembled precision.  Used by the learned preconditioner. */
__attribute__((visibility("hidden"))) int bfmi_set_precond_blocks(struct bfm_gpu_problem* P, const double* blocks);

/* Learned preconditioner blocks of the selected network for an assembled
 * problem, written with bfmi_set_precond_blocks; jacobi != 0 writes the
 * Jacobi blocks instead (the fallback), without a network. */
__attribute__((visibility("hidden"))) int bfmi_learned_precond(struct bfm_gpu_problem* P, int jacobi);

__attribute__((visibility("hidden"))) int bfmi_buffers(struct bfm_gpu_problem* P, bfmi_buffers_t* out);

/* Solve the assembled FP64 system for the right-hand side b (2 n_nodes
 * doubles, host, the caller's node order) with the options' rtol and
 * preconditioner (re-assembling first when the preconditioner changes) and
 * copy the solution to x (host, the caller's order); *status gets the
 * solver's BFM_GPU_* status.  Used by the sparse system matrices. */
__attribute__((visibility("hidden"))) int bfmi_solve_rhs(struct bfm_gpu_problem* P, const double* b, double* x,
                                                         const bfm_gpu_opts_t* opts, int* status, int* iterations,
                                                         double* rel_residual);

/* Sparse system matrices (host_sparse.c): a matrix of kind
 * BFM_MATRIX_KIND_SPARSE around an assembled FP64 problem it then owns
 * (n_nodes nodes; its right-hand side copied to b); the kind's operations. */
#include <bfm/matrix.h>
#include <bfm/perm.h>
__attribute__((visibility("hidden"))) int bfmi_sparse_wrap(bfm_matrix_t* A, bfm_state_t* state, bfm_gpu_problem_t* P,
                                                           size_t n_nodes, double* b);
__attribute__((visibility("hidden"))) int bfmi_sparse_destroy(bfm_matrix_t* A);
__attribute__((visibility("hidden"))) double bfmi_sparse_get(bfm_matrix_t* A, size_t i, size_t j);
__attribute__((visibility("hidden"))) size_t bfmi_sparse_bandwidth(bfm_matrix_t* A);
__attribute__((visibility("hidden"))) int bfmi_sparse_rcm(bfm_perm_t* perm, bfm_matrix_t* A);
__attribute__((visibility("hidden"))) int bfmi_sparse_permute(bfm_perm_t* perm, bfm_matrix_t* A, bool inv);
__attribute__((visibility("hidden"))) int bfmi_sparse_solve(bfm_matrix_t* A, bfm_vec_t* y);

/* Extension slot of a problem: freed by bfm_gpu_problem_destroy. */
__attribute__((visibility("hidden"))) void** bfmi_ext_slot(struct bfm_gpu_problem* P, void (**free_fn)(void*));

/* Preconditioner layout of the next assembly (BFM_GPU_PC_JACOBI: 2 values per
 * node, BFM_GPU_PC_BLOCK_JACOBI: the inverse 2x2 diagonal block); a change
 * marks the problem unassembled.  Used by the batched solver. */
__attribute__((visibility("hidden"))) int bfmi_set_precond(struct bfm_gpu_problem* P, int precond);

/* bfm_gpu_problem_set_geometry from host arrays with 64-bit node ids (the
 * reference's size_t element array), narrowed to int32 on the device: no host
 * pass over the elements.  *bad_index = the lowest position holding an id at
 * or beyond n_nodes (the elements are then not usable), else -1.  Waits for
 * the copies. */
__attribute__((visibility("hidden"))) int bfmi_set_geometry_u64(struct bfm_gpu_problem* P, const double* coords,
                                                                const uint64_t* elems, long* bad_index);

#ifdef __cplusplus
}
#endif
