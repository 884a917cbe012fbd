/* GB300 hot path of libbfm: additive C ABI.
 *
 * Nothing here replaces or changes a reference prototype.  The reference's
 * hot entry bfm_sim_run (libbfm/src/sim.c:137-155, sim.h:33) keeps its
 * signature and runs on top of these functions; this header adds what the old
 * API cannot express (solver options, statistics, per-element material) and a
 * device-resident problem handle for callers that keep meshes in GPU memory.
 *
 * Conventions: 0 = success, -1 = failure (as the reference, bfm.h:27-34); on
 * failure bfm_gpu_last_error() returns a message.  Plain pointers and sizes
 * only.  `where` arguments say whether a pointer is host (BFM_GPU_HOST) or
 * device (BFM_GPU_DEVICE) memory.  `stream` is a cudaStream_t passed as void*
 * (NULL: the problem creates and owns a stream).
 *
 * Data layout on the device: node coordinates as interleaved doubles,
 * connectivity as int32, stiffness as 2x2-block CSR (one block per pair of
 * nodes sharing an element, columns ascending, block entries row-major
 * k_uu k_uv k_vu k_vv), right-hand side and solution as interleaved u,v.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <bfm/instance.h>
#include <bfm/sim.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { BFM_GPU_HOST = 0, BFM_GPU_DEVICE = 1 };

/* arithmetic of the stiffness matrix and Krylov vectors */
enum {
	BFM_GPU_FP64 = 0,  /* FP64 element integration (reference operation order), FP64 CG          */
	BFM_GPU_MIXED = 1, /* FP32 element integration and SpMV, FP32 Krylov vectors; FP64-accurate
	                      inner products, FP64 solution and FP64 residual replacement with the
	                      FP32 operator widened: converges to the FP32-integrated system         */
	BFM_GPU_MIXED_EXACT = 2, /* as MIXED, but the element loop runs in FP64 once: the FP64 matrix is
	                            the residual operator (solution of the FP64 system) and its FP32
	                            rounding the iteration operator                                    */
	BFM_GPU_FP64_DF = 3, /* FP64-accurate CG on the FP32 pipe: matrix, vectors and solution held as
	                        pairs of floats (about 48 significant bits), error-free FP32
	                        arithmetic; FP64 element loop and final FP64 residual              */
};

/* preconditioner */
enum {
	BFM_GPU_PC_JACOBI = 0,       /* diagonal                                   */
	BFM_GPU_PC_BLOCK_JACOBI = 1, /* inverse of each node's 2x2 diagonal block  */
	BFM_GPU_PC_LEARNED = 2,      /* message-passing network, flexible CG       */
	/* Multicolour block symmetric Gauss-Seidel (SSOR with the 2x2 diagonal
	 * blocks as relaxation blocks), swept colour by colour in FP32.  The
	 * problem is then assembled and solved with its nodes renumbered colour
	 * by colour (bfm_gpu_problem_ordering); bfm_gpu_problem_solution returns
	 * the caller's order.  FP64 and FP64_DF precisions. */
	BFM_GPU_PC_SSOR = 3,
	/* The same sweeps with relaxation blocks from the message-passing
	 * network (bfm_gpu_mpnn_use); block SSOR is its fallback. */
	BFM_GPU_PC_LEARNED_SSOR = 4,
	/* Two-level: the SSOR sweeps plus a coarse correction, additively,
	 * M^-1 = M_SSOR^-1 + P A_c^-1 P^T, with P the rigid-body modes (two
	 * translations and a rotation) of the cells of a grid over the mesh's
	 * bounding box (about one cell per 1,000 nodes, BFM_GPU_COARSE_NODES;
	 * at most 1,024 cells) and A_c = P^T A P factored (band Cholesky, then
	 * X = L^-1) on the device at assembly.  FP64 and FP64_DF. */
	BFM_GPU_PC_SSOR2 = 5,
	/* The two-level form with the network's relaxation blocks. */
	BFM_GPU_PC_LEARNED_SSOR2 = 6,
	/* Batched solver only (bfm_gpu_problem_solve_parts / _step_parts): two-level
	 * block Jacobi, M^-1 = D^-1 + P A_c^-1 P^T per part, with D the nodes' 2x2
	 * diagonal blocks and P the rigid-body modes of the cells of a grid over
	 * each part's bounding box (about one cell per 48 nodes,
	 * BFM_GPU_BATCH_COARSE_NODES; at most 64 cells per part).  A_c = P^T A P
	 * and its inverse are formed on the device at every step, inside the
	 * step's graph.  The iteration count then depends little on a part's
	 * size, so the persistent kernel no longer waits on its largest part. */
	BFM_GPU_PC_TWO_LEVEL_JACOBI = 7,
};

/* solver status codes (bfm_gpu_stats_t.status) */
enum {
	BFM_GPU_OK = 0,
	BFM_GPU_NOT_CONVERGED = 1, /* max_iters reached                         */
	BFM_GPU_BREAKDOWN = 2,     /* p.Ap <= 0 or NaN: matrix not SPD / singular */
	BFM_GPU_BAD_MESH = 3,      /* valence or row length above the kernel caps */
	BFM_GPU_CUDA_ERROR = 4,
	BFM_GPU_STAGNATED = 5,     /* the FP64 true residual stopped decreasing above rtol: the
	                              roundoff floor of this system; x is as accurate as it gets */
	BFM_GPU_TIMEOUT = 6,       /* a grid barrier of a persistent kernel waited past
	                              opts.barrier_polls; the solve stopped, the problem stays usable */
};

typedef struct {
	int precision;     /* BFM_GPU_FP64 or BFM_GPU_MIXED                         */
	int precond;       /* BFM_GPU_PC_*                                          */
	double rtol;       /* stop when the true ||b - A x||_2 <= rtol ||b||_2      */
	int max_iters;     /* hard cap on CG iterations                             */
	double replace_drop; /* replace the recurrence residual by the true residual
	                        (computed from the matrix) each time it has dropped by
	                        this factor, and whenever it claims convergence     */
	int deterministic; /* 1: fixed reduction order (always on; kept for ABI)    */
	int autotune;      /* 1: pick the SpMV shape (lanes per block row) by timing
	                      the candidates on the problem's own matrix, once    */
	int64_t barrier_polls; /* grid barriers inside the persistent kernels (SSOR
	                          sweeps, coarse correction, batched solver) give up
	                          after this many polls and the solve ends with
	                          BFM_GPU_TIMEOUT instead of waiting forever;
	                          0: the default, 2^24 (seconds)                  */
	int refine_restart;    /* MIXED and MIXED_EXACT: every FP64 residual
	                          replacement is an iterative-refinement step
	                          (x += dx in FP64, r = b - A x in compensated
	                          FP64).  0 (default): the inner FP32 PCG keeps its
	                          search direction across it (reliable updates);
	                          1: it restarts from the new residual (beta = 0),
	                          the classic refinement loop                      */
} bfm_gpu_opts_t;

typedef struct {
	int status;           /* BFM_GPU_* status code                        */
	int iterations;       /* CG iterations performed                      */
	int replacements;     /* mixed: FP64 residual replacements             */
	int fallback;         /* learned: 1 if Jacobi took over                */
	double rel_residual;  /* FP64 ||b - A x|| / ||b|| of the returned x    */
	int64_t n_blocks;     /* 2x2 blocks in the stiffness matrix            */
	int64_t n_dof;
	double ms_assemble;   /* pattern + element loop + conditions (device)  */
	double ms_solve;      /* CG (device)                                   */
} bfm_gpu_stats_t;

/* Defaults: FP64, Jacobi, rtol 1e-10, max_iters 200000, replace_drop 0.1, autotune on,
 * barrier_polls 0 (2^24). */
void bfm_gpu_default_opts(bfm_gpu_opts_t* opts);

/* Options used by bfm_sim_run and the bfm_system_* creators of this thread. */
int bfm_gpu_set_opts(const bfm_gpu_opts_t* opts);
int bfm_gpu_get_opts(bfm_gpu_opts_t* opts);

/* Statistics of the last instance solved by bfm_sim_run on this thread. */
int bfm_gpu_last_stats(bfm_gpu_stats_t* stats);

/* Message of the last failure on this thread ("" if none). */
const char* bfm_gpu_last_error(void);

/* Storage of the stiffness matrix the bfm_system_create_planar_* and
 * bfm_system_create_axisymmetric_strain creators of this thread return (an
 * extension: the reference stores it dense, n^2 doubles, system.c:13):
 * BFM_MATRIX_KIND_FULL (the default) or BFM_MATRIX_KIND_SPARSE.  Without a
 * call, BFM_GPU_SYSTEM_STORAGE=sparse in the environment selects SPARSE, and
 * systems whose dense matrix would pass 16 GB are SPARSE anyway.  A SPARSE
 * system renumbers with the reference's RCM (the same permutation) but keeps
 * its storage; bfm_matrix_solve then solves it on the GPU. */
int bfm_gpu_set_system_storage(int kind);

/* Number of usable CUDA devices (0 without a GPU; never fails). */
int bfm_gpu_device_count(void);

/* Per-element Young's modulus and Poisson ratio for one instance (an
 * extension: the reference holds one material per object, obj.h:8-14).
 * Arrays of n_elems doubles, host memory, owned by the caller and read at
 * bfm_sim_run time; NULL for either keeps the material's value.  Passing both
 * NULL removes the override. */
int bfm_gpu_instance_set_elem_material(bfm_instance_t* instance, const double* E, const double* nu);

/* ---------------------------------------------------------------- device-resident problems */

typedef struct bfm_gpu_problem bfm_gpu_problem_t;

/* Allocate device storage for a mesh of n_nodes nodes and n_elems elements of
 * `kind` nodes (3 or 4), with up to n_edges boundary edges and n_conds
 * conditions.  Sizes every buffer for the worst case, so nothing is
 * allocated after this call. */
int bfm_gpu_problem_create(bfm_gpu_problem_t** problem, int kind, int n_nodes, int n_elems,
                           int n_edges, int n_conds, void* stream);
int bfm_gpu_problem_destroy(bfm_gpu_problem_t* problem);

/* coords[2*n_nodes] (x,y interleaved), elems[kind*n_elems] (int32). */
int bfm_gpu_problem_set_geometry(bfm_gpu_problem_t* problem, const double* coords, const int32_t* elems, int where);

/* Uniform material (E, nu, rho) and the element formulation `stress`:
 * plane strain (0), plane stress (1), axisymmetric with x the radius (2), or
 * axisymmetric with the reference's formulas (3: libbfm/src/system.c:241,
 * 337 and 591-601 as written, for bit-exact parity; K is then indefinite for
 * usual nu and CG is not expected to converge).
 * elem_E / elem_nu (n_elems each, may be NULL) override E / nu per element.
 * Per-edge loads (bfm_gpu_problem_set_edge_loads) are planar only. */
int bfm_gpu_problem_set_material(bfm_gpu_problem_t* problem, double E, double nu, double rho, int stress,
                                 const double* elem_E, const double* elem_nu, int where);

/* Integration rule sampled on the host: weights[n_points], and phi, dxi, deta
 * [n_points*kind] (shape value and derivatives at each point). */
int bfm_gpu_problem_set_rule(bfm_gpu_problem_t* problem, int n_points, const double* weights,
                             const double* phi, const double* dxi, const double* deta);

/* Body forces (accelerations, multiplied by rho as in the reference).
 * force k is constant (values[2k..2k+1]) when node_values[k] is NULL, else a
 * per-node field node_values[k][2*n_nodes] in `where` memory. */
int bfm_gpu_problem_set_forces(bfm_gpu_problem_t* problem, int n_forces, const double* values,
                               const double* const* node_values, int where);

/* Conditions in application order: kinds[c] (BFM_CONDITION_KIND_DIRICHLET_X/Y,
 * NEUMANN_X/Y), values[c], masks[c*n_nodes + i] != 0 when node i is flagged;
 * edges[2*n_edges] node pairs used by the Neumann conditions. */
int bfm_gpu_problem_set_conditions(bfm_gpu_problem_t* problem, int n_conds, const int* kinds, const double* values,
                                   const uint8_t* masks, int n_edges, const int32_t* edges, int where);

/* Enqueue: sparsity pattern, element loop, Dirichlet elimination, Neumann
 * loads and preconditioner set-up, in `precision`.  Asynchronous. */
int bfm_gpu_problem_assemble(bfm_gpu_problem_t* problem, int precision);

/* Enqueue the CG solve (one CUDA graph launch).  Asynchronous; statistics via
 * bfm_gpu_problem_stats. */
int bfm_gpu_problem_solve(bfm_gpu_problem_t* problem, const bfm_gpu_opts_t* opts);

/* Wait for the problem's stream and report the last assemble/solve. */
int bfm_gpu_problem_stats(bfm_gpu_problem_t* problem, bfm_gpu_stats_t* stats);

/* Copy the solution (2*n_nodes doubles, interleaved u,v) out. */
int bfm_gpu_problem_solution(bfm_gpu_problem_t* problem, double* out, int where);

/* Inspection: number of 2x2 blocks of the last assembled matrix. */
int bfm_gpu_problem_n_blocks(bfm_gpu_problem_t* problem, int64_t* n_blocks);

/* Inspection: copy the assembled system to the host.  row_ptr[n_nodes+1] and
 * cols[n_blocks] of the node-block pattern, vals[4*n_blocks] (FP64; FP32
 * entries widened in mixed precision) and b[2*n_nodes].  Any may be NULL.
 * Like bfm_gpu_problem_apply, it works in the problem's working node order
 * (bfm_gpu_problem_ordering). */
int bfm_gpu_problem_download(bfm_gpu_problem_t* problem, int32_t* row_ptr, int32_t* cols, double* vals, double* b);

/* Measurement hook: launch the CG's SpMV+dots kernel and its vector-update
 * kernel `reps` times each on the problem's stream and return their mean
 * durations (ms, CUDA events).  Overwrites the Krylov vectors. */
int bfm_gpu_problem_time_kernels(bfm_gpu_problem_t* problem, int reps, double* ms_spmv, double* ms_update);

/* Project autotuner: time the SpMV shapes -- 1, 2, 4, 8 or 16 lanes per block
 * row, and 1, 2, 4 or 8 entries batched per lane (column indices, then
 * gathers and block loads, then arithmetic) -- on the assembled matrix and
 * keep the fastest for this problem's solves.  Returns the lanes per row of
 * the winner (and its shape code, lanes + 100 x batch, if shape != NULL).
 * Overwrites the Krylov vectors. */
int bfm_gpu_problem_autotune(bfm_gpu_problem_t* problem, int* lanes_per_row);
int bfm_gpu_problem_shape(bfm_gpu_problem_t* problem, int* shape);
/* Force an SpMV shape code (as returned above; 0 restores autotuning). */
int bfm_gpu_problem_set_shape(bfm_gpu_problem_t* problem, int shape);

/* The CUDA stream the problem's work is enqueued on (cudaStream_t as void*). */
void* bfm_gpu_problem_stream(bfm_gpu_problem_t* problem);

/* Per-edge tractions, an extension of the Neumann X/Y conditions for loads
 * that differ from edge to edge: edge e (nodes edges[2e], edges[2e+1])
 * carries the traction (loads[2e], loads[2e+1]) per unit length, and each of
 * its ends receives length/2 times it, as the reference's Neumann loop does
 * (system.c:477-498).  DOFs under a Dirichlet condition keep their value.
 * Applied by the next bfm_gpu_problem_assemble. */
int bfm_gpu_problem_set_edge_loads(bfm_gpu_problem_t* problem, int n_loads, const int32_t* edges, const double* loads,
                                   int where);

/* ---------------------------------------------------------------- batches of uneven meshes */

/* Declare the problem a batch: node ranges [node_offsets[k], node_offsets[k+1])
 * (host array of n_parts+1, from 0 to n_nodes, 1 <= n_parts <= 512) are
 * independent meshes sharing no element.  Their elements are assembled
 * together as one block-diagonal system (bfm_gpu_problem_assemble), and
 * bfm_gpu_problem_solve_parts then solves every part with its own CG. */
int bfm_gpu_problem_set_parts(bfm_gpu_problem_t* problem, int n_parts, const int32_t* node_offsets);

/* Per edge of the last bfm_gpu_problem_set_conditions call: 1 if the edge has
 * one adjacent element (a boundary edge), 0 otherwise.  The normal/tangent
 * Dirichlet conditions sum over boundary edges only (reference system.c:396);
 * without this call every edge counts as one. */
int bfm_gpu_problem_set_edge_boundary(bfm_gpu_problem_t* problem, const uint8_t* boundary, int where);

/* Enqueue the batched solve: one kernel launch in which each part runs
 * mixed-precision PCG (FP32 operator and vectors, FP64 inner products and
 * residual replacement) with its own scalars and stopping test, captured in a
 * CUDA graph.  Preconditioner (opts->precond): BFM_GPU_PC_JACOBI,
 * BFM_GPU_PC_BLOCK_JACOBI or BFM_GPU_PC_TWO_LEVEL_JACOBI.  When every part
 * has at most 131,072 nodes, one thread block runs each part (block barriers
 * only, largest parts launched first); otherwise, or with
 * BFM_GPU_BATCH_KERNEL=tiled when the parts are set, one persistent
 * cooperative kernel cuts the parts into row tiles, with grid barriers that
 * wait a bounded time and then report an error.  Needs an assembly in
 * BFM_GPU_MIXED or BFM_GPU_MIXED_EXACT.  With opts->autotune the first call
 * times the shapes (threads per block, or rows per tile, x lanes per row) on
 * this batch and keeps the fastest. */
int bfm_gpu_problem_solve_parts(bfm_gpu_problem_t* problem, const bfm_gpu_opts_t* opts);

/* One step of the batch -- assembly in `precision` (MIXED or MIXED_EXACT)
 * and the batched solve -- as ONE CUDA graph launch: the first call runs the
 * step directly (sizing every buffer, tuning the tile shape), then captures
 * the whole step (pattern, element loop, conditions, loads, the persistent
 * solver kernel and the per-part residuals) into a graph that later calls
 * replay.  A change of options, precision or any input set through
 * bfm_gpu_problem_set_* captures again.  Asynchronous; statistics via
 * bfm_gpu_problem_part_stats (ms_solve: the device time of the whole step). */
int bfm_gpu_problem_step_parts(bfm_gpu_problem_t* problem, int precision, const bfm_gpu_opts_t* opts);

/* After a batched solve with BFM_GPU_PC_TWO_LEVEL_JACOBI: per part its number
 * of coarse DOFs (3 per cell) and where its A_c^-1 starts in `ainv`
 * (ainv_offsets has n_parts + 1 entries), and every part's A_c^-1 (FP32,
 * dense, row-major; ainv_offsets[n_parts] floats).  Any pointer may be NULL. */
int bfm_gpu_problem_parts_coarse(bfm_gpu_problem_t* problem, int* n_coarse, int64_t* ainv_offsets, float* ainv);

/* Wait, then per part (arrays of n_parts, any may be NULL): iterations,
 * status (BFM_GPU_*), FP64 residual replacements, FP64 relative residual;
 * and the shape used (rows_per_tile: the threads per block of the
 * block-per-part kernel, or the rows per tile of the tiled one; lanes per
 * row) and the device time of the last solve. */
int bfm_gpu_problem_part_stats(bfm_gpu_problem_t* problem, int* iterations, int* status, int* replacements,
                               double* rel_residual, int* rows_per_tile, int* lanes_per_row, double* ms_solve);

/* Mean duration (ms) of one application of an SSOR preconditioner (the
 * coarse correction of the two-level form and every sweep phase) over `reps`
 * standalone launches on a scratch solver state; *ms_sweeps (may be NULL)
 * the sweeps alone; *persistent = 1 when the phases run as one cooperative
 * kernel, 2 when that kernel stages its operands by TMA (k_ssor_tma).  Needs a solve with one of the SSOR preconditioners first (which
 * forms the colour order); overwrites the Krylov vectors. */
int bfm_gpu_problem_time_precond(bfm_gpu_problem_t* problem, int reps, double* ms, double* ms_sweeps, int* persistent);

/* The coarse space of the two-level SSOR preconditioner after a solve with
 * it: *n_coarse coarse DOFs (0: none; the solve ran plain SSOR), *n_chunks
 * restriction chunks, *x_bytes the bytes of X = L^-1 and X^T the correction
 * reads per application, *fused = 1 when the correction runs inside the
 * sweep kernel.  Any pointer may be NULL. */
int bfm_gpu_problem_coarse_info(bfm_gpu_problem_t* problem, int64_t* n_coarse, int64_t* n_chunks, int64_t* x_bytes,
                                int* fused);

/* Working node order of the last assembly: perm[w] = the caller's index of
 * working node w (n_nodes ints, host memory; the identity unless an SSOR
 * preconditioner renumbered the nodes colour by colour), and the colour
 * ranges: the nodes of colour c are [color_offsets[c], color_offsets[c+1])
 * (at most 65 ints; *n_colors = 0 for the caller's order).  Any may be NULL. */
int bfm_gpu_problem_ordering(bfm_gpu_problem_t* problem, int32_t* perm, int32_t* color_offsets, int* n_colors);

/* y = K x with the assembled FP64 operator (after Dirichlet elimination);
 * x and y are 2*n_nodes doubles in host or device memory (`where`).  Needs an
 * assembly in FP64, MIXED_EXACT or FP64_DF.  Forms r = K e from an error e
 * when generating training pairs for the learned preconditioner. */
int bfm_gpu_problem_apply(bfm_gpu_problem_t* problem, const double* x, double* y, int where);

/* ---------------------------------------------------------------- learned preconditioner */

/* No counterpart in the reference.  A message-passing network over the node
 * graph predicts, per node i, a correction C_i of the block-Jacobi block:
 *     B_i = K_ii^-1 + L_i C_i L_i^T,  L_i L_i^T = K_ii^-1 (Cholesky),
 *     C_i = 0.45 tanh(o_i) as [[c0, c1], [c1, c2]]
 * (K_ii: node i's 2x2 diagonal block; o_i: the network's 3 outputs).  B_i =
 * L_i (I + C_i) L_i^T is SPD for any output, and PCG uses it in place of the
 * Jacobi diagonal when opts->precond is BFM_GPU_PC_LEARNED.  Inputs per node:
 * log-stiffness contrasts of the incident elements, Poisson ratio, Dirichlet
 * flags, graph degree, the Jacobi-scaled load (the initial residual), and the
 * diagonal block's scale ratio and coupling.  Layers: 16 -> 64, three times
 * [h, mean of h over the graph row] 128 -> 64 (ReLU), head 64 -> 3.  BF16
 * weights and activations on the tensor cores, FP32 accumulation and FP32
 * master weights; 26,051 parameters.  An untrained network (zero head) gives
 * block Jacobi.  The solve falls back to plain Jacobi (stats.fallback = 1)
 * when the learned solve breaks down or stagnates above 1e-6. */
typedef struct bfm_gpu_mpnn bfm_gpu_mpnn_t;

int bfm_gpu_mpnn_param_count(void);
/* He-normal hidden weights from `seed`, zero biases, zero head. */
int bfm_gpu_mpnn_create(bfm_gpu_mpnn_t** net, unsigned seed);
int bfm_gpu_mpnn_destroy(bfm_gpu_mpnn_t* net);
/* FP32 parameters in the order W0[64x16], b0, W1[64x128], b1, W2, b2, W3, b3,
 * Wo[3x64], bo (row-major, out x in); host memory. */
int bfm_gpu_mpnn_get_weights(bfm_gpu_mpnn_t* net, float* theta);
int bfm_gpu_mpnn_set_weights(bfm_gpu_mpnn_t* net, const float* theta);
/* Versioned weights file: "BFMMPNN\0", u32 version, input width, hidden
 * width, layers, outputs, parameter count, FP32 parameters. */
int bfm_gpu_mpnn_save(bfm_gpu_mpnn_t* net, const char* path);
int bfm_gpu_mpnn_load(bfm_gpu_mpnn_t* net, const char* path);
/* Run the network on an assembled problem; any output may be NULL (host):
 * features[16*n_nodes] as fed to the first layer (BF16 values), c[3*n_nodes]
 * = (c0, c1, c2) per node, blocks[4*n_nodes] = B_i row-major. */
int bfm_gpu_mpnn_forward(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* problem, float* features, float* c, double* blocks);
/* Training loss of one (residual r = K e, error e) pair: the log of a
 * condition-number estimate of the preconditioned operator B K,
 *     L = log R(v) - log R(e),  R(x) = (x.K x) / (x.B^-1 x),
 * with v the power-iteration vector of B K (top of its spectrum) and e a
 * solver error (smooth: the bottom).  v (device, 2*n_nodes doubles, kept by
 * the caller between calls) first takes power_iters steps v <- B K v with the
 * current network.  Returns the loss and its gradient (FP32, parameter order
 * above; NULL to skip).  r and e are device arrays of 2*n_nodes doubles;
 * needs the FP64 operator. */
int bfm_gpu_mpnn_gradient(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* problem, const double* r, const double* e,
                          double* v, int power_iters, double* loss, float* grad);
/* One Adam step (beta 0.9 / 0.999) on that gradient; loss may be NULL. */
int bfm_gpu_mpnn_train_step(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* problem, const double* r, const double* e,
                            double* v, int power_iters, double lr, double* loss);
/* Network used by BFM_GPU_PC_LEARNED solves (NULL: none). */
int bfm_gpu_mpnn_use(bfm_gpu_mpnn_t* net);

/* ---------------------------------------------------------------- allocation-free solve */

/* No counterpart in the reference: an additive entry point for callers that
 * cannot allocate device memory (an application that owns every device byte
 * through its own pool, or code that must not call cudaMalloc).  Solves
 * A x = b by FP64 Jacobi-PCG with the kernels and stopping rule of
 * bfm_gpu_problem_solve's FP64 path (Hestenes-Stiefel PCG with FP64 true
 * residual replacements; converged when the true residual is at most rtol,
 * or stagnated at the roundoff floor above it), launched from a host loop.
 * A is a 2x2-block CSR matrix already in device memory: row_ptr[n_nodes+1],
 * cols[row_ptr[n_nodes]], vals[4*row_ptr[n_nodes]] (the layout
 * bfm_gpu_problem_download returns), b and x interleaved u,v, all device
 * pointers; x is written.  Nothing is allocated: the Krylov vectors and
 * solver state live in a fixed scratch array of about 6.4 MB that the library
 * keeps on every GPU that loads it, which limits n_nodes to 65,536
 * (131,072 DOF); larger sizes return -1 with a message.  Every call looks up
 * that array's address on the current device.  The call waits on `stream`
 * and reads the solver state back, so it must not be made while that stream
 * is being captured.  Calls share the array, so calls that overlap on the
 * GPU (two streams, two threads) race: serialize them.  Reports the
 * iteration count and the FP64 relative residual of x; returns 0 when
 * converged or stagnated (as bfm_sim_run), -1 when CG does not converge or
 * breaks down. */
int bfm_gpu_pcg_solve_noalloc(int n_nodes, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                              const double* b, double* x, double rtol, int max_iters, int* iterations,
                              double* rel_residual, void* stream);

/* ---------------------------------------------------------------- sparse RCM */

/* Reverse Cuthill-McKee of a scalar CSR matrix (columns ascending per row),
 * ignoring entries that are exactly zero: the permutation the reference's
 * bfm_perm_rcm (perm.c:117-331) computes on the equivalent dense matrix,
 * bit for bit, in O(nnz log) instead of O(n^2).  perm[old] = new. */
int bfm_gpu_rcm_csr(int64_t n, const int64_t* row_ptr, const int64_t* cols, const double* vals,
                    int64_t* perm, int64_t* inv_perm);

#ifdef __cplusplus
}
#endif
