// Allocation-free FP64 Jacobi-PCG entry point of the GB300 libbfm (see
// bfm_gpu_pcg_solve_noalloc in include/bfm/gpu.h).
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <bfm/gpu.h>

#include "internal.h"

#include "cg_kernels.cuh"

namespace {

thread_local char g_na_err[512];

int fail(const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_na_err, sizeof g_na_err, fmt, ap);
	va_end(ap);
	bfm_gpu_set_last_error(g_na_err);
	return -1;
}

#define CK(call)                                                                                     \
	do {                                                                                             \
		cudaError_t const e_ = (call);                                                               \
		if (e_ != cudaSuccess) return fail("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
	} while (0)

inline int blocks_for(long n, int tpb = TPB_K) { return (int) ((n + tpb - 1) / tpb) > 0 ? (int) ((n + tpb - 1) / tpb) : 1; }

}  // namespace

// ====================================================================== allocation-free solve
//
// bfm_gpu_pcg_solve_noalloc: FP64 Jacobi-PCG for a caller who already holds
// the matrix, right-hand side and solution in device memory and cannot
// allocate any more (a solver embedded in a larger application that owns
// every device byte, or code that must not call cudaMalloc at all).  It
// runs the kernels of bfm_gpu_problem_solve's FP64 path -- Hestenes-Stiefel
// PCG with reliable updates: an FP64 true residual (compensated) whenever the
// recurrence residual has dropped by 10 or claims convergence, convergence
// judged on that true residual only, stagnation after five replacements in a
// row without halving the best one -- launched from a host loop instead of a
// CUDA graph.  Its Krylov vectors, reduction slots and solver state live in
// the fixed array below, which every GPU that loads the library holds until
// the process exits.

namespace {

constexpr int NOALLOC_MAX_NODES = 65536;  // 131,072 DOF
constexpr int NOALLOC_MAX_GRID = 2048;
constexpr size_t NOALLOC_VEC = 2ul * NOALLOC_MAX_NODES * sizeof(double);      // one interleaved vector
constexpr size_t NOALLOC_PARTIALS = 4ul * NOALLOC_MAX_GRID * sizeof(double);
constexpr size_t NOALLOC_STATE = (sizeof(CgState) + 255) / 256 * 256;
constexpr size_t NOALLOC_BYTES = 6 * NOALLOC_VEC + NOALLOC_PARTIALS + NOALLOC_STATE + 256;  // about 6.4 MB

// Host code must not take this symbol's address directly: on the host it is
// a stand-in, not a device address.  Every call asks cudaGetSymbolAddress
// for the current device's address (a host-side lookup; it stays right after
// a context reset, which may move the array).
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Jacobi diagonal of a caller's 2x2-block matrix
__global__ void k_noalloc_diag(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                               const double* __restrict__ vals, double* __restrict__ dinv) {
	int const r = blockIdx.x * blockDim.x + threadIdx.x;
	if (r >= N) return;
	double d0 = 0.0, d1 = 0.0;
	for (int k = row_ptr[r]; k < row_ptr[r + 1]; k++)
		if (cols[k] == r) {
			d0 = vals[4l * k];
			d1 = vals[4l * k + 3];
		}
	dinv[2 * r] = d0 != 0.0 ? 1.0 / d0 : 0.0;
	dinv[2 * r + 1] = d1 != 0.0 ? 1.0 / d1 : 0.0;
}

}  // namespace

extern "C" int bfm_gpu_pcg_solve_noalloc(int n_nodes, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                                         const double* b, double* x, double rtol, int max_iters, int* iterations,
                                         double* rel_residual, void* stream) {
	g_na_err[0] = 0;
	bfm_gpu_set_last_error("");
	if (n_nodes <= 0 || n_nodes > NOALLOC_MAX_NODES)
		return fail("bfm_gpu_pcg_solve_noalloc handles 1 to %d nodes (%d DOF); got %d nodes", NOALLOC_MAX_NODES,
		            2 * NOALLOC_MAX_NODES, n_nodes);
	if (!row_ptr || !cols || !vals || !b || !x) return fail("bfm_gpu_pcg_solve_noalloc: null pointer");
	if (!(rtol >= 0.0) || max_iters < 0) return fail("bfm_gpu_pcg_solve_noalloc: invalid rtol or max_iters");
	int dev = 0;
	CK(cudaGetDevice(&dev));
	void* ptr = nullptr;
	cudaError_t const e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
	if (e != cudaSuccess) return fail("cudaGetSymbolAddress of the solver scratch failed: %s", cudaGetErrorString(e));
	unsigned char* const base = (unsigned char*) ptr;
	cudaStream_t const st = (cudaStream_t) stream;
	int sms = 0;
	CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	int const grid = 4 * sms < NOALLOC_MAX_GRID ? 4 * sms : NOALLOC_MAX_GRID;

	// vectors: r, z (u), p and p' (ping-pong), q (w); the Jacobi diagonal
	CgArgs<double> a[2];
	memset(&a[0], 0, sizeof a[0]);
	a[0].N = n_nodes;
	a[0].row_ptr = row_ptr;
	a[0].cols = cols;
	a[0].vals = vals;
	a[0].vals64 = vals;
	a[0].r = (double*) (base + 0 * NOALLOC_VEC);
	a[0].u = (double*) (base + 1 * NOALLOC_VEC);
	a[0].p = (double*) (base + 2 * NOALLOC_VEC);
	a[0].pn = (double*) (base + 3 * NOALLOC_VEC);
	a[0].w = (double*) (base + 4 * NOALLOC_VEC);
	a[0].s = a[0].pn;  // written by the init only (as p's zero start)
	double* const dinv = (double*) (base + 5 * NOALLOC_VEC);
	a[0].dinv = dinv;
	a[0].partials = (double*) (base + 6 * NOALLOC_VEC);
	a[0].st = (CgState*) (base + 6 * NOALLOC_VEC + NOALLOC_PARTIALS);
	a[0].ticket = (unsigned*) (base + 6 * NOALLOC_VEC + NOALLOC_PARTIALS + NOALLOC_STATE);
	a[0].b = b;
	a[0].x = x;
	a[0].opts.rtol = rtol;
	a[0].opts.drop2 = 0.1 * 0.1;  // bfm_gpu_default_opts' replace_drop
	a[0].opts.max_iters = max_iters;
	a[1] = a[0];
	a[1].p = a[0].pn;
	a[1].pn = a[0].p;

	// the array keeps the previous call's contents: the reduction ticket must start at zero
	CK(cudaMemsetAsync(a[0].ticket, 0, sizeof(unsigned), st));
	k_noalloc_diag<<<blocks_for(n_nodes), TPB_K, 0, st>>>(n_nodes, row_ptr, cols, vals, dinv);
	k_cg_init<double><<<grid, TPB_K, 0, st>>>(a[0], 0);
	CK(cudaGetLastError());
	CgState h;
	int const chunk = 16;  // iterations between host checks (each a pair, p and p' swapping)
	for (long launched = 0;; launched += 2 * chunk) {
		for (int k = 0; k < chunk; k++)
			for (int half = 0; half < 2; half++) {
				k_hs64_spmv<8><<<grid, TPB_K, 0, st>>>(a[half]);
				k_hs64_update<<<grid, TPB_K, 0, st>>>(a[half]);
				k_hs64_replace<8><<<grid, TPB_K, 0, st>>>(a[half]);
			}
		CK(cudaGetLastError());
		CK(cudaMemcpyAsync(&h, a[0].st, sizeof h, cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		// the kernels stop themselves (converged or stagnated on the FP64 true
		// residual, max_iters, breakdown); the host bound only guards against a
		// state that never reports done
		if (h.done || launched > (long) max_iters + 4 * chunk) break;
	}
	// the reported residual: ||b - A x|| of the returned x
	k_true_residual<8, double><<<grid, TPB_K, 0, st>>>(a[0]);
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(&h, a[0].st, sizeof h, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	double const rel = h.bnorm2 > 0 ? sqrt(h.true_res2 / h.bnorm2) : 0.0;
	if (iterations) *iterations = h.iter;
	if (rel_residual) *rel_residual = rel;
	if (!h.done) return fail("bfm_gpu_pcg_solve_noalloc: solver state never reported completion");
	if (h.status == BFM_GPU_NOT_CONVERGED) return fail("CG did not reach rtol %g in %d iterations", rtol, h.iter);
	if (h.status == BFM_GPU_BREAKDOWN) return fail("CG broke down after %d iterations (matrix not SPD?)", h.iter);
	if (h.status != BFM_GPU_OK && h.status != BFM_GPU_STAGNATED) return fail("CG ended with status %d", h.status);
	// BFM_GPU_STAGNATED: the FP64 true residual stopped decreasing above rtol
	// (the roundoff floor of this system); x is as accurate as FP64 gets, as
	// bfm_sim_run also accepts
	return 0;
}
