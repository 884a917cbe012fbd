// Allocation-free FP64 Jacobi-PCG entry point of the GB300 libbfm (see
// bfm_gpu_pcg_solve_noalloc in include/bfm/gpu.h).
#include <cuda_runtime.h>

#include <math.h>
#include <pthread.h>
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
// bfm_gpu_pcg_solve_noalloc: the FP64 Jacobi-PCG of bfm_gpu_problem_solve for
// a caller who already holds the matrix, right-hand side and solution in
// device memory and cannot allocate any more (a solver embedded in a larger
// application that owns every device byte, or code that must not call
// cudaMalloc at all).  Its Krylov vectors, reduction slots and solver state
// live in the fixed array below, which every GPU that loads the library holds
// until the process exits.

namespace {

constexpr int NOALLOC_MAX_NODES = 65536;  // 131,072 DOF
constexpr int NOALLOC_MAX_GRID = 2048;
constexpr size_t NOALLOC_VEC = 2ul * NOALLOC_MAX_NODES * sizeof(double);      // one interleaved vector
constexpr size_t NOALLOC_PARTIALS = 4ul * NOALLOC_MAX_GRID * sizeof(double);
constexpr size_t NOALLOC_STATE = (sizeof(CgState) + 255) / 256 * 256;
constexpr size_t NOALLOC_BYTES = 6 * NOALLOC_VEC + NOALLOC_PARTIALS + NOALLOC_STATE + 256;  // about 6.4 MB

// Host code must not take this symbol's address directly: on the host it is
// a stand-in, not a device address.  The device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// per-device device address of g_noalloc_scratch (set-up on a device's first call)
void* g_noalloc_base[64];
pthread_mutex_t g_noalloc_lock = PTHREAD_MUTEX_INITIALIZER;

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
	if (dev < 0 || dev >= 64) return fail("device ordinal %d out of range", dev);
	pthread_mutex_lock(&g_noalloc_lock);
	if (!g_noalloc_base[dev]) {
		void* ptr = nullptr;
		cudaError_t const e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
		if (e != cudaSuccess) {
			pthread_mutex_unlock(&g_noalloc_lock);
			return fail("cudaGetSymbolAddress of the solver scratch failed: %s", cudaGetErrorString(e));
		}
		g_noalloc_base[dev] = ptr;
	}
	unsigned char* const base = (unsigned char*) g_noalloc_base[dev];
	pthread_mutex_unlock(&g_noalloc_lock);
	cudaStream_t const st = (cudaStream_t) stream;
	int sms = 0;
	CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
	int const grid = 4 * sms < NOALLOC_MAX_GRID ? 4 * sms : NOALLOC_MAX_GRID;

	CgArgs<double> a;
	memset(&a, 0, sizeof a);
	a.N = n_nodes;
	a.row_ptr = row_ptr;
	a.cols = cols;
	a.vals = vals;
	a.vals64 = vals;
	a.r = (double*) (base + 0 * NOALLOC_VEC);
	a.u = (double*) (base + 1 * NOALLOC_VEC);
	a.p = (double*) (base + 2 * NOALLOC_VEC);
	a.s = (double*) (base + 3 * NOALLOC_VEC);
	a.w = (double*) (base + 4 * NOALLOC_VEC);
	double* const dinv = (double*) (base + 5 * NOALLOC_VEC);
	a.dinv = dinv;
	a.partials = (double*) (base + 6 * NOALLOC_VEC);
	a.st = (CgState*) (base + 6 * NOALLOC_VEC + NOALLOC_PARTIALS);
	a.ticket = (unsigned*) (base + 6 * NOALLOC_VEC + NOALLOC_PARTIALS + NOALLOC_STATE);
	a.b = b;
	a.x = x;
	a.opts.rtol = rtol;
	a.opts.max_iters = max_iters;

	// the array keeps the previous call's contents: the reduction ticket must start at zero
	CK(cudaMemsetAsync(a.ticket, 0, sizeof(unsigned), st));
	k_noalloc_diag<<<blocks_for(n_nodes), TPB_K, 0, st>>>(n_nodes, row_ptr, cols, vals, dinv);
	k_cg_init<double><<<grid, TPB_K, 0, st>>>(a, 0);
	CK(cudaGetLastError());
	CgState h;
	int const chunk = 32;
	for (long launched = 0;; launched += chunk) {
		for (int k = 0; k < chunk; k++) {
			k_cg64_spmv<8><<<grid, TPB_K, 0, st>>>(a);
			k_cg64_update<<<grid, TPB_K, 0, st>>>(a);
		}
		CK(cudaGetLastError());
		CK(cudaMemcpyAsync(&h, a.st, sizeof h, cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		// the kernels stop themselves (converged, max_iters or breakdown); the
		// host bound only guards against a state that never reports done
		if (h.done || launched > (long) max_iters + 2 * chunk) break;
	}
	k_true_residual<8, double><<<grid, TPB_K, 0, st>>>(a);
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(&h, a.st, sizeof h, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	if (iterations) *iterations = h.iter;
	if (rel_residual) *rel_residual = h.bnorm2 > 0 ? sqrt(h.true_res2 / h.bnorm2) : 0.0;
	if (!h.done) return fail("bfm_gpu_pcg_solve_noalloc: solver state never reported completion");
	if (h.status == BFM_GPU_NOT_CONVERGED) return fail("CG did not reach rtol %g in %d iterations", rtol, h.iter);
	if (h.status == BFM_GPU_BREAKDOWN) return fail("CG broke down after %d iterations (matrix not SPD?)", h.iter);
	return 0;
}
