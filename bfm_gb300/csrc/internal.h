/* Library-internal helpers shared by the translation units (not exported). */
#pragma once

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
	const float* dinv32;
	const double* vals64;
	const double* b;
	double* x;
	void* vec[5];
	void* stream;
} bfmi_buffers_t;

__attribute__((visibility("hidden"))) int bfmi_buffers(struct bfm_gpu_problem* P, bfmi_buffers_t* out);

/* Extension slot of a problem: freed by bfm_gpu_problem_destroy. */
__attribute__((visibility("hidden"))) void** bfmi_ext_slot(struct bfm_gpu_problem* P, void (**free_fn)(void*));

#ifdef __cplusplus
}
#endif
