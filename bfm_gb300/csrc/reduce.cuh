// Deterministic grid reductions and node-pair vector access shared by the
// solver and learned-preconditioner kernels (internal linkage).
#pragma once

#include <cuda_runtime.h>

namespace {

#ifndef BFM_TPB
#define BFM_TPB 256
#endif
constexpr int TPB_K = BFM_TPB;

// ------------------------------------------------------------------ reductions

// Sum NV values over the whole grid: every block writes its partial sums,
// the last block to arrive (atomic ticket) adds them in block order and
// returns true with the totals in `out`.  The result does not depend on which
// block arrives last.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double* __restrict__ partials, unsigned* ticket,
                                         double (&out)[NV]) {
	__shared__ double sm[TPB_K / 32][NV];
	__shared__ bool is_last;
	int const lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
	for (int i = 0; i < NV; i++)
		for (int o = 16; o; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
	if (lane == 0)
		for (int i = 0; i < NV; i++) sm[wid][i] = v[i];
	__syncthreads();
	if (wid == 0) {
#pragma unroll
		for (int i = 0; i < NV; i++) {
			double t = lane < nw ? sm[lane][i] : 0.0;
			for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
			if (lane == 0) partials[blockIdx.x * NV + i] = t;
		}
	}
	if (threadIdx.x == 0) {
		__threadfence();
		unsigned const tk = atomicAdd(ticket, 1u);
		is_last = tk == gridDim.x - 1;
	}
	__syncthreads();
	if (!is_last) return false;
	__threadfence();
	double w[NV];
#pragma unroll
	for (int i = 0; i < NV; i++) w[i] = 0.0;
	for (int blk = threadIdx.x; blk < gridDim.x; blk += blockDim.x)
#pragma unroll
		for (int i = 0; i < NV; i++) w[i] += __ldcg(&partials[blk * NV + i]);
#pragma unroll
	for (int i = 0; i < NV; i++)
		for (int o = 16; o; o >>= 1) w[i] += __shfl_down_sync(0xffffffffu, w[i], o);
	__syncthreads();
	if (lane == 0)
		for (int i = 0; i < NV; i++) sm[wid][i] = w[i];
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int i = 0; i < NV; i++) {
			double t = 0.0;
			for (int k = 0; k < nw; k++) t += sm[k][i];
			out[i] = t;
		}
		*ticket = 0u;
	}
	__syncthreads();
	return true;
}

template <typename V> struct Vec2;
template <> struct Vec2<double> { using T = double2; };
template <> struct Vec2<float> { using T = float2; };

template <typename V>
__device__ __forceinline__ typename Vec2<V>::T ld2(const V* p, int i) {
	return reinterpret_cast<const typename Vec2<V>::T*>(p)[i];
}
template <typename V>
__device__ __forceinline__ void st2(V* p, int i, V a, V b) {
	typename Vec2<V>::T t;
	t.x = a;
	t.y = b;
	reinterpret_cast<typename Vec2<V>::T*>(p)[i] = t;
}

}  // namespace
