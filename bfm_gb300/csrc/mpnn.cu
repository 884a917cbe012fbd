// Learned block preconditioner of the GB300 libbfm: a message-passing network
// over the mesh's node graph that predicts, per node, a correction of the
// block-Jacobi block,
//     B_i = K_ii^-1 + L_i C_i L_i^T,  L_i L_i^T = K_ii^-1,  C_i = [[c0, c1], [c1, c2]],
// used in place of the Jacobi diagonal inside PCG (c = 0 is block Jacobi,
// which is where an untrained network starts).  No counterpart in the
// reference; its CPU oracle is oracle/mpnn_ref.py.
//
// Network: h0 = relu(W0 f + b0) (16 -> 64); three layers
// h = relu(W [h, mean_nbr(h)] + b) (128 -> 64); head c = 0.45 tanh(Wo h + bo)
// (64 -> 3).  Weights are FP32 masters with BF16 copies; the dense layers of
// the forward pass and both GEMMs of each layer's backward pass (dX and dW)
// run on the tensor cores (mma.sync m16n8k16, BF16 inputs, FP32
// accumulation).  Everything per node is deterministic: split-K partials are
// reduced in block order.
//
// Training loss of one (residual r = K e, error e) pair: the log of a
// condition-number estimate of the preconditioned operator,
//     L = log R(v) - log R(e),  R(x) = (x.K x) / (x.B^-1 x),
// v a power-iteration vector of B K (top of the spectrum), e the solver's
// error (bottom of the spectrum).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <bfm/gpu.h>

#include "internal.h"
#include "trace.h"
#include "reduce.cuh"

namespace {

constexpr int FIN = 16, HID = 64, HK = 128;
constexpr int NPARAM = HID * FIN + HID + 3 * (HID * HK + HID) + 3 * HID + 3;
// offsets of the parameter blocks, in the oracle's order
constexpr int O_W0 = 0, O_B0 = O_W0 + HID * FIN, O_W1 = O_B0 + HID;
constexpr int O_WO = O_W1 + 3 * (HID * HK + HID), O_BO = O_WO + 3 * HID;
__host__ __device__ constexpr int o_w(int l) { return O_W1 + (l - 1) * (HID * HK + HID); }  // l = 1..3
__host__ __device__ constexpr int o_b(int l) { return o_w(l) + HID * HK; }
constexpr float C_SCALE = 0.45f;
constexpr int MT = 128;        // threads per block of the tensor-core kernels
constexpr int TILE = 64;       // nodes per tile
constexpr int DW_CHUNK = 2048; // nodes per block in the weight-gradient reduction
constexpr int FEAT_GRID = 256; // blocks of the reduction kernels

thread_local char g_merr[512];

int mfail(const char* fmt, ...) {
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_merr, sizeof g_merr, fmt, ap);
	va_end(ap);
	bfm_gpu_set_last_error(g_merr);
	return -1;
}

#define MCK(call)                                                                                     \
	do {                                                                                              \
		cudaError_t const e_ = (call);                                                                \
		if (e_ != cudaSuccess) return mfail("CUDA error %s at %s:%d", cudaGetErrorString(e_), __FILE__, __LINE__); \
	} while (0)

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
	return (uint32_t) __bfloat16_as_ushort(lo) | ((uint32_t) __bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t const (&a)[4], uint32_t b0, uint32_t b1) {
	asm volatile(
		"mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
		: "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
		: "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One warp: acc[j] (16 x 8 tile j) += A(16 x K) B(K x 8j..8j+7).  The
// accessors return operand elements from shared memory, so transposed
// operands cost nothing; fragments follow the m16n8k16 register layout
// (group g = lane/4, thread t = lane%4).
template <int NT, typename FA, typename FB>
__device__ __forceinline__ void warp_gemm(float (&acc)[NT][4], int K, FA at_a, FB at_b) {
	int const lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	for (int k0 = 0; k0 < K; k0 += 16) {
		int const k1 = k0 + 2 * t;
		uint32_t a[4];
		a[0] = pack2(at_a(g, k1), at_a(g, k1 + 1));
		a[1] = pack2(at_a(g + 8, k1), at_a(g + 8, k1 + 1));
		a[2] = pack2(at_a(g, k1 + 8), at_a(g, k1 + 9));
		a[3] = pack2(at_a(g + 8, k1 + 8), at_a(g + 8, k1 + 9));
#pragma unroll
		for (int j = 0; j < NT; j++) {
			int const n = 8 * j + g;
			mma16816(acc[j], a, pack2(at_b(k1, n), at_b(k1 + 1, n)), pack2(at_b(k1 + 8, n), at_b(k1 + 9, n)));
		}
	}
}

struct MpnnDev {
	float* theta;   // FP32 masters
	float* grad;
	float* adam_m;
	float* adam_v;
	bf16* wb;       // BF16 copies, same offsets as theta (biases unused)
	double* gpart;  // split-K partials of the weight gradients
	long gpart_cap;
};

// ---------------------------------------------------------------- features

struct FeatArgs {
	int N, kind, n_elems;
	const int* inc_ptr;
	const int* inc;
	const double* elemE;
	const double* elemNu;
	double E, nu;
	const int* row_ptr;
	const int* cols;
	const double* vals64;
	const float* vals32;
	const int* last_ci;
	const double* b;
	double* scratch;   // N doubles: per-node log10 E, then reductions
	double* partials;
	unsigned* ticket;
	double* rms;       // (Dinv b) root-mean-square
	bf16* f;           // N x FIN
};

__device__ __forceinline__ void diag_block(const FeatArgs& a, int r, double& k00, double& k01, double& k11) {
	k00 = k11 = 1.0;
	k01 = 0.0;
	for (int k = a.row_ptr[r]; k < a.row_ptr[r + 1]; k++)
		if (a.cols[k] == r) {
			k00 = a.vals64 ? a.vals64[4l * k] : (double) a.vals32[4l * k];
			k01 = a.vals64 ? a.vals64[4l * k + 1] : (double) a.vals32[4l * k + 1];
			k11 = a.vals64 ? a.vals64[4l * k + 3] : (double) a.vals32[4l * k + 3];
		}
}

// per node: mean log10 E of the incident elements; RMS of Dinv b.  The
// features end up in BF16, so they are computed in FP32 (FP64 is scarce on
// GB300); the per-node means are stored exactly so that equal materials give
// exactly zero contrasts.
__global__ void k_feat1(FeatArgs a) {
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		float s = 0.f;
		int const s0 = a.inc_ptr[i], s1 = a.inc_ptr[i + 1];
		for (int t = s0; t < s1; t++) s += log10f((float) (a.elemE ? a.elemE[a.inc[t]] : a.E));
		a.scratch[i] = s1 > s0 ? (double) (s / (float) (s1 - s0)) : (double) log10f((float) a.E);
		double k00, k01, k11;
		diag_block(a, i, k00, k01, k11);
		double2 const bb = ld2(a.b, i);
		float const z0 = k00 != 0.0 ? (float) bb.x / (float) k00 : 0.f, z1 = k11 != 0.0 ? (float) bb.y / (float) k11 : 0.f;
		v[0] += (double) (z0 * z0 + z1 * z1);
	}
	double out[1];
	if (grid_sum<1>(v, a.partials, a.ticket, out) && threadIdx.x == 0) a.rms[0] = sqrt(out[0] / (2.0 * (a.N > 0 ? a.N : 1)));
}

__global__ void k_feat2(FeatArgs a) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.N) return;
	float f[FIN];
	for (int k = 0; k < FIN; k++) f[k] = 0.f;
	int const r0 = a.row_ptr[i], r1 = a.row_ptr[i + 1];
	float nb = 0.f;
	for (int k = r0; k < r1; k++) nb += (float) a.scratch[a.cols[k]];
	nb /= (float) (r1 - r0);
	float nu = 0.f, lmin = 0.f, lmax = 0.f;
	int const s0 = a.inc_ptr[i], s1 = a.inc_ptr[i + 1];
	for (int t = s0; t < s1; t++) {
		nu += (float) (a.elemNu ? a.elemNu[a.inc[t]] : a.nu);
		float const le = log10f((float) (a.elemE ? a.elemE[a.inc[t]] : a.E));
		lmin = t == s0 ? le : fminf(lmin, le);
		lmax = t == s0 ? le : fmaxf(lmax, le);
	}
	nu = s1 > s0 ? nu / (float) (s1 - s0) : (float) a.nu;
	double k00d, k01d, k11d;
	diag_block(a, i, k00d, k01d, k11d);
	float const k00 = (float) k00d, k01 = (float) k01d, k11 = (float) k11d;
	double2 const bb = ld2(a.b, i);
	float const rms = a.rms[0] > 0.0 ? (float) a.rms[0] : 1.f;
	float const z0 = (k00 != 0.f ? (float) bb.x / k00 : 0.f) / rms, z1 = (k11 != 0.f ? (float) bb.y / k11 : 0.f) / rms;
	f[0] = (float) a.scratch[i] - nb;
	f[1] = (nu - 0.3f) * 10.f;
	f[2] = a.last_ci[2 * i] >= 0 ? 1.f : 0.f;
	f[3] = a.last_ci[2 * i + 1] >= 0 ? 1.f : 0.f;
	f[4] = (float) (r1 - r0) / 9.f;
	f[5] = z0;
	f[6] = z1;
	f[7] = (k00 > 0.f && k11 > 0.f) ? log10f(k00 / k11) : 0.f;
	f[8] = (k00 > 0.f && k11 > 0.f) ? k01 / sqrtf(k00 * k11) : 0.f;
	f[9] = fabsf(z0) + fabsf(z1);
	f[10] = lmin - lmax;
	for (int k = 0; k < FIN; k++) a.f[(long) i * FIN + k] = __float2bfloat16(f[k]);
}

// ---------------------------------------------------------------- forward

// Y = relu(W [X0 | X1] + b): X0, X1 are N x 64 (or X0 alone N x 16), Y N x 64
// BF16.  Persistent blocks: the weight tile is staged in shared memory once,
// then the block walks 64-node tiles; activations move in 16-byte vectors.
template <int K>
__global__ void __launch_bounds__(MT) k_dense_fwd(int N, const bf16* __restrict__ x0, const bf16* __restrict__ x1,
                                                  const bf16* __restrict__ w, const float* __restrict__ bias,
                                                  bf16* __restrict__ y) {
	__shared__ __align__(16) bf16 xs[TILE][K + 8];
	__shared__ __align__(16) bf16 ws[HID][K + 8];
	constexpr int CH = K / 8;  // 16-byte chunks per row
	for (int e = threadIdx.x; e < HID * CH; e += MT) {
		int const n = e / CH, c = e % CH;
		*reinterpret_cast<uint4*>(&ws[n][8 * c]) = reinterpret_cast<const uint4*>(w)[e];
	}
	int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	int const tiles = (N + TILE - 1) / TILE;
	for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
		int const node0 = tile * TILE;
		__syncthreads();  // the previous tile's reads of xs are done (and ws is staged)
		for (int e = threadIdx.x; e < TILE * CH; e += MT) {
			int const n = e / CH, c = e % CH, node = node0 + n;
			uint4 v = make_uint4(0u, 0u, 0u, 0u);
			if (node < N) {
				if (K == FIN) v = reinterpret_cast<const uint4*>(x0 + (long) node * FIN)[c];
				else v = c < HID / 8 ? reinterpret_cast<const uint4*>(x0 + (long) node * HID)[c]
				                     : reinterpret_cast<const uint4*>(x1 + (long) node * HID)[c - HID / 8];
			}
			*reinterpret_cast<uint4*>(&xs[n][8 * c]) = v;
		}
		__syncthreads();
		float acc[8][4] = {};
		auto at_a = [&](int m, int k) { return xs[warp * 16 + m][k]; };
		auto at_b = [&](int k, int n) { return ws[n][k]; };  // B(k, n) = W[n][k]
		warp_gemm<8>(acc, K, at_a, at_b);
#pragma unroll
		for (int j = 0; j < 8; j++) {
			int const n = 8 * j + 2 * t;
#pragma unroll
			for (int h = 0; h < 2; h++) {
				int const node = node0 + warp * 16 + g + 8 * h;
				if (node >= N) continue;
				float const v0 = fmaxf(acc[j][2 * h] + bias[n], 0.f), v1 = fmaxf(acc[j][2 * h + 1] + bias[n + 1], 0.f);
				*reinterpret_cast<uint32_t*>(y + (long) node * HID + n) = pack2(__float2bfloat16(v0), __float2bfloat16(v1));
			}
		}
	}
}

// m_i = mean of h over the node's graph row (itself included); one thread
// per node and 8-channel chunk, 16-byte loads
__global__ void k_agg(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols, const bf16* __restrict__ h,
                      bf16* __restrict__ m) {
	constexpr int CH = HID / 8;
	long const e = blockIdx.x * (long) blockDim.x + threadIdx.x;
	int const i = (int) (e / CH), c = (int) (e % CH);
	if (i >= N) return;
	float s[8] = {};
	int const r0 = row_ptr[i], r1 = row_ptr[i + 1];
	for (int k = r0; k < r1; k++) {
		uint4 const v = reinterpret_cast<const uint4*>(h + (long) cols[k] * HID)[c];
		uint32_t const u[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
		for (int q = 0; q < 4; q++) {
			s[2 * q] += __uint_as_float(u[q] << 16);
			s[2 * q + 1] += __uint_as_float(u[q] & 0xFFFF0000u);
		}
	}
	float const d = (float) (r1 - r0);  // a correctly rounded quotient, as the mean is defined
	uint4 o;
	o.x = pack2(__float2bfloat16(s[0] / d), __float2bfloat16(s[1] / d));
	o.y = pack2(__float2bfloat16(s[2] / d), __float2bfloat16(s[3] / d));
	o.z = pack2(__float2bfloat16(s[4] / d), __float2bfloat16(s[5] / d));
	o.w = pack2(__float2bfloat16(s[6] / d), __float2bfloat16(s[7] / d));
	reinterpret_cast<uint4*>(m + (long) i * HID)[c] = o;
}

// o = Wo h3 + bo, c = 0.45 tanh(o); the preconditioner blocks from c:
//     B = Kd^-1 + L C L^T,  L L^T = Kd^-1 (Cholesky),  C = [[c0, c1], [c1, c2]],
// Kd the node's 2x2 diagonal block.  L = [[sqrt(k11/det), 0],
// [-k01/sqrt(det k11), 1/sqrt(k11)]].  B = L (I + C) L^T is SPD for
// |c| <= 0.45, and at c = 0 it is block Jacobi (the inverse computed as the
// assembly epilogue does).  A non-SPD diagonal block gives B = 0 (the solve
// then breaks down and falls back to Jacobi).
__global__ void k_head(int N, const bf16* __restrict__ h3, const float* __restrict__ theta, float* __restrict__ o,
                       const int* __restrict__ row_ptr, const int* __restrict__ cols, const double* __restrict__ vals64,
                       const float* __restrict__ vals32, double* __restrict__ blocks, double* __restrict__ lfac) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	float oo[3];
	for (int q = 0; q < 3; q++) {
		float s = theta[O_BO + q];
		for (int k = 0; k < HID; k++) s += theta[O_WO + q * HID + k] * __bfloat162float(h3[(long) i * HID + k]);
		oo[q] = s;
		if (o) o[3 * i + q] = s;
	}
	double k00 = 0.0, k01 = 0.0, k10 = 0.0, k11 = 0.0;
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++)
		if (cols[k] == i) {
			k00 = vals64 ? vals64[4l * k] : (double) vals32[4l * k];
			k01 = vals64 ? vals64[4l * k + 1] : (double) vals32[4l * k + 1];
			k10 = vals64 ? vals64[4l * k + 2] : (double) vals32[4l * k + 2];
			k11 = vals64 ? vals64[4l * k + 3] : (double) vals32[4l * k + 3];
		}
	double const det = k00 * k11 - k01 * k10;
	bool const spd = det > 0.0 && k11 > 0.0;
	double const id = spd ? 1.0 / det : 0.0;
	double const m0 = k11 * id, m1 = -k01 * id, m3 = k00 * id;
	double const l00 = spd ? sqrt(k11 * id) : 0.0;
	double const l10 = spd ? -k01 / sqrt(det * k11) : 0.0;
	double const l11 = spd ? 1.0 / sqrt(k11) : 0.0;
	lfac[3 * i] = l00;
	lfac[3 * i + 1] = l10;
	lfac[3 * i + 2] = l11;
	double const c0 = C_SCALE * tanh((double) oo[0]), c1 = C_SCALE * tanh((double) oo[1]), c2 = C_SCALE * tanh((double) oo[2]);
	double const b01 = l00 * l10 * c0 + l00 * l11 * c1;
	blocks[4 * i + 0] = m0 + l00 * l00 * c0;
	blocks[4 * i + 1] = m1 + b01;
	blocks[4 * i + 2] = m1 + b01;
	blocks[4 * i + 3] = m3 + (l10 * l10 * c0 + 2.0 * l10 * l11 * c1 + l11 * l11 * c2);
}

// ---------------------------------------------------------------- loss
// Condition-number loss of the preconditioned operator B K.  With the
// generalized Rayleigh quotient R(x) = (x.Kx) / (x.B^-1 x), which lies in
// [lambda_min, lambda_max] of B K:
//     L = log R(v) - log R(e),
// v from power iterations on B K (approaching the top eigenvector; the
// caller keeps it between steps), e a solver error (smooth: dominated by the
// bottom of the spectrum).  Per node, with u = L_i^-1 x_i and
// w = (I + C_i)^-1 u: x_i.B_i^-1 x_i = u.w, and d(u.w)/dC = -w w^T.

struct LossArgs {
	int N;
	const int* row_ptr;
	const int* cols;
	const double* vals64;
	const double* blocks;
	const double* lfac;
	const float* o;
	const double* r;   // K e
	const double* e;
	const double* v;   // power vector
	double* partials;
	unsigned* ticket;
	double* sc;  // v.Kv, Q(v), e.Ke, Q(e), loss, v.v
	// SSOR context (the problem in colour-major order, B the relaxation
	// block inverses): M = (B^-1 + L) B (B^-1 + U) and
	//     Q(x) = x.M x = sum_i (x_i.B_i^-1 x_i + u_i.B_i u_i) + 2 x.L x,
	// u_i = sum over higher-colour neighbours A_ij x_j; with s = L_i^T u_i,
	// u_i.B_i u_i = s.(I + C_i) s and d/dC = s s^T.  Otherwise Q(x) = x.B^-1 x.
	int ssor;
};

// lower- and higher-colour parts of row i of A x (colour-major order: a
// column below i is a lower colour)
__device__ __forceinline__ void lu_parts(const LossArgs& a, const double* x, int i, double& l0, double& l1, double& u0,
                                         double& u1) {
	l0 = l1 = u0 = u1 = 0.0;
	for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; k++) {
		int const c = a.cols[k];
		if (c == i) continue;
		double2 const xv = ld2(x, c);
		const double* m = a.vals64 + 4l * k;
		double const y0 = m[0] * xv.x + m[1] * xv.y, y1 = m[2] * xv.x + m[3] * xv.y;
		if (c < i) {
			l0 += y0;
			l1 += y1;
		}
		else {
			u0 += y0;
			u1 += y1;
		}
	}
}

// s = L_i^T u and s.(I + C) s
__device__ __forceinline__ double b_quad(const double* lf, double c0, double c1, double c2, double u0, double u1, double& s0,
                                         double& s1) {
	s0 = lf[0] * u0 + lf[1] * u1;
	s1 = lf[2] * u1;
	return s0 * s0 + s1 * s1 + c0 * s0 * s0 + 2.0 * c1 * s0 * s1 + c2 * s1 * s1;
}

// x_i.B_i^-1 x_i and w = (I + C_i)^-1 L_i^-1 x_i
__device__ __forceinline__ double binv_quad(const double* lf, double c0, double c1, double c2, double x0, double x1,
                                            double& w0, double& w1) {
	double const l00 = lf[0], l10 = lf[1], l11 = lf[2];
	if (!(l00 > 0.0 && l11 > 0.0)) {
		w0 = w1 = 0.0;
		return 0.0;
	}
	double const u0 = x0 / l00, u1 = (x1 - l10 * u0) / l11;
	double const det = (1.0 + c0) * (1.0 + c2) - c1 * c1;
	w0 = ((1.0 + c2) * u0 - c1 * u1) / det;
	w1 = (-c1 * u0 + (1.0 + c0) * u1) / det;
	return u0 * w0 + u1 * w1;
}

__device__ __forceinline__ void node_c(const float* o, int i, double& c0, double& c1, double& c2) {
	c0 = C_SCALE * tanh((double) o[3 * i]);
	c1 = C_SCALE * tanh((double) o[3 * i + 1]);
	c2 = C_SCALE * tanh((double) o[3 * i + 2]);
}

// one power step: out = B (K in) (blocks == nullptr: out = K in)
__global__ void k_power(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols, const double* __restrict__ vals,
                        const double* __restrict__ blocks, const double* __restrict__ vin, double* __restrict__ vout) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N) return;
	double y0 = 0.0, y1 = 0.0;
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
		double2 const x = ld2(vin, cols[k]);
		const double* m = vals + 4l * k;
		y0 += m[0] * x.x + m[1] * x.y;
		y1 += m[2] * x.x + m[3] * x.y;
	}
	if (!blocks) {
		st2(vout, i, y0, y1);
		return;
	}
	const double* B = blocks + 4l * i;
	st2(vout, i, B[0] * y0 + B[1] * y1, B[2] * y0 + B[3] * y1);
}

// SSOR power step, after t = K v: forward sweep of colour range [lo, hi),
// v_i = B_i (t_i - sum_L A_ij v_j) (rows of one colour are independent)
__global__ void k_pssor_fwd(int lo, int hi, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                            const double* __restrict__ vals, const double* __restrict__ blocks, const double* __restrict__ t,
                            double* __restrict__ v) {
	int const i = lo + blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= hi) return;
	double s0 = t[2l * i], s1 = t[2l * i + 1];
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
		int const c = cols[k];
		if (c >= lo) break;
		const double* m = vals + 4l * k;
		s0 -= m[0] * v[2l * c] + m[1] * v[2l * c + 1];
		s1 -= m[2] * v[2l * c] + m[3] * v[2l * c + 1];
	}
	const double* B = blocks + 4l * i;
	v[2l * i] = B[0] * s0 + B[1] * s1;
	v[2l * i + 1] = B[2] * s0 + B[3] * s1;
}

// backward sweep of [lo, hi): v_i -= B_i sum_U A_ij v_j
__global__ void k_pssor_bwd(int lo, int hi, const int* __restrict__ row_ptr, const int* __restrict__ cols,
                            const double* __restrict__ vals, const double* __restrict__ blocks, double* __restrict__ v) {
	int const i = lo + blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= hi) return;
	double s0 = 0.0, s1 = 0.0;
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
		int const c = cols[k];
		if (c < hi) continue;
		const double* m = vals + 4l * k;
		s0 += m[0] * v[2l * c] + m[1] * v[2l * c + 1];
		s1 += m[2] * v[2l * c] + m[3] * v[2l * c + 1];
	}
	const double* B = blocks + 4l * i;
	v[2l * i] -= B[0] * s0 + B[1] * s1;
	v[2l * i + 1] -= B[2] * s0 + B[3] * s1;
}

// v.v into sc[5]; then v /= |v| (the loss and its gradient do not depend on v's scale)
__global__ void k_vnorm(int N, const double* __restrict__ v, double* partials, unsigned* ticket, double* sc) {
	double t[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
		double2 const x = ld2(v, i);
		t[0] += x.x * x.x + x.y * x.y;
	}
	double out[1];
	if (grid_sum<1>(t, partials, ticket, out) && threadIdx.x == 0) sc[5] = out[0];
}

__global__ void k_vscale(int N, double* __restrict__ v, const double* __restrict__ sc) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= N || !(sc[5] > 0.0)) return;
	double const f = 1.0 / sqrt(sc[5]);
	double2 const x = ld2(v, i);
	st2(v, i, x.x * f, x.y * f);
}

__global__ void k_loss_terms(LossArgs a) {
	double v[4] = {0.0, 0.0, 0.0, 0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += gridDim.x * blockDim.x) {
		double y0 = 0.0, y1 = 0.0;
		for (int k = a.row_ptr[i]; k < a.row_ptr[i + 1]; k++) {
			double2 const x = ld2(a.v, a.cols[k]);
			const double* m = a.vals64 + 4l * k;
			y0 += m[0] * x.x + m[1] * x.y;
			y1 += m[2] * x.x + m[3] * x.y;
		}
		double c0, c1, c2, w0, w1;
		node_c(a.o, i, c0, c1, c2);
		double2 const vv = ld2(a.v, i), ee = ld2(a.e, i), rr = ld2(a.r, i);
		v[0] += vv.x * y0 + vv.y * y1;
		v[1] += binv_quad(a.lfac + 3l * i, c0, c1, c2, vv.x, vv.y, w0, w1);
		v[2] += ee.x * rr.x + ee.y * rr.y;
		v[3] += binv_quad(a.lfac + 3l * i, c0, c1, c2, ee.x, ee.y, w0, w1);
		if (a.ssor) {
			double l0, l1, u0, u1, s0, s1;
			lu_parts(a, a.v, i, l0, l1, u0, u1);
			v[1] += b_quad(a.lfac + 3l * i, c0, c1, c2, u0, u1, s0, s1) + 2.0 * (vv.x * l0 + vv.y * l1);
			lu_parts(a, a.e, i, l0, l1, u0, u1);
			v[3] += b_quad(a.lfac + 3l * i, c0, c1, c2, u0, u1, s0, s1) + 2.0 * (ee.x * l0 + ee.y * l1);
		}
	}
	double out[4];
	if (grid_sum<4>(v, a.partials, a.ticket, out) && threadIdx.x == 0) {
		for (int k = 0; k < 4; k++) a.sc[k] = out[k];
		a.sc[4] = log(out[0]) - log(out[1]) - log(out[2]) + log(out[3]);
	}
}

// dL/dc = (w_v w_v^T) / Q_v - (w_e w_e^T) / Q_e as (c0, c1, c2) -> dL/do (N x 3, FP32)
__global__ void k_loss_back(LossArgs a, float* __restrict__ d_o) {
	int const i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= a.N) return;
	double const qv = a.sc[1], qe = a.sc[3];
	double c0, c1, c2, a0, a1, b0, b1;
	node_c(a.o, i, c0, c1, c2);
	double2 const vv = ld2(a.v, i), ee = ld2(a.e, i);
	binv_quad(a.lfac + 3l * i, c0, c1, c2, vv.x, vv.y, a0, a1);
	binv_quad(a.lfac + 3l * i, c0, c1, c2, ee.x, ee.y, b0, b1);
	double dc0 = a0 * a0 / qv - b0 * b0 / qe;
	double dc1 = 2.0 * (a0 * a1 / qv - b0 * b1 / qe);
	double dc2 = a1 * a1 / qv - b1 * b1 / qe;
	if (a.ssor) {
		// dQ/dC of the u.B u terms is + s s^T, so they enter with the opposite sign
		double l0, l1, u0, u1, p0, p1, q0, q1;
		lu_parts(a, a.v, i, l0, l1, u0, u1);
		b_quad(a.lfac + 3l * i, c0, c1, c2, u0, u1, p0, p1);
		lu_parts(a, a.e, i, l0, l1, u0, u1);
		b_quad(a.lfac + 3l * i, c0, c1, c2, u0, u1, q0, q1);
		dc0 += -p0 * p0 / qv + q0 * q0 / qe;
		dc1 += 2.0 * (-p0 * p1 / qv + q0 * q1 / qe);
		dc2 += -p1 * p1 / qv + q1 * q1 / qe;
	}
	double const t0 = c0 / C_SCALE, t1 = c1 / C_SCALE, t2 = c2 / C_SCALE;
	d_o[3 * i + 0] = (float) (dc0 * C_SCALE * (1.0 - t0 * t0));
	d_o[3 * i + 1] = (float) (dc1 * C_SCALE * (1.0 - t1 * t1));
	d_o[3 * i + 2] = (float) (dc2 * C_SCALE * (1.0 - t2 * t2));
}

// ---------------------------------------------------------------- backward

// head: dh3 = do Wo (FP32 N x 64); per-block partial sums of dWo = do^T h3
// and dbo (thread t < 195 owns one output, nodes summed in ascending order)
constexpr int HEAD_TPB = 256, HEAD_NODES = 256, HEAD_OUT = 3 * HID + 3;
__global__ void __launch_bounds__(HEAD_TPB) k_head_back(int N, const float* __restrict__ d_o, const bf16* __restrict__ h3,
                                                        const float* __restrict__ theta, float* __restrict__ dh,
                                                        double* __restrict__ part) {
	int const i0 = blockIdx.x * HEAD_NODES, i1 = min(N, i0 + HEAD_NODES);
	for (int e = threadIdx.x; e < (i1 - i0) * HID; e += HEAD_TPB) {
		int const i = i0 + e / HID, k = e % HID;
		dh[(long) i * HID + k] = d_o[3 * i] * theta[O_WO + k] + d_o[3 * i + 1] * theta[O_WO + HID + k] +
		                         d_o[3 * i + 2] * theta[O_WO + 2 * HID + k];
	}
	int const t = threadIdx.x;
	if (t < HEAD_OUT) {
		double acc = 0.0;
		if (t < 3 * HID) {
			int const q = t / HID, k = t % HID;
			for (int i = i0; i < i1; i++) acc += (double) d_o[3 * i + q] * (double) __bfloat162float(h3[(long) i * HID + k]);
		}
		else {
			for (int i = i0; i < i1; i++) acc += (double) d_o[3 * i + t - 3 * HID];
		}
		part[(long) blockIdx.x * HEAD_OUT + t] = acc;
	}
}

// dpre = dh * (h > 0), as BF16 (the tensor-core operand)
__global__ void k_relu_back(long n, const float* __restrict__ dh, const bf16* __restrict__ h, bf16* __restrict__ dpre) {
	for (long e = blockIdx.x * (long) blockDim.x + threadIdx.x; e < n; e += (long) gridDim.x * blockDim.x)
		dpre[e] = __float2bfloat16(__bfloat162float(h[e]) > 0.f ? dh[e] : 0.f);
}

// dX (N x 128, FP32) = dpre (N x 64) W (64 x 128)
__global__ void __launch_bounds__(MT) k_dense_dx(int N, const bf16* __restrict__ dpre, const bf16* __restrict__ w,
                                                 float* __restrict__ dx) {
	__shared__ bf16 ps[TILE][HID + 8];
	__shared__ bf16 ws[HID][HK + 8];
	int const node0 = blockIdx.x * TILE;
	for (int e = threadIdx.x; e < TILE * HID; e += MT) {
		int const n = e / HID, k = e % HID, node = node0 + n;
		ps[n][k] = node < N ? dpre[(long) node * HID + k] : __float2bfloat16(0.f);
	}
	for (int e = threadIdx.x; e < HID * HK; e += MT) ws[e / HK][e % HK] = w[e];
	__syncthreads();
	int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	float acc[16][4] = {};
	auto at_a = [&](int m, int k) { return ps[warp * 16 + m][k]; };
	auto at_b = [&](int k, int n) { return ws[k][n]; };  // B(k=out, n=in) = W[out][in]
	warp_gemm<16>(acc, HID, at_a, at_b);
#pragma unroll
	for (int j = 0; j < 16; j++) {
		int const n = 8 * j + 2 * t;
#pragma unroll
		for (int h = 0; h < 2; h++) {
			int const node = node0 + warp * 16 + g + 8 * h;
			if (node >= N) continue;
			dx[(long) node * HK + n] = acc[j][2 * h];
			dx[(long) node * HK + n + 1] = acc[j][2 * h + 1];
		}
	}
}

// Partial weight gradient of one block of nodes: dW (64 x K) = dpre^T [X0 | X1],
// plus the bias gradient column sums, on the tensor cores.
template <int K>
__global__ void __launch_bounds__(MT) k_dense_dw(int N, const bf16* __restrict__ dpre, const bf16* __restrict__ x0,
                                                 const bf16* __restrict__ x1, double* __restrict__ part) {
	__shared__ bf16 ps[TILE][HID + 8];
	__shared__ bf16 xs[TILE][K + 8];
	int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	constexpr int NT = K / 8;
	float acc[NT][4] = {};
	float bsum = 0.f;
	int const c0 = blockIdx.x * DW_CHUNK, c1 = min(N, c0 + DW_CHUNK);
	for (int node0 = c0; node0 < c1; node0 += TILE) {
		__syncthreads();
		for (int e = threadIdx.x; e < TILE * HID; e += MT) {
			int const n = e / HID, k = e % HID, node = node0 + n;
			ps[n][k] = node < c1 ? dpre[(long) node * HID + k] : __float2bfloat16(0.f);
		}
		for (int e = threadIdx.x; e < TILE * K; e += MT) {
			int const n = e / K, k = e % K, node = node0 + n;
			bf16 v = __float2bfloat16(0.f);
			if (node < c1) v = K == FIN ? x0[(long) node * FIN + k] : (k < HID ? x0[(long) node * HID + k] : x1[(long) node * HID + k - HID]);
			xs[n][k] = v;
		}
		__syncthreads();
		auto at_a = [&](int m, int k) { return ps[k][warp * 16 + m]; };  // A(m=out, k=node)
		auto at_b = [&](int k, int n) { return xs[k][n]; };              // B(k=node, n=in)
		warp_gemm<NT>(acc, TILE, at_a, at_b);
		if (threadIdx.x < HID)
			for (int n = 0; n < TILE; n++) bsum += __bfloat162float(ps[n][threadIdx.x]);
	}
	double* out = part + (long) blockIdx.x * (HID * K + HID);
#pragma unroll
	for (int j = 0; j < NT; j++) {
		int const n = 8 * j + 2 * t;
#pragma unroll
		for (int h = 0; h < 2; h++) {
			int const m = warp * 16 + g + 8 * h;
			out[m * K + n] = acc[j][2 * h];
			out[m * K + n + 1] = acc[j][2 * h + 1];
		}
	}
	if (threadIdx.x < HID) out[HID * K + threadIdx.x] = bsum;
}

// grad[off + k] = sum over blocks of part[blk][k], in block order
__global__ void k_reduce_parts(const double* __restrict__ part, int nblk, int len, float* __restrict__ grad, int off_w,
                               int n_w, int off_b) {
	int const k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= len) return;
	double s = 0.0;
	for (int b = 0; b < nblk; b++) s += part[(long) b * len + k];
	if (k < n_w) grad[off_w + k] = (float) s;
	else grad[off_b + k - n_w] = (float) s;
}

// dh_prev = dX[:, :64] + sum over the node's row of dX[j, 64:] / deg_j  (adjoint of the mean)
__global__ void k_agg_back(int N, const int* __restrict__ row_ptr, const int* __restrict__ cols, const float* __restrict__ dx,
                           float* __restrict__ dh) {
	int const i = blockIdx.x * (blockDim.x / HID) + threadIdx.x / HID, c = threadIdx.x % HID;
	if (i >= N) return;
	float s = dx[(long) i * HK + c];
	for (int k = row_ptr[i]; k < row_ptr[i + 1]; k++) {
		int const j = cols[k];
		s += dx[(long) j * HK + HID + c] / (float) (row_ptr[j + 1] - row_ptr[j]);
	}
	dh[(long) i * HID + c] = s;
}

__global__ void k_adam(int n, float* theta, const float* g, float* m, float* v, bf16* wb, float lr, float b1t, float b2t) {
	int const k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) return;
	float const gk = g[k];
	float const mk = 0.9f * m[k] + 0.1f * gk;
	float const vk = 0.999f * v[k] + 0.001f * gk * gk;
	m[k] = mk;
	v[k] = vk;
	float const th = theta[k] - lr * (mk / (1.f - b1t)) / (sqrtf(vk / (1.f - b2t)) + 1e-8f);
	theta[k] = th;
	wb[k] = __float2bfloat16(th);
}

__global__ void k_to_bf16(int n, const float* theta, bf16* wb) {
	int const k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k < n) wb[k] = __float2bfloat16(theta[k]);
}


// ---------------------------------------------------------------- tcgen05 forward layer
//
// y = relu(x W^T + bias) for a 128-node tile per MMA, on the fifth-generation
// tensor cores: the x tile (128 x K BF16) and W (64 x K BF16) are staged in
// shared memory in the canonical K-major layout without swizzle (core
// matrices of 8 rows x 16 bytes: element (m, k) of a 16-wide K-slice s at
// s * slice_bytes + (m / 8) * 256 + ((k % 16) / 8) * 128 + (m % 8) * 16 +
// (k % 8) * 2, so core matrices adjacent along K are 128 bytes apart and along
// M (or N) 256 bytes); one elected thread issues K / 16 tcgen05.mma
// (kind::f16, M = 128, N = 64, BF16 in, FP32 accumulator in 64 TMEM columns)
// and commits them to an mbarrier; after a bounded wait each warp reads its 32
// TMEM lanes (rows) with tcgen05.ld and applies bias and ReLU.  A wait that
// runs out sets *err and the block stops issuing MMAs; TMEM is freed on every
// path.
constexpr int TC_M = 128;               // nodes per tile (the MMA's M)
constexpr int TC_T = 128;               // threads: warp w reads TMEM lanes 32w .. 32w + 31
constexpr long TC_POLLS = 1l << 24;     // mbarrier polls before a wait gives up

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t) __cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices along K), stride byte offset (along M or N),
// all in 16-byte units; descriptor version 1 (bits 46-47); no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
	return (uint64_t) ((addr >> 4) & 0x3FFFu) | ((uint64_t) ((lbo >> 4) & 0x3FFFu) << 16) |
	       ((uint64_t) ((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 and 10-12 = 1), both K-major, N / 8 at bit 17, M / 16 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ bool tc_mbar_try(uint32_t bar, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok)
	             : "r"(bar), "r"(parity)
	             : "memory");
	return ok != 0;
}

// 16 consecutive accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
	    "[%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr)
	    : "memory");
}

constexpr size_t tc_smem_bytes(int K) { return (size_t) (2 * TC_M + HID) * K * sizeof(bf16); }

// one 16-byte piece of a node's input row into the tile's layout by cp.async
// (zero-filled past the last node), chunk q of row m
template <int K>
__device__ __forceinline__ void tc_fetch(unsigned char* xs, int N, int node0, const bf16* x0, const bf16* x1, int e) {
	constexpr int CH = K / 8;
	int const m = e / CH, q = e % CH, node = node0 + m;
	const void* src = x0;
	int bytes = 0;
	if (node < N) {
		bytes = 16;
		if (K == FIN) src = reinterpret_cast<const uint4*>(x0 + (long) node * FIN) + q;
		else src = q < HID / 8 ? reinterpret_cast<const uint4*>(x0 + (long) node * HID) + q
		                       : reinterpret_cast<const uint4*>(x1 + (long) node * HID) + (q - HID / 8);
	}
	uint32_t const dst = tc_smem(xs + (q >> 1) * (TC_M * 32) + (m >> 3) * 256 + (q & 1) * 128 + (m & 7) * 16);
	asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}

template <int K>
__global__ void __launch_bounds__(TC_T) k_dense_fwd_tc(int N, const bf16* __restrict__ x0, const bf16* __restrict__ x1,
                                                       const bf16* __restrict__ w, const float* __restrict__ bias,
                                                       bf16* __restrict__ y, int* err) {
	extern __shared__ __align__(1024) unsigned char tc_sm[];
	constexpr int NS = K / 16;   // MMA K-slices
	constexpr int CH = K / 8;    // 16-byte chunks per row
	constexpr int XB = TC_M * K * 2;  // bytes of one x tile
	unsigned char* const ws = tc_sm + 2 * XB;  // W, slice s at s * HID * 32 bytes; two x tiles before it
	__shared__ __align__(8) unsigned long long mbar;
	__shared__ uint32_t tmem_slot;
	__shared__ int s_ok;
	__shared__ float bs[HID];
	int const tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	int const tiles = (N + TC_M - 1) / TC_M;
	// the first tile in flight while W is staged
	if ((int) blockIdx.x < tiles)
		for (int e = tid; e < TC_M * CH; e += TC_T) tc_fetch<K>(tc_sm, N, blockIdx.x * TC_M, x0, x1, e);
	asm volatile("cp.async.commit_group;" ::: "memory");
	for (int e = tid; e < HID * CH; e += TC_T) {
		int const n = e / CH, q = e % CH;
		uint4 const v = reinterpret_cast<const uint4*>(w)[e];  // row n of W, features 8q .. 8q + 7
		*reinterpret_cast<uint4*>(ws + (q >> 1) * (HID * 32) + (n >> 3) * 256 + (q & 1) * 128 + (n & 7) * 16) = v;
	}
	if (tid < HID) bs[tid] = bias[tid];
	if (warp == 0) {
		asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_slot)), "r"(HID)
		             : "memory");
		asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
	}
	if (tid == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mbar)) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		s_ok = 1;
	}
	uint32_t phase = 0;
	int buf = 0;
	uint32_t const bar = tc_smem(&mbar);
	for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, buf ^= 1) {
		int const node0 = tile * TC_M;
		unsigned char* const xs = tc_sm + buf * XB;
		// this tile's copies landed; the generic-proxy writes (W, the copies)
		// before the tensor cores' (async-proxy) reads
		asm volatile("cp.async.wait_all;" ::: "memory");
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
		__syncthreads();
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		uint32_t const tmem = tmem_slot;
		if (s_ok == 0) break;  // the same in every thread: a wait ran out
		if (tid == 0) {
#pragma unroll
			for (int sl = 0; sl < NS; sl++) {
				uint64_t const ad = tc_desc(tc_smem(xs) + sl * TC_M * 32, 128, 256);
				uint64_t const bd = tc_desc(tc_smem(ws) + sl * HID * 32, 128, 256);
				asm volatile(
				    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
				    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
				    "l"(ad), "l"(bd), "r"(tc_idesc(TC_M, HID)), "r"(sl > 0 ? 1 : 0)
				    : "memory");
			}
			asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
			             : "memory");
		}
		// the next tile's copies into the other buffer (its last reader, the
		// previous tile's MMAs, has completed), in flight during this epilogue
		int const next = tile + gridDim.x;
		if (next < tiles)
			for (int e = tid; e < TC_M * CH; e += TC_T) tc_fetch<K>(tc_sm + (buf ^ 1) * XB, N, next * TC_M, x0, x1, e);
		asm volatile("cp.async.commit_group;" ::: "memory");
		bool got = false;
		for (long it = 0; it < TC_POLLS; it++)
			if (tc_mbar_try(bar, phase)) {
				got = true;
				break;
			}
		if (got) phase ^= 1u;  // else the drain below waits for this completion
		else {
			atomicExch(err, 1);
			s_ok = 0;
		}
		asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
		int const node = node0 + warp * 32 + lane;
		uint32_t const taddr = tmem + ((uint32_t) (warp * 32) << 16);
#pragma unroll
		for (int c0 = 0; c0 < HID; c0 += 16) {
			uint32_t r[16];
			tc_ld16(taddr + c0, r);
			asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
			if (got && node < N) {
				uint32_t pk[8];
#pragma unroll
				for (int j = 0; j < 8; j++) {
					float const v0 = fmaxf(__uint_as_float(r[2 * j]) + bs[c0 + 2 * j], 0.f);
					float const v1 = fmaxf(__uint_as_float(r[2 * j + 1]) + bs[c0 + 2 * j + 1], 0.f);
					pk[j] = pack2(__float2bfloat16(v0), __float2bfloat16(v1));
				}
				uint4* dst = reinterpret_cast<uint4*>(y + (long) node * HID + c0);
				dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
				dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
			}
		}
		asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	}
	// copies still in flight land before the block exits; a wait that ran out
	// gets one more bounded wait for the MMAs in flight; then TMEM is freed
	asm volatile("cp.async.wait_all;" ::: "memory");
	if (!s_ok) {
		for (long it = 0; it < TC_POLLS; it++)
			if (tc_mbar_try(bar, phase)) break;
	}
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
	__syncthreads();
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
	if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot), "r"(HID) : "memory");
}

inline int nb(long n, int t = 256) { return (int) ((n + t - 1) / t) > 0 ? (int) ((n + t - 1) / t) : 1; }

}  // namespace

// ====================================================================== host side

struct bfm_gpu_mpnn {
	MpnnDev d;
	int step;
	// activations of the problem last seen
	long cap_n;
	bf16 *f, *h[4], *m[3], *dpre;
	float *o, *d_o, *dh, *dx;
	double *blocks, *lfac, *z, *az, *sc, *partials, *rms, *scratch;
	unsigned* ticket;
	int* tc_err;   // set by a tcgen05 layer whose completion wait ran out
};

namespace {

// blocks of the persistent dense kernels: six per SM
int persistent_grid() {
	static int g = 0;
	if (!g) {
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		g = 6 * (sms > 0 ? sms : 1);
	}
	return g;
}

// the forward dense layers run on tcgen05 unless BFM_GPU_MPNN_GEMM=mma asks
// for the warp-level mma.sync kernels (read at each forward)
bool tc_layers() {
	char const* e = getenv("BFM_GPU_MPNN_GEMM");
	return !(e && strcmp(e, "mma") == 0);
}

// blocks of the tcgen05 layers: two per SM (80 KB of shared memory and 64
// TMEM columns each at K = 128); the shared-memory attribute is set once
int tc_grid() {
	static int g = 0;
	if (!g) {
		int dev = 0, sms = 0;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		cudaFuncSetAttribute(k_dense_fwd_tc<FIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) tc_smem_bytes(FIN));
		cudaFuncSetAttribute(k_dense_fwd_tc<HK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) tc_smem_bytes(HK));
		g = 2 * (sms > 0 ? sms : 1);
	}
	return g;
}

void free_acts(bfm_gpu_mpnn* net) {
	void* p[] = {net->f, net->h[0], net->h[1], net->h[2], net->h[3], net->m[0], net->m[1], net->m[2], net->dpre, net->o,
	             net->d_o, net->dh, net->dx, net->blocks, net->lfac, net->z, net->az, net->scratch};
	for (void* q : p)
		if (q) cudaFree(q);
	net->f = net->dpre = nullptr;
	for (auto& q : net->h) q = nullptr;
	for (auto& q : net->m) q = nullptr;
	net->o = net->d_o = net->dh = net->dx = nullptr;
	net->blocks = net->lfac = net->z = net->az = net->scratch = nullptr;
	net->cap_n = 0;
}

template <typename T>
int alloc(T** p, long n) {
	*p = nullptr;
	cudaError_t const e = cudaMalloc((void**) p, (n > 0 ? n : 1) * sizeof(T));
	if (e != cudaSuccess) return mfail("cudaMalloc of %ld bytes failed: %s", n * (long) sizeof(T), cudaGetErrorString(e));
	return 0;
}

int ensure_acts(bfm_gpu_mpnn* net, long N) {
	if (N <= net->cap_n) return 0;
	free_acts(net);
	long const n = N > 0 ? N : 1;
	if (alloc(&net->f, n * FIN)) return -1;
	for (auto& q : net->h)
		if (alloc(&q, n * HID)) return -1;
	for (auto& q : net->m)
		if (alloc(&q, n * HID)) return -1;
	if (alloc(&net->dpre, n * HID) || alloc(&net->o, n * 3) || alloc(&net->d_o, n * 3) || alloc(&net->dh, n * HID) ||
	    alloc(&net->dx, n * HK) || alloc(&net->blocks, n * 4) || alloc(&net->lfac, n * 3) || alloc(&net->z, n * 2) ||
	    alloc(&net->az, n * 2) || alloc(&net->scratch, n))
		return -1;
	long const chunks = (n + DW_CHUNK - 1) / DW_CHUNK, heads = (n + HEAD_NODES - 1) / HEAD_NODES;
	long const need = chunks * (HID * HK + HID) > heads * HEAD_OUT ? chunks * (HID * HK + HID) : heads * HEAD_OUT;
	if (need > net->d.gpart_cap) {
		if (net->d.gpart) cudaFree(net->d.gpart);
		net->d.gpart = nullptr;
		if (alloc(&net->d.gpart, need)) return -1;
		net->d.gpart_cap = need;
	}
	net->cap_n = N;
	return 0;
}

// features and forward pass on the problem's stream; blocks and scales of every node
int forward(bfm_gpu_mpnn* net, bfm_gpu_problem_t* P, cudaStream_t st) {
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	bfmi_mesh_t ms;
	bfmi_mesh(P, &ms);
	if (!bf.assembled) return mfail("assemble the problem before running the network");
	int const N = bf.N;
	if (ensure_acts(net, N)) return -1;
	FeatArgs fa;
	memset(&fa, 0, sizeof fa);
	fa.N = N;
	fa.kind = bf.kind;
	fa.inc_ptr = ms.inc_ptr;
	fa.inc = ms.inc;
	fa.elemE = ms.elemE;
	fa.elemNu = ms.elemNu;
	fa.E = ms.E;
	fa.nu = ms.nu;
	fa.row_ptr = bf.row_ptr;
	fa.cols = bf.cols;
	fa.vals64 = bf.vals64_any;
	fa.vals32 = bf.vals32;
	fa.last_ci = ms.last_ci;
	fa.b = bf.b;
	fa.scratch = net->scratch;
	fa.partials = net->partials;
	fa.ticket = net->ticket;
	fa.rms = net->rms;
	fa.f = net->f;
	k_feat1<<<FEAT_GRID, TPB_K, 0, st>>>(fa);
	k_feat2<<<nb(N), 256, 0, st>>>(fa);
	if (tc_layers()) {
		// the dense layers on the tcgen05 tensor cores (128-node tiles)
		int const tiles = (N + TC_M - 1) / TC_M > 0 ? (N + TC_M - 1) / TC_M : 1;
		int const g = tiles < tc_grid() ? tiles : tc_grid();
		k_dense_fwd_tc<FIN><<<g, TC_T, tc_smem_bytes(FIN), st>>>(N, net->f, nullptr, net->d.wb + O_W0,
		                                                           net->d.theta + O_B0, net->h[0], net->tc_err);
		for (int l = 1; l <= 3; l++) {
			k_agg<<<nb((long) N * (HID / 8)), 256, 0, st>>>(N, bf.row_ptr, bf.cols, net->h[l - 1], net->m[l - 1]);
			k_dense_fwd_tc<HK><<<g, TC_T, tc_smem_bytes(HK), st>>>(N, net->h[l - 1], net->m[l - 1], net->d.wb + o_w(l),
			                                                          net->d.theta + o_b(l), net->h[l], net->tc_err);
		}
	}
	else {
		int const tiles = (N + TILE - 1) / TILE > 0 ? (N + TILE - 1) / TILE : 1;
		int const pgrid = tiles < persistent_grid() ? tiles : persistent_grid();
		k_dense_fwd<FIN><<<pgrid, MT, 0, st>>>(N, net->f, nullptr, net->d.wb + O_W0, net->d.theta + O_B0, net->h[0]);
		for (int l = 1; l <= 3; l++) {
			k_agg<<<nb((long) N * (HID / 8)), 256, 0, st>>>(N, bf.row_ptr, bf.cols, net->h[l - 1], net->m[l - 1]);
			k_dense_fwd<HK><<<pgrid, MT, 0, st>>>(N, net->h[l - 1], net->m[l - 1], net->d.wb + o_w(l),
			                                      net->d.theta + o_b(l), net->h[l]);
		}
	}
	k_head<<<nb(N), 256, 0, st>>>(N, net->h[3], net->d.theta, net->o, bf.row_ptr, bf.cols, bf.vals64_any, bf.vals32,
	                               net->blocks, net->lfac);
	MCK(cudaGetLastError());
	return 0;
}

// loss of the pair (r, e) and the gradient of every parameter into d.grad
int backward(bfm_gpu_mpnn* net, bfm_gpu_problem_t* P, const double* r, const double* e, double* v, int power_iters,
             cudaStream_t st) {
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	if (!bf.vals64_any) return mfail("training needs the FP64 operator: assemble in FP64, MIXED_EXACT or FP64_DF");
	int const N = bf.N;
	// the power vector: v <- B K v (SSOR context: v <- M^-1 K v, the sweeps
	// colour by colour in FP64), power_iters times, rescaled to unit length
	// every 16 steps and at the end
	bool const ssor = bf.ncol > 0 && (bf.precond == BFM_GPU_PC_SSOR || bf.precond == BFM_GPU_PC_LEARNED_SSOR);
	for (int k = 0; k < power_iters; k++) {
		if (ssor) {
			k_power<<<nb(N), 256, 0, st>>>(N, bf.row_ptr, bf.cols, bf.vals64_any, nullptr, v, net->z);
			for (int c = 0; c < bf.ncol; c++) {
				int const lo = bf.col_off[c], hi = bf.col_off[c + 1];
				if (hi > lo)
					k_pssor_fwd<<<nb(hi - lo), 256, 0, st>>>(lo, hi, bf.row_ptr, bf.cols, bf.vals64_any, net->blocks, net->z, v);
			}
			for (int c = bf.ncol - 2; c >= 0; c--) {
				int const lo = bf.col_off[c], hi = bf.col_off[c + 1];
				if (hi > lo) k_pssor_bwd<<<nb(hi - lo), 256, 0, st>>>(lo, hi, bf.row_ptr, bf.cols, bf.vals64_any, net->blocks, v);
			}
		}
		else {
			k_power<<<nb(N), 256, 0, st>>>(N, bf.row_ptr, bf.cols, bf.vals64_any, net->blocks, v, net->z);
			MCK(cudaMemcpyAsync(v, net->z, 2l * N * sizeof(double), cudaMemcpyDeviceToDevice, st));
		}
		if (k % 16 == 15 || k == power_iters - 1) {
			k_vnorm<<<FEAT_GRID, TPB_K, 0, st>>>(N, v, net->partials, net->ticket, net->sc);
			k_vscale<<<nb(N), 256, 0, st>>>(N, v, net->sc);
		}
	}
	LossArgs la;
	memset(&la, 0, sizeof la);
	la.N = N;
	la.row_ptr = bf.row_ptr;
	la.cols = bf.cols;
	la.vals64 = bf.vals64_any;
	la.blocks = net->blocks;
	la.lfac = net->lfac;
	la.o = net->o;
	la.r = r;
	la.e = e;
	la.v = v;
	la.partials = net->partials;
	la.ticket = net->ticket;
	la.sc = net->sc;
	la.ssor = ssor;
	k_loss_terms<<<FEAT_GRID, TPB_K, 0, st>>>(la);
	k_loss_back<<<nb(N), 256, 0, st>>>(la, net->d_o);
	int const heads = (N + HEAD_NODES - 1) / HEAD_NODES > 0 ? (N + HEAD_NODES - 1) / HEAD_NODES : 1;
	k_head_back<<<heads, HEAD_TPB, 0, st>>>(N, net->d_o, net->h[3], net->d.theta, net->dh, net->d.gpart);
	k_reduce_parts<<<nb(HEAD_OUT), 256, 0, st>>>(net->d.gpart, heads, HEAD_OUT, net->d.grad, O_WO, 3 * HID, O_BO);
	int const tiles = (N + TILE - 1) / TILE > 0 ? (N + TILE - 1) / TILE : 1;
	int const chunks = (N + DW_CHUNK - 1) / DW_CHUNK > 0 ? (N + DW_CHUNK - 1) / DW_CHUNK : 1;
	long const nh = (long) N * HID;
	for (int l = 3; l >= 1; l--) {
		k_relu_back<<<nb(nh), 256, 0, st>>>(nh, net->dh, net->h[l], net->dpre);
		k_dense_dw<HK><<<chunks, MT, 0, st>>>(N, net->dpre, net->h[l - 1], net->m[l - 1], net->d.gpart);
		k_reduce_parts<<<nb(HID * HK + HID), 256, 0, st>>>(net->d.gpart, chunks, HID * HK + HID, net->d.grad, o_w(l), HID * HK,
		                                                    o_b(l));
		k_dense_dx<<<tiles, MT, 0, st>>>(N, net->dpre, net->d.wb + o_w(l), net->dx);
		k_agg_back<<<nb(nh), 256, 0, st>>>(N, bf.row_ptr, bf.cols, net->dx, net->dh);
	}
	k_relu_back<<<nb(nh), 256, 0, st>>>(nh, net->dh, net->h[0], net->dpre);
	k_dense_dw<FIN><<<chunks, MT, 0, st>>>(N, net->dpre, net->f, nullptr, net->d.gpart);
	k_reduce_parts<<<nb(HID * FIN + HID), 256, 0, st>>>(net->d.gpart, chunks, HID * FIN + HID, net->d.grad, O_W0, HID * FIN,
	                                                     O_B0);
	MCK(cudaGetLastError());
	return 0;
}

int read_loss(bfm_gpu_mpnn* net, double* loss, cudaStream_t st) {
	if (!loss) return 0;
	double sc[5];
	MCK(cudaMemcpyAsync(sc, net->sc, sizeof sc, cudaMemcpyDeviceToHost, st));
	MCK(cudaStreamSynchronize(st));
	*loss = sc[4];
	return 0;
}

// He-normal weights from a fixed-seed generator (xorshift64 + Box-Muller),
// zero biases and a zero head: c = 0, so an untrained network is block Jacobi
void init_theta(float* th, unsigned seed) {
	uint64_t s = 0x9E3779B97F4A7C15ull ^ ((uint64_t) seed * 0xD1B54A32D192ED03ull);
	auto uni = [&]() {
		s ^= s << 13;
		s ^= s >> 7;
		s ^= s << 17;
		return ((double) (s >> 11) + 0.5) * (1.0 / 9007199254740992.0);
	};
	auto normal = [&]() { return sqrt(-2.0 * log(uni())) * cos(6.283185307179586 * uni()); };
	memset(th, 0, sizeof(float) * NPARAM);
	for (int k = 0; k < HID * FIN; k++) th[O_W0 + k] = (float) (normal() * sqrt(2.0 / FIN));
	for (int l = 1; l <= 3; l++)
		for (int k = 0; k < HID * HK; k++) th[o_w(l) + k] = (float) (normal() * sqrt(2.0 / HK));
}

bfm_gpu_mpnn* g_active_net = nullptr;


// weights file: magic, version, layer sizes, parameter count, FP32 parameters (little endian)
constexpr char MAGIC[8] = {'B', 'F', 'M', 'M', 'P', 'N', 'N', '\0'};
constexpr uint32_t FILE_VERSION = 1;

}  // namespace

extern "C" {

int bfm_gpu_mpnn_param_count(void) { return NPARAM; }

int bfm_gpu_mpnn_create(bfm_gpu_mpnn_t** out, unsigned seed) {
	*out = nullptr;
	bfm_gpu_mpnn* net = (bfm_gpu_mpnn*) calloc(1, sizeof *net);
	if (!net) return mfail("out of host memory");
	if (alloc(&net->d.theta, NPARAM) || alloc(&net->d.grad, NPARAM) || alloc(&net->d.adam_m, NPARAM) ||
	    alloc(&net->d.adam_v, NPARAM) || alloc(&net->d.wb, NPARAM) || alloc(&net->sc, 6) ||
	    alloc(&net->partials, 4 * FEAT_GRID) || alloc(&net->rms, 1) || alloc(&net->ticket, 1) || alloc(&net->tc_err, 1)) {
		bfm_gpu_mpnn_destroy(net);
		return -1;
	}
	float* th = (float*) malloc(NPARAM * sizeof(float));
	if (!th) {
		bfm_gpu_mpnn_destroy(net);
		return mfail("out of host memory");
	}
	init_theta(th, seed);
	cudaError_t e = cudaMemcpy(net->d.theta, th, NPARAM * sizeof(float), cudaMemcpyHostToDevice);
	free(th);
	if (e == cudaSuccess) e = cudaMemset(net->ticket, 0, sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMemset(net->tc_err, 0, sizeof(int));
	if (e == cudaSuccess) e = cudaMemset(net->d.adam_m, 0, NPARAM * sizeof(float));
	if (e == cudaSuccess) e = cudaMemset(net->d.adam_v, 0, NPARAM * sizeof(float));
	if (e == cudaSuccess) {
		k_to_bf16<<<nb(NPARAM), 256>>>(NPARAM, net->d.theta, net->d.wb);
		e = cudaDeviceSynchronize();
	}
	if (e != cudaSuccess) {
		bfm_gpu_mpnn_destroy(net);
		return mfail("CUDA error %s creating the network", cudaGetErrorString(e));
	}
	*out = net;
	return 0;
}

int bfm_gpu_mpnn_destroy(bfm_gpu_mpnn_t* net) {
	if (!net) return 0;
	if (g_active_net == net) g_active_net = nullptr;
	cudaDeviceSynchronize();
	free_acts(net);
	void* p[] = {net->d.theta, net->d.grad, net->d.adam_m, net->d.adam_v, net->d.wb, net->d.gpart, net->sc, net->partials,
	             net->rms, net->ticket, net->tc_err};
	for (void* q : p)
		if (q) cudaFree(q);
	free(net);
	return 0;
}

int bfm_gpu_mpnn_get_weights(bfm_gpu_mpnn_t* net, float* out) {
	MCK(cudaMemcpy(out, net->d.theta, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
	return 0;
}

int bfm_gpu_mpnn_set_weights(bfm_gpu_mpnn_t* net, const float* in) {
	MCK(cudaMemcpy(net->d.theta, in, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
	MCK(cudaMemset(net->d.adam_m, 0, NPARAM * sizeof(float)));
	MCK(cudaMemset(net->d.adam_v, 0, NPARAM * sizeof(float)));
	net->step = 0;
	k_to_bf16<<<nb(NPARAM), 256>>>(NPARAM, net->d.theta, net->d.wb);
	MCK(cudaDeviceSynchronize());
	return 0;
}

int bfm_gpu_mpnn_save(bfm_gpu_mpnn_t* net, const char* path) {
	float* th = (float*) malloc(NPARAM * sizeof(float));
	if (!th) return mfail("out of host memory");
	if (bfm_gpu_mpnn_get_weights(net, th)) {
		free(th);
		return -1;
	}
	FILE* f = fopen(path, "wb");
	if (!f) {
		free(th);
		return mfail("cannot open %s for writing", path);
	}
	uint32_t const hdr[6] = {FILE_VERSION, FIN, HID, 3, 3, NPARAM};
	bool ok = fwrite(MAGIC, 1, 8, f) == 8 && fwrite(hdr, sizeof hdr, 1, f) == 1 &&
	          fwrite(th, sizeof(float), NPARAM, f) == (size_t) NPARAM;
	ok = (fclose(f) == 0) && ok;
	free(th);
	return ok ? 0 : mfail("short write to %s", path);
}

int bfm_gpu_mpnn_load(bfm_gpu_mpnn_t* net, const char* path) {
	FILE* f = fopen(path, "rb");
	if (!f) return mfail("cannot open %s", path);
	char magic[8];
	uint32_t hdr[6];
	float* th = (float*) malloc(NPARAM * sizeof(float));
	bool ok = th && fread(magic, 1, 8, f) == 8 && memcmp(magic, MAGIC, 8) == 0 && fread(hdr, sizeof hdr, 1, f) == 1;
	if (ok && (hdr[0] != FILE_VERSION || hdr[1] != FIN || hdr[2] != HID || hdr[3] != 3 || hdr[4] != 3 || hdr[5] != (uint32_t) NPARAM)) {
		fclose(f);
		free(th);
		return mfail("%s: unsupported network file (version %u, %u parameters)", path, hdr[0], hdr[5]);
	}
	ok = ok && fread(th, sizeof(float), NPARAM, f) == (size_t) NPARAM;
	fclose(f);
	if (!ok) {
		free(th);
		return mfail("%s: not a network file or truncated", path);
	}
	int const rc = bfm_gpu_mpnn_set_weights(net, th);
	free(th);
	return rc;
}

int bfm_gpu_mpnn_forward(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* P, float* features, float* c_out, double* blocks) {
	BFM_RANGE("bfm_gpu_mpnn_forward");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	if (forward(net, P, st)) return -1;
	MCK(cudaStreamSynchronize(st));
	int tc_err = 0;
	MCK(cudaMemcpy(&tc_err, net->tc_err, sizeof tc_err, cudaMemcpyDeviceToHost));
	if (tc_err) return mfail("a tcgen05 layer's completion wait ran out");
	long const N = bf.N;
	if (features) {
		bf16* tmp = (bf16*) malloc(N * FIN * sizeof(bf16) + 1);
		if (!tmp) return mfail("out of host memory");
		cudaError_t const e = cudaMemcpy(tmp, net->f, N * FIN * sizeof(bf16), cudaMemcpyDeviceToHost);
		for (long k = 0; k < N * FIN; k++) features[k] = __bfloat162float(tmp[k]);
		free(tmp);
		MCK(e);
	}
	if (c_out) {
		MCK(cudaMemcpy(c_out, net->o, N * 3 * sizeof(float), cudaMemcpyDeviceToHost));
		for (long k = 0; k < N * 3; k++) c_out[k] = C_SCALE * tanhf(c_out[k]);
	}
	if (blocks) MCK(cudaMemcpy(blocks, net->blocks, N * 4 * sizeof(double), cudaMemcpyDeviceToHost));
	return 0;
}

int bfm_gpu_mpnn_gradient(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* P, const double* r, const double* e, double* v,
                          int power_iters, double* loss, float* grad) {
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	if (forward(net, P, st) || backward(net, P, r, e, v, power_iters, st) || read_loss(net, loss, st)) return -1;
	if (grad) {
		MCK(cudaStreamSynchronize(st));
		MCK(cudaMemcpy(grad, net->d.grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
	}
	return 0;
}

int bfm_gpu_mpnn_train_step(bfm_gpu_mpnn_t* net, bfm_gpu_problem_t* P, const double* r, const double* e, double* v,
                            int power_iters, double lr, double* loss) {
	BFM_RANGE("bfm_gpu_mpnn_train_step");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	cudaStream_t const st = (cudaStream_t) bf.stream;
	if (forward(net, P, st) || backward(net, P, r, e, v, power_iters, st)) return -1;
	net->step += 1;
	float const b1t = powf(0.9f, (float) net->step), b2t = powf(0.999f, (float) net->step);
	k_adam<<<nb(NPARAM), 256, 0, st>>>(NPARAM, net->d.theta, net->d.grad, net->d.adam_m, net->d.adam_v, net->d.wb, (float) lr,
	                                    b1t, b2t);
	MCK(cudaGetLastError());
	return read_loss(net, loss, st);
}

int bfm_gpu_mpnn_use(bfm_gpu_mpnn_t* net) {
	g_active_net = net;
	return 0;
}

}  // extern "C"

int bfmi_learned_precond(bfm_gpu_problem_t* P, int jacobi) {
	if (jacobi) return bfmi_set_precond_blocks(P, nullptr);
	if (!g_active_net) return mfail("BFM_GPU_PC_LEARNED needs a network: call bfm_gpu_mpnn_use first");
	bfmi_buffers_t bf;
	bfmi_buffers(P, &bf);
	if (forward(g_active_net, P, (cudaStream_t) bf.stream)) return -1;
	return bfmi_set_precond_blocks(P, g_active_net->blocks);
}
