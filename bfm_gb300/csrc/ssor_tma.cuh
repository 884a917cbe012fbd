// One application of the multicolour block SSOR preconditioner (and of the
// two-level form's coarse correction) as ONE persistent kernel per SM whose
// operands stream through shared memory by TMA bulk copies.
//
// The sweeps read, per phase (one colour, forward or backward), the phase's
// sliced-ELL blocks and column indices and the rows' relaxation blocks:
// nothing any phase writes.  So a producer warp per block streams them,
// tile by tile, into a ring of shared-memory stages (cp.async.bulk, one
// mbarrier per stage for "full" and one for "empty") as far ahead as the
// ring allows -- across the grid barriers that separate the phases -- while
// the block's consumer warps gather the neighbours' sweep values (the only
// operands a phase depends on) from L2 and do the arithmetic.  A phase then
// costs about its bytes at HBM bandwidth instead of a chain of dependent
// loads per row.
//
// Layout of one stage (a tile: up to spt consecutive slices of 32 rows of
// the block's share of the phase's colour):
//   [0, 128)            entry offset of each slice relative to the tile
//                       (spt + 1 ints; the last is the tile's entry count E)
//   [128, 128 + 16 E)   the blocks (float4), column-major per slice
//   [.., + 4 E)         their columns (int, -1 = padding)
//   [.., + 16 rows)     the rows' FP32 relaxation block inverses
//
// Work split: block b takes slices [S b / G, S (b + 1) / G) of each colour
// (S slices, G blocks); within a tile, slice j goes to consumer warp
// (k + j) mod 31, k the number of slices the block has had before the tile,
// so consecutive tiles fill all warps.  Lane = row within the slice.
//
// Two-level correction (at least 3 colours): its stages run between the
// sweeps' own grid barriers -- at the start of phase 0, while the producer
// fills the ring, each block restricts whole aggregates (its share of them:
// the chunks' partial sums, then each aggregate's sum in chunk order into
// r_c); at the start of phase 1 every block stages r_c in shared memory and
// forms its rows of y_t = X r_c; at the start of phase 2 it stages y_t and
// forms its rows of y_c = X^T y_t.  The triangular products follow a work
// list built on the host for the grid (st_tri_list: whole rows per block in
// zig-zag order, cut into segments dealt to the warps): they are bound by
// instruction issue, so every warp gets about the same number of entries and
// no index arithmetic beyond a table lookup.  The backward phases (from
// phase nc on) add P y_c where they store z; the rows of colour nc - 1,
// stored in phase nc - 1, get it at the start of phase nc when that is
// phase 3.
//
// Dynamic shared memory: the ring (ST_NS stages), then (fused form) the
// staged coarse vector in 4 planes, the block's work list of the
// triangular products (copied at kernel start) and the restriction's table
// of the block's chunks and their partial sums.  The grid barriers between
// the phases count arrivals on a monotone counter (st_grid_barrier).
//
// Every wait is bounded: grid barriers by the polls argument (a timeout
// sets the solve's error flag), the mbarrier waits by MBAR_POLLS.  A block
// that gave up still drains the ring (waits for every copy it issued) so no
// copy lands in the shared memory of an exited block.
#pragma once

#include "cg_kernels.cuh"

namespace {

constexpr int ST_THREADS = 1024;            // one block per SM
constexpr int ST_CW = ST_THREADS / 32 - 1;  // consumer warps; warp ST_CW produces
constexpr int ST_NS = 4;                    // ring stages
constexpr int ST_HDR = 128;                 // header bytes of a stage
constexpr int ST_MAX_SPT = 31;              // slices per tile (header: spt + 1 ints)
constexpr long MBAR_POLLS = 1l << 26;       // tries per mbarrier wait before giving up

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned) __cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
	unsigned ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(bar), "r"(parity)
	    : "memory");
	return ok != 0;
}
// wait for the phase of the given parity to complete; false after MBAR_POLLS tries
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
	for (long k = 0; k < MBAR_POLLS; k++)
		if (mbar_try(bar, parity)) return true;
	return false;
}
// bulk copy global -> this block's shared memory, completing on mbarrier `bar`
// (addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(bar)
	             : "memory");
}
// the consumer warps only (named barrier 1)
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"r"(ST_CW * 32) : "memory"); }

// bytes of the staged coarse vector (nc + 4 entries in 4 planes of
// (nc + 7) / 4), then the work list's TRI_SLOTS segments and TRI_SLOTS rows
__host__ __device__ __forceinline__ size_t st_vec_bytes(int nc) { return (((size_t) nc + 8) * sizeof(float2) + 127) / 128 * 128; }
constexpr size_t ST_LIST_BYTES = 2 * TRI_SLOTS * sizeof(int4);
// the restriction's table of the block's chunks (first row, rows), their
// partial sums and the aggregates' first chunks, after the work list
constexpr int RST_CHUNKS = 192;
constexpr int RST_AGGS = 64;
constexpr size_t ST_RST_BYTES = RST_CHUNKS * (sizeof(int2) + 3 * sizeof(double)) + (RST_AGGS + 1) * sizeof(int);

// Grid barrier of the consumer warps (the producer streams on), on a
// monotone arrival counter of its own cache line (word 64 of the barrier
// words): thread 0 of each block adds 1 with a release reduction (no reply
// to wait for) and polls with acquire loads until the counter reaches the
// next multiple of the grid size -- one trip to L2 after the last arrival,
// where a counter that is reset needs the last arriver's atomic reply and
// then its store of a new generation.  Every launch that uses the word has
// the same grid and passes all its barriers, and the word is zeroed before
// each solve, so the counter is a multiple of the grid size at each launch
// start (st_grid_barrier_init).  Block-level synchronisation on named
// barrier 1.  Every consumer thread calls it; a block that has given up
// (*dead: a wait of one of its threads ran out) does not arrive and returns
// false, as do all threads of a block whose wait here runs out -- so the
// result is the same in every thread of the block
constexpr int BAR_CUM = 64;
__device__ __forceinline__ unsigned& st_bar_target() {
	__shared__ unsigned g;
	return g;
}
// at kernel start, before any block can pass the first barrier: the count
// read here lies between the launch's base (a multiple of the grid size)
// and base + gridDim.x - 1
__device__ __forceinline__ void st_grid_barrier_init(unsigned* bar) {
	if (threadIdx.x == 0) {
		unsigned v;
		asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar + BAR_CUM) : "memory");
		st_bar_target() = v - v % gridDim.x;
	}
}
__device__ bool st_grid_barrier(unsigned* bar, int* err, long polls, volatile int* dead) {
	__shared__ int ok;
	consumers_sync();
	if (threadIdx.x == 0 && *dead) ok = 0;
	else if (threadIdx.x == 0) {
		unsigned* count = bar + BAR_CUM;
		unsigned const target = st_bar_target() + gridDim.x;
		int good = 1;
		asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
		long spins = 0;
		unsigned cur;
		while (true) {
			asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(count) : "memory");
			if ((int) (cur - target) >= 0) break;
			++spins;
			if (spins > polls || ((spins & 1023) == 0 && *(volatile int*) err != 0)) {
				atomicExch(err, 1);
				good = 0;
				break;
			}
		}
		st_bar_target() = target;
		ok = good;
		if (!good) *dead = 1;
	}
	consumers_sync();
	return ok;
}

// the block's share [lo, hi) of n items
// (32-bit division when n G fits: a few instructions instead of a 64-bit
// division routine in every consumer warp)
__device__ __forceinline__ void st_share(int n, int& lo, int& hi) {
	unsigned const G = gridDim.x, b = blockIdx.x;
	if ((unsigned long long) n * G < (1ull << 32)) {
		lo = (int) ((unsigned) n * b / G);
		hi = (int) ((unsigned) n * (b + 1) / G);
	}
	else {
		lo = (int) ((long) n * b / G);
		hi = (int) ((long) n * (b + 1) / G);
	}
}

// the block's rows of a padded triangle (row i has i + 1 entries, xrow(i)
// its start): equal shares of the stored floats
__device__ __forceinline__ void st_tri_share(int n, int& lo, int& hi) {
	long const tot = xrow(n);
	auto first = [&](long target) {  // smallest i with xrow(i) >= target
		int a = 0, b = n;
		while (a < b) {
			int const m = (a + b) >> 1;
			if (xrow(m) < target) a = m + 1;
			else b = m;
		}
		return a;
	};
	lo = first(tot * blockIdx.x / gridDim.x);
	hi = first(tot * (blockIdx.x + 1) / gridDim.x);
}

// one warp: the dot product of a padded FP32 triangle row (len entries,
// groups of 4) with a double-float vector in shared memory; lanes take
// groups lane, lane + 32, .. (4 in flight), then a fixed shuffle tree
__device__ __forceinline__ dfl st_row_dot(const float* __restrict__ row, int len, const float2* v, int lane) {
	int const ng = (len + 3) >> 2;
	const float4* r4 = reinterpret_cast<const float4*>(row);
	dfl s = {0.f, 0.f};
	for (int g0 = lane; g0 < ng; g0 += 128) {
		float4 x[4];
#pragma unroll
		for (int u = 0; u < 4; u++) {
			int const g = g0 + 32 * u;
			x[u] = g < ng ? __ldcs(r4 + g) : make_float4(0.f, 0.f, 0.f, 0.f);
		}
#pragma unroll
		for (int u = 0; u < 4; u++) {
			int const g = g0 + 32 * u;
			if (g >= ng) continue;
			float2 const a = v[4 * g], b = v[4 * g + 1], c = v[4 * g + 2], d = v[4 * g + 3];
			s = df_add(s, df_mul_f(x[u].x, {a.x, a.y}));
			s = df_add(s, df_mul_f(x[u].y, {b.x, b.y}));
			s = df_add(s, df_mul_f(x[u].z, {c.x, c.y}));
			s = df_add(s, df_mul_f(x[u].w, {d.x, d.y}));
		}
	}
#pragma unroll
	for (int o = 16; o; o >>= 1) s = df_add(s, {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
	return s;
}

// restriction of one chunk (its nodes: the consecutive rows row0 ..
// row0 + len - 1, len <= COARSE_CHUNK): lane l takes rows l, l + 32, ..
// (all loads first), then double-float sums in that order and a fixed
// shuffle tree; the chunk's 3 sums to part[3 q ..]
template <int VT>
__device__ __forceinline__ void st_restrict_chunk(const CoarseArgs& co, const void* r, int row0, int len, double* out,
                                                  int lane) {
	constexpr int PER = COARSE_CHUNK / 32;
	dfl r0[PER], r1[PER];
	float4 pq[PER];
#pragma unroll
	for (int u = 0; u < PER; u++) {
		int const k = lane + 32 * u;
		double q0, q1;
		r0[u] = r1[u] = {0.f, 0.f};
		pq[u] = make_float4(0.f, 0.f, 0.f, 0.f);
		if (k < len) {
			ssor_ld_r<VT>(r, row0 + k, r0[u], r1[u], q0, q1);
			pq[u] = co.pnode[row0 + k];
		}
	}
	dfl s0 = {0.f, 0.f}, s1 = {0.f, 0.f}, s2 = {0.f, 0.f};
#pragma unroll
	for (int u = 0; u < PER; u++) {
		if (lane + 32 * u >= len) continue;
		dfl const x0 = pq[u].z == 0.f ? dfl{0.f, 0.f} : r0[u];
		dfl const x1 = pq[u].w == 0.f ? dfl{0.f, 0.f} : r1[u];
		s0 = df_add(s0, x0);
		s1 = df_add(s1, x1);
		s2 = df_add(s2, df_add(df_mul_f(-pq[u].y, x0), df_mul_f(pq[u].x, x1)));
	}
#pragma unroll
	for (int o = 16; o; o >>= 1) {
		s0 = df_add(s0, {__shfl_xor_sync(0xffffffffu, s0.hi, o), __shfl_xor_sync(0xffffffffu, s0.lo, o)});
		s1 = df_add(s1, {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)});
		s2 = df_add(s2, {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)});
	}
	if (lane == 0) {
		out[0] = df_dbl(s0);
		out[1] = df_dbl(s1);
		out[2] = df_dbl(s2);
	}
}

// r_c of aggregate I: the partial sums of its chunks (part[3 c ..], c in
// [c0, c1)) in chunk order, lanes 0-2 one component each
__device__ __forceinline__ void st_restrict_sum(const CoarseArgs& co, const double* part, int c0, int c1, int I, int lane) {
	if (lane >= 3) return;
	double s = 0.0;
	for (int c = c0; c < c1; c++) s += part[3 * c + lane];
	dfl const d = df_make(s);
	co.rc[3 * I + lane] = make_float2(d.hi, d.lo);
}

// one warp: the dot product of a segment of a padded FP32 triangle row
// (len <= TRI_SEG entries, groups of 4; lane takes groups lane, lane + 32,
// lane + 64, lane + 96, all loads first) with the entries c, c + 1, .. of a
// double-float vector staged in shared memory in 4 planes of S (entry e at
// vs[(e & 3) S + (e >> 2)]), so that the lanes of a warp read consecutive
// words of one plane: no bank conflicts, whatever c.  Each lane sums in the manner of Ogita, Rump and Oishi's
// Dot2: the products x v_hi split exactly by an FMA, the running sum by
// TwoSum, the rounding errors and x v_lo gathered in a second float -- 11
// FP32 operations per entry where a double-float multiply-add takes 17,
// the same accuracy class (as if summed in twice the working precision);
// then the lanes' double-float sums in a fixed shuffle tree
__device__ __forceinline__ dfl st_seg_dot(const float* __restrict__ row, int len, const float2* vs, int S, int c,
                                          int lane) {
	int const ng = (len + 3) >> 2;
	const float2* v0 = vs + (c & 3) * S + (c >> 2);
	const float2* v1 = vs + ((c + 1) & 3) * S + ((c + 1) >> 2);
	const float2* v2 = vs + ((c + 2) & 3) * S + ((c + 2) >> 2);
	const float2* v3 = vs + ((c + 3) & 3) * S + ((c + 3) >> 2);
	const float4* r4 = reinterpret_cast<const float4*>(row);
	float4 x[4];
#pragma unroll
	for (int u = 0; u < 4; u++) {
		int const g = lane + 32 * u;
		x[u] = g < ng ? __ldcs(r4 + g) : make_float4(0.f, 0.f, 0.f, 0.f);
	}
	float p = 0.f, er = 0.f;
	auto acc = [&](float xv, float2 vv) {
		float const h = __fmul_rn(xv, vv.x);
		float r = __fmaf_rn(xv, vv.x, -h);
		r = __fmaf_rn(xv, vv.y, r);
		float const s = __fadd_rn(p, h);
		float const bb = __fsub_rn(s, p);
		float const q = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(h, bb));
		p = s;
		er = __fadd_rn(er, __fadd_rn(q, r));
	};
#pragma unroll
	for (int u = 0; u < 4; u++) {
		int const g = lane + 32 * u;
		if (g >= ng) continue;
		acc(x[u].x, v0[g]);
		acc(x[u].y, v1[g]);
		acc(x[u].z, v2[g]);
		acc(x[u].w, v3[g]);
	}
	float const h = __fadd_rn(p, er);
	dfl s = {h, __fsub_rn(er, __fsub_rn(h, p))};
#pragma unroll
	for (int o = 16; o; o >>= 1) s = df_add(s, {__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)});
	return s;
}

// the segments of the block's work list that consumer warp `warp` will take,
// of triangle T, prefetched into L2 by the TMA unit (lane 0; addresses and
// sizes are whole groups of 4 floats: 16-byte multiples), so the stage's
// loads hit L2 instead of waiting on DRAM
__device__ __forceinline__ void st_tri_prefetch(const int4* seg_s, int nseg, const float* T, int warp, int lane) {
	if (lane != 0) return;
	for (int q = warp; q < nseg; q += ST_CW) {
		int4 const w = seg_s[q];
		unsigned const bytes = 16u * (unsigned) ((w.z + 3) >> 2);
		asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(T + xrow(w.x) + w.y), "r"(bytes) : "memory");
	}
}

// y_t = X r_c (tr false: row i of X gives y_t[i]) or y_c = X^T y_t (tr true:
// row r of X^T gives y_c[n - 1 - r]) over the block's work list (built on the
// host for this grid: whole rows per block in a zig-zag order, each cut into
// segments of at most TRI_SEG entries, longest first; copied to shared
// memory at kernel start), vec_s the staged vector in 4 planes of S
// (st_seg_dot).  Consumer warp w takes the block's segments w, w + ST_CW, ..; their
// double-float sums go to s_seg, and after the consumers' barrier one thread
// per row adds the row's segments in order.  Deterministic; every warp gets
// about the same number of entries whatever the rows' lengths
__device__ void st_tri_list(const CoarseArgs& co, bool tr, const float2* vec_s, int S, float2* s_seg,
                            const int4* seg_s, int nseg, const int4* row_s, int nrow, int warp, int lane) {
	int const n = co.nc;
	const float* T = tr ? co.xu : co.xl;
	for (int q = warp; q < nseg; q += ST_CW) {
		int4 const w = seg_s[q];  // row, first entry, entries, slot
		int const j = tr ? n - 1 - w.x : 0;
		dfl const d = st_seg_dot(T + xrow(w.x) + w.y, w.z, vec_s, S, j + w.y, lane);
		if (lane == 0) s_seg[w.w] = make_float2(d.hi, d.lo);
	}
	consumers_sync();
	for (int k = threadIdx.x; k < nrow; k += ST_CW * 32) {
		int4 const w = row_s[k];  // row, first slot, slots
		dfl acc = {0.f, 0.f};
		for (int q = 0; q < w.z; q++) acc = df_add(acc, {s_seg[w.y + q].x, s_seg[w.y + q].y});
		(tr ? co.yc : co.yt)[tr ? n - 1 - w.x : w.x] = make_float2(acc.hi, acc.lo);
	}
}

// sum of A_ij y_j over the staged blocks of one row: w blocks at stride 32
// in shared memory, 4 gathers of y (L2) in flight
__device__ __forceinline__ void st_row_sum(const float4* sv, const int* sc, int w, const float* y, dfl& t0, dfl& t1) {
	for (int kb = 0; kb < w; kb += 4) {
		int c[4];
#pragma unroll
		for (int j = 0; j < 4; j++) c[j] = kb + j < w ? sc[32 * (kb + j)] : -1;
		float4 g[4];
#pragma unroll
		for (int j = 0; j < 4; j++)
			g[j] = c[j] >= 0 ? __ldcg(reinterpret_cast<const float4*>(y) + c[j]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
		for (int j = 0; j < 4; j++) {
			if (c[j] < 0) continue;
			float4 const m = sv[32 * (kb + j)];
			dfl const g0 = {g[j].x, g[j].z}, g1 = {g[j].y, g[j].w};
			t0 = df_add(t0, df_add(df_mul_f(m.x, g0), df_mul_f(m.y, g1)));
			t1 = df_add(t1, df_add(df_mul_f(m.z, g0), df_mul_f(m.w, g1)));
		}
	}
}

template <int VT>
__global__ void __launch_bounds__(ST_THREADS, 1) k_ssor_tma(SsorArgs a) {
	if (a.st->done && !a.timing) return;
	extern __shared__ __align__(128) unsigned char st_smem[];
	__shared__ __align__(8) unsigned long long full[ST_NS], empty[ST_NS];
	__shared__ volatile int s_abort, s_issued, s_dead;
	__shared__ double s_red[ST_THREADS / 32];
	__shared__ bool s_last;
	__shared__ float2 s_seg[TRI_SLOTS];  // segment sums of the triangular products
	__shared__ int s_nseg, s_nrow;       // the block's work list: segments, rows
	int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	int const nc = a.ncol > 0 ? a.ncol : 1, nph = 2 * nc - 1;
	bool const fuse = a.fuse && nc >= 3;
	float2* vec_s = reinterpret_cast<float2*>(st_smem + (size_t) ST_NS * a.stage_bytes);  // r_c, then y_t (fused)
	// the block's work list of the triangular products (fused), after the vector
	int4* seg_s = reinterpret_cast<int4*>(st_smem + (size_t) ST_NS * a.stage_bytes + st_vec_bytes(a.co.nc));
	int4* row_s = seg_s + TRI_SLOTS;
	double* rpart_s = reinterpret_cast<double*>(row_s + TRI_SLOTS);  // 3 per chunk
	int2* rchk_s = reinterpret_cast<int2*>(rpart_s + 3 * RST_CHUNKS);  // first row, rows
	int* ragg_s = reinterpret_cast<int*>(rchk_s + RST_CHUNKS);         // first chunk of each aggregate (local)
	if (threadIdx.x == 0) {
		for (int s = 0; s < ST_NS; s++) {
			mbar_init(smem_u32(&full[s]), 1);
			mbar_init(smem_u32(&empty[s]), ST_CW);
		}
		s_abort = 0;
		s_issued = 0;
		s_dead = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	st_grid_barrier_init(a.bar);
	__syncthreads();
	dfl acc = {0.f, 0.f};
	double acc64 = 0.0;
	if (warp == ST_CW) {
		// ---------------------------------------------------------- producer
		int t = 0;
		bool ok = true;
		for (int ph = 0; ph < nph && ok; ph++) {
			bool const fwd = ph < nc;
			int const c = fwd ? ph : 2 * nc - 2 - ph;
			int const lo = a.off[c], hi = a.off[c + 1];
			const int* ptr = fwd ? a.lp : a.up;
			const float4* V = fwd ? a.lv : a.uv;
			const int* CI = fwd ? a.lc : a.uc;
			int sa, sb;
			st_share(a.sbase[c + 1] - a.sbase[c], sa, sb);
			sa += a.sbase[c];
			sb += a.sbase[c];
			int const spt = a.spt[ph];
			for (int s0 = sa; s0 < sb; s0 += spt, t++) {
				int const ns = min(spt, sb - s0), stg = t % ST_NS;
				if (t >= ST_NS && !mbar_wait(smem_u32(&empty[stg]), ((t / ST_NS) - 1) & 1)) {
					ok = false;
					break;
				}
				unsigned char* base = st_smem + (size_t) stg * a.stage_bytes;
				int const pk = lane <= ns ? __ldg(ptr + s0 + lane) : 0;
				int const p0 = __shfl_sync(0xffffffffu, pk, 0), pe = __shfl_sync(0xffffffffu, pk, ns);
				if (lane <= ns) reinterpret_cast<int*>(base)[lane] = pk - p0;
				__syncwarp();
				int const E = pe - p0;
				int const r0 = lo + 32 * (s0 - a.sbase[c]);
				int const rows = min(32 * ns, hi - r0);
				if (ST_HDR + 20l * E + 16l * rows > a.stage_bytes) {  // tiling does not match the slices: stop
					ok = false;
					break;
				}
				if (lane == 0) {
					unsigned const bar = smem_u32(&full[stg]);
					mbar_expect_tx(bar, 20u * (unsigned) E + 16u * (unsigned) rows);
					if (E > 0) {
						bulk_g2s(smem_u32(base + ST_HDR), V + p0, 16u * (unsigned) E, bar);
						bulk_g2s(smem_u32(base + ST_HDR + 16 * E), CI + p0, 4u * (unsigned) E, bar);
					}
					bulk_g2s(smem_u32(base + ST_HDR + 20 * E), reinterpret_cast<const float4*>(a.dinv) + r0, 16u * (unsigned) rows,
					         bar);
					s_issued = t + 1;
				}
				__syncwarp();
			}
		}
		if (!ok && lane == 0) {
			s_abort = 1;
			atomicExch(&a.st->ssor_err, 1);
		}
	}
	else {
		// ---------------------------------------------------------- consumers
		int t = 0, kg = 0;
		bool alive = true;
		CoarseArgs const& co = a.co;
		bool const lst = fuse && co.tri_g == (int) gridDim.x;  // the work list (planar vector), else rows per warp
		if (lst) {
			// the block's work list to shared memory (read first in phase 0,
			// after the restriction's consumer barrier)
			int const sa = co.tri_sp[blockIdx.x], sb = co.tri_sp[blockIdx.x + 1];
			int const ra = co.tri_rp[blockIdx.x], rb = co.tri_rp[blockIdx.x + 1];
			if (threadIdx.x == 0) {
				s_nseg = sb - sa;
				s_nrow = rb - ra;
			}
			for (int u = threadIdx.x; u < sb - sa; u += ST_CW * 32) seg_s[u] = co.tri_seg[sa + u];
			for (int u = threadIdx.x; u < rb - ra; u += ST_CW * 32) row_s[u] = co.tri_row[ra + u];
		}

		for (int ph = 0; ph < nph; ph++) {
			bool const fwd = ph < nc;
			int const c = fwd ? ph : 2 * nc - 2 - ph;
			int const lo = a.off[c], hi = a.off[c + 1];
			if (ph > 0) alive = st_grid_barrier(a.bar, &a.st->ssor_err, a.polls, &s_dead);
			if (fuse && ph == 0) {
				// restriction by whole aggregates per block, while the producer
				// fills the ring: the chunks' partial sums, then (after a
				// consumers' barrier) each aggregate's sum in chunk order into
				// r_c.  No other block touches these aggregates; the grid
				// barrier before phase 1 publishes r_c.  The block's chunks and
				// partial sums sit in a shared-memory table when it fits (one
				// round of lookups instead of a chain per chunk), else in the
				// global arrays
				int A0, A1;
				st_share(co.na, A0, A1);
				int const qa = co.agg_chunk[A0], qb = co.agg_chunk[A1];
				bool const rtab = co.tables && qb - qa <= RST_CHUNKS && A1 - A0 <= RST_AGGS;
				if (rtab) {
					for (int u = threadIdx.x; u < qb - qa; u += ST_CW * 32) {
						int const k0 = co.chunk_start[qa + u], k1 = co.chunk_start[qa + u + 1];
						rchk_s[u] = make_int2(co.agg_nodes[k0], k1 - k0);
					}
					for (int u = threadIdx.x; u <= A1 - A0; u += ST_CW * 32) ragg_s[u] = co.agg_chunk[A0 + u] - qa;
					consumers_sync();  // the table
					for (int q = warp; q < qb - qa; q += ST_CW)
						st_restrict_chunk<VT>(co, a.r, rchk_s[q].x, rchk_s[q].y, rpart_s + 3 * q, lane);
					consumers_sync();
					for (int I = A0 + warp; I < A1; I += ST_CW)
						st_restrict_sum(co, rpart_s, ragg_s[I - A0], ragg_s[I - A0 + 1], I, lane);
				}
				else {
					for (int q = qa + warp; q < qb; q += ST_CW) {
						int const k0 = co.chunk_start[q];
						st_restrict_chunk<VT>(co, a.r, co.agg_nodes[k0], co.chunk_start[q + 1] - k0, co.part + 3l * q, lane);
					}
					consumers_sync();  // orders the block's global writes of the partial sums
					for (int I = A0 + warp; I < A1; I += ST_CW)
						st_restrict_sum(co, co.part, co.agg_chunk[I], co.agg_chunk[I + 1], I, lane);
				}
				if (lst) st_tri_prefetch(seg_s, s_nseg, co.xl, warp, lane);  // X, for phase 1
			}
			if (fuse && alive && (ph == 1 || ph == 2)) {
				// y_t = X r_c (phase 1) or y_c = X^T y_t (phase 2), the vector
				// (from the other blocks, published by the grid barrier) staged
				// in shared memory
				bool const tr = ph == 2;
				int const S = (co.nc + 7) >> 2;
				for (int u = threadIdx.x; u < co.nc + 4; u += ST_CW * 32)
					vec_s[lst ? (u & 3) * S + (u >> 2) : u] = u < co.nc ? __ldcg((tr ? co.yt : co.rc) + u) : make_float2(0.f, 0.f);
				consumers_sync();
				if (lst) {
					st_tri_list(co, tr, vec_s, S, s_seg, seg_s, s_nseg, row_s, s_nrow, warp, lane);
					if (!tr) st_tri_prefetch(seg_s, s_nseg, co.xu, warp, lane);  // X^T, for phase 2
				}
				else {
					// one warp per row of the block's contiguous share
					int i0, i1;
					st_tri_share(co.nc, i0, i1);
					for (int i = i0 + warp; i < i1; i += ST_CW) {
						int const j = tr ? co.nc - 1 - i : i;
						dfl const d = st_row_dot((tr ? co.xu : co.xl) + xrow(i), i + 1, tr ? vec_s + j : vec_s, lane);
						if (lane == 0) (tr ? co.yc : co.yt)[j] = make_float2(d.hi, d.lo);
					}
				}
			}
			if (fuse && alive && ph == 3 && nc == 3) {
				// colour 2 was stored in phase 2, before y_c: its coarse term now
				int ra, rb;
				st_share(a.off[3] - a.off[2], ra, rb);
				for (int i = a.off[2] + ra + threadIdx.x; i < a.off[2] + rb; i += ST_CW * 32) ssor_add_coarse<VT>(a, i, acc, acc64);
			}
			// the sweep tiles of this phase (also drained when the block gave up)
			int sa, sb;
			st_share(a.sbase[c + 1] - a.sbase[c], sa, sb);
			sa += a.sbase[c];
			sb += a.sbase[c];
			int const spt = a.spt[ph];
			bool const final_rows = !fwd || c == nc - 1;
			bool const plain = fuse && fwd && nc == 3;  // final before y_c exists
			for (int s0 = sa; s0 < sb; s0 += spt, t++) {
				int const ns = min(spt, sb - s0), stg = t % ST_NS;
				bool const have = !(s_abort && t >= s_issued);
				bool const got = have && mbar_wait(smem_u32(&full[stg]), (t / ST_NS) & 1);
				if (!got) {
					if (alive && lane == 0) atomicExch(&a.st->ssor_err, 1);
					alive = false;
					s_dead = 1;
				}
				if (got && alive) {
					const unsigned char* base = st_smem + (size_t) stg * a.stage_bytes;
					const int* hdr = reinterpret_cast<const int*>(base);
					int const E = hdr[ns];
					int j = (warp - kg % ST_CW + ST_CW) % ST_CW;
					for (; j < ns; j += ST_CW) {
						int const e0 = hdr[j], w = (hdr[j + 1] - e0) >> 5;
						int const i = lo + 32 * (s0 + j - a.sbase[c]) + lane;
						if (i >= hi) continue;
						const float4* sv = reinterpret_cast<const float4*>(base + ST_HDR) + e0 + lane;
						const int* sc = reinterpret_cast<const int*>(base + ST_HDR + 16 * E) + e0 + lane;
						float4 const d = reinterpret_cast<const float4*>(base + ST_HDR + 20 * E)[32 * j + lane];
						dfl r0, r1, z0, z1;
						double q0 = 0.0, q1 = 0.0;
						dfl t0 = {0.f, 0.f}, t1 = {0.f, 0.f};
						if (fwd) {
							ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
							st_row_sum(sv, sc, w, a.y, t0, t1);
							ssor_blk(d, df_add(r0, df_neg(t0)), df_add(r1, df_neg(t1)), z0, z1);
						}
						else {
							float4 const yv = __ldcg(reinterpret_cast<const float4*>(a.y) + i);
							ssor_ld_r<VT>(a.r, i, r0, r1, q0, q1);
							st_row_sum(sv, sc, w, a.y, t0, t1);
							dfl w0, w1;
							ssor_blk(d, t0, t1, w0, w1);
							z0 = df_add({yv.x, yv.z}, df_neg(w0));
							z1 = df_add({yv.y, yv.w}, df_neg(w1));
						}
						__stcg(reinterpret_cast<float4*>(a.y) + i, make_float4(z0.hi, z1.hi, z0.lo, z1.lo));
						if (final_rows) {
							if (plain) ssor_st_plain<VT>(a, i, z0, z1);
							else ssor_st_z<VT>(a, i, z0, z1, r0, r1, q0, q1, acc, acc64);
						}
					}
				}
				kg += ns;
				__syncwarp();
				if (got && lane == 0) mbar_arrive(smem_u32(&empty[stg]));
			}
		}
	}
	// every thread of every block reaches the reduction, finished or not:
	// warps in order, then blocks in order (deterministic)
	double v = VT == VT_F64 ? acc64 : df_dbl(acc);
	for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	if (lane == 0) s_red[warp] = v;
	__syncthreads();
	if (threadIdx.x == 0) {
		double s = 0.0;
		for (int k = 0; k < ST_THREADS / 32; k++) s += s_red[k];
		a.partials[blockIdx.x] = s;
		__threadfence();
		unsigned const tk = atomicAdd(a.ticket, 1u);
		s_last = tk == gridDim.x - 1;
	}
	__syncthreads();
	if (!s_last) return;
	__threadfence();
	double w = 0.0;
	for (int blk = threadIdx.x; blk < gridDim.x; blk += blockDim.x) w += __ldcg(a.partials + blk);
	for (int o = 16; o; o >>= 1) w += __shfl_down_sync(0xffffffffu, w, o);
	__syncthreads();
	if (lane == 0) s_red[warp] = w;
	__syncthreads();
	if (threadIdx.x == 0) {
		double s = 0.0;
		for (int k = 0; k < ST_THREADS / 32; k++) s += s_red[k];
		*a.ticket = 0u;
		ssor_finish(a, s);
	}
}

}  // namespace
