// "sbitonic" and "abitonic": the reference's bitonic sorting network,
// replayed exactly on sm_103a.
//
// Network (src/cl_ops/sort/clo_sort_sbitonic.cl:38-69 and the grouped
// kernels of clo_sort_abitonic.cl:31-1067): over N = nlpo2(n) elements,
// for stage s = 1..log2 N and step t = s..1, elements i and i + 2^(t-1)
// with bit t-1 of i clear are compared; the block direction is bit s of i
// (1 = descending); they swap iff COMPARE(key_i, key_j) XOR desc, with
// COMPARE(a, b) = a > b. Every step touches disjoint pairs, so any
// implementation that applies the same steps in the same order produces
// the same array, bit for bit, including where the compare is not a total
// order (equal keys, NaN, -0.0/+0.0).
//
// sbitonic keeps the reference's one-step-per-launch structure.
// abitonic groups the steps:
//   - abitonic_tile_sort: each shared-memory tile of 2^t elements runs
//     stages 1..t (the stage-t direction comes from the tile's index);
//   - abitonic_global_steps<g>: g (<= 6) consecutive steps with strides
//     >= the tile, 2^g elements per thread held in registers;
//   - abitonic_tile_finish: the remaining steps t..1 of a stage in shared
//     memory.
// Inside the tile kernels steps are also applied 4 at a time on 16
// registers per thread between barriers.
// Sizes that are not a power of two are padded (in a temporary buffer)
// with the element type's maximum, which the final ascending stage moves
// past the real elements; the reference requires power-of-two sizes.
//
// HBM roofline: 2 x sizeof(T) x N bytes per launch (one read, one write).
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <climits>

#include "clo_internal.h"
#include <type_traits>

#include "dev_common.cuh"
#include "timing.h"

namespace clo {
namespace {

struct Half16 {
	uint16_t bits;
};

template <typename T>
struct BT {
	__device__ __forceinline__ static bool gt(T a, T b) { return a > b; }
};
template <>
struct BT<Half16> {
	__device__ __forceinline__ static bool gt(Half16 a, Half16 b) {
		return __half2float(__ushort_as_half(a.bits)) >
			__half2float(__ushort_as_half(b.bits));
	}
};

template <typename T>
__device__ __forceinline__ void cmpxchg(T &a, T &b, bool desc) {
	if (BT<T>::gt(a, b) != desc) {
		T t = a;
		a = b;
		b = t;
	}
}

// ------------------------------------------------------------ sbitonic
template <typename T>
__global__ void __launch_bounds__(256)
sbitonic_step(T *data, size_t half_n, int stage, int step) {
	size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (gid >= half_n) return;
	size_t stride = (size_t)1 << (step - 1);
	size_t i1 = gid + (gid & ~(stride - 1));
	size_t i2 = i1 + stride;
	bool desc = (gid >> (stage - 1)) & 1;
	T a = data[i1], b = data[i2];
	if (BT<T>::gt(a, b) != desc) {
		data[i1] = b;
		data[i2] = a;
	}
}

// ------------------------------------------------- abitonic global steps
// Steps step .. step-G+1 of `stage`, 2^G elements per thread.
// Threads per CTA of the global passes: 128 for 7 steps (128 elements and
// 168 registers a thread, three CTAs per SM), else 256.
template <int G>
constexpr int gs_threads() { return G >= 7 ? 128 : 256; }

template <typename T, int G>
__global__ void __launch_bounds__(gs_threads<G>(), G >= 7 ? 3 : G >= 6 ? 2 : 1)
abitonic_global_steps(T *data, size_t groups, int stage, int step) {
	size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (q >= groups) return;
	const int lo_bits = step - G;
	size_t low = q & (((size_t)1 << lo_bits) - 1);
	size_t high = q >> lo_bits;
	size_t base = (high << step) | low;
	const size_t inc = (size_t)1 << lo_bits;
	const bool desc = (base >> stage) & 1;
	T r[1 << G];
	T *p = data + base;
#pragma unroll
	for (int m = 0; m < (1 << G); ++m) r[m] = p[m * inc];
#pragma unroll
	for (int s = G - 1; s >= 0; --s) {
#pragma unroll
		for (int m = 0; m < (1 << G); ++m)
			if (!(m & (1 << s))) cmpxchg(r[m], r[m | (1 << s)], desc);
	}
	// With 64 or more elements a thread, the store addresses are computed
	// afresh rather than kept from the loads (as many more live registers).
	if constexpr (G >= 6) asm volatile("" : "+l"(p));
#pragma unroll
	for (int m = 0; m < (1 << G); ++m) p[m * inc] = r[m];
}

// ------------------------------------------------- shared-memory tiles
constexpr int kTileThreads = 512;

__device__ __forceinline__ uint32_t spad(uint32_t i) { return i + (i >> 5); }

// Applies steps j .. j-g+1 of a stage to the tile in shared memory, in
// groups of 2^g elements held in registers. `desc_fn(i)` gives the
// direction of element i (tile-local index).
template <typename T, int G, typename DescFn>
__device__ __forceinline__ void smem_steps(T *s, uint32_t tile_n, int j,
	DescFn desc_fn) {
	const int lo_bits = j - G;
	const uint32_t groups = tile_n >> G;
	const uint32_t inc = 1u << lo_bits;
	for (uint32_t q = threadIdx.x; q < groups; q += blockDim.x) {
		uint32_t low = q & (inc - 1);
		uint32_t base = ((q >> lo_bits) << j) | low;
		bool desc = desc_fn(base);
		T r[1 << G];
#pragma unroll
		for (int m = 0; m < (1 << G); ++m) r[m] = s[spad(base + m * inc)];
#pragma unroll
		for (int b = G - 1; b >= 0; --b) {
#pragma unroll
			for (int m = 0; m < (1 << G); ++m)
				if (!(m & (1 << b))) cmpxchg(r[m], r[m | (1 << b)], desc);
		}
#pragma unroll
		for (int m = 0; m < (1 << G); ++m) s[spad(base + m * inc)] = r[m];
	}
}

// Steps j..1 of one stage, at most maxg (<= 4) per barrier interval.
template <typename T, typename DescFn>
__device__ __forceinline__ void smem_stage_tail(T *s, uint32_t tile_n, int j,
	int maxg, DescFn desc_fn) {
	while (j >= 1) {
		int g = j < maxg ? j : maxg;
		switch (g) {
		case 4: smem_steps<T, 4>(s, tile_n, j, desc_fn); break;
		case 3: smem_steps<T, 3>(s, tile_n, j, desc_fn); break;
		case 2: smem_steps<T, 2>(s, tile_n, j, desc_fn); break;
		default: smem_steps<T, 1>(s, tile_n, j, desc_fn); break;
		}
		__syncthreads();
		j -= g;
	}
}

template <typename T>
__device__ __forceinline__ void tile_load(T *s, const T *g, uint32_t tile_n) {
	for (uint32_t i = threadIdx.x; i < tile_n; i += blockDim.x) s[spad(i)] = g[i];
	__syncthreads();
}

template <typename T>
__device__ __forceinline__ void tile_store(T *g, const T *s, uint32_t tile_n) {
	for (uint32_t i = threadIdx.x; i < tile_n; i += blockDim.x) g[i] = s[spad(i)];
}

// Stages 1..t of every tile of 2^t elements.
template <typename T>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) <= 4 ? 3 : 2)
abitonic_tile_sort(T *data, int t, int maxg) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *s = reinterpret_cast<T *>(smem_raw);
	const uint32_t tile_n = 1u << t;
	const size_t tile_base = (size_t)blockIdx.x << t;
	T *g = data + tile_base;
	tile_load(s, g, tile_n);
	for (int stage = 1; stage <= t; ++stage) {
		if (stage < t) {
			smem_stage_tail(s, tile_n, stage, maxg,
				[stage](uint32_t i) { return (bool)((i >> stage) & 1); });
		} else {
			const bool d = (tile_base >> stage) & 1;
			smem_stage_tail(s, tile_n, stage, maxg, [d](uint32_t) { return d; });
		}
	}
	tile_store(g, s, tile_n);
}

// Steps t..1 of `stage` (> t) for every tile.
template <typename T>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) <= 4 ? 3 : 2)
abitonic_tile_finish(T *data, int t, int stage, int maxg) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *s = reinterpret_cast<T *>(smem_raw);
	const uint32_t tile_n = 1u << t;
	const size_t tile_base = (size_t)blockIdx.x << t;
	T *g = data + tile_base;
	const bool d = (tile_base >> stage) & 1;
	tile_load(s, g, tile_n);
	smem_stage_tail(s, tile_n, t, maxg, [d](uint32_t) { return d; });
	tile_store(g, s, tile_n);
}

// ------------------------------------ register-phase tiles (<= 4 bytes)
// Tiles of 2^14 elements, 512 threads, 32 elements per thread held in
// registers. In layout L(B0) register m of thread tid holds tile element
//   ((tid >> B0) << (B0 + 5)) | (m << B0) | (tid & (2^B0 - 1)),
// so the steps on index bits B0 .. B0 + 4 are compare-exchanges between a
// thread's own registers. A stage's steps (bits top .. 0) run in up to
// three such phases -- bits 13..9 in L(9), 8..5 in L(4), 4..0 in L(0) --
// joined by transposes through the padded shared tile (each layout puts a
// warp's 32 accesses in 32 banks). Per tile pass this is two shared
// stores and two loads per element instead of one of each per four steps.
// The steps and their order are those of the network, so the result is
// the same as the shared-memory rounds' (and the reference's).
constexpr int kRLog = 14, kRE = 5, kRThreads = 512, kRN = 1 << kRE;

template <int B0>
__device__ __forceinline__ uint32_t lidx(uint32_t tid, uint32_t m) {
	return ((tid >> B0) << (B0 + kRE)) | (m << B0) | (tid & ((1u << B0) - 1u));
}

// Compare-exchange with a direction fixed at compile time: for integers a
// min/max pair (swap iff a > b ascending, iff a <= b descending: the same
// values either way), otherwise the network's own compare.
template <bool DESC, typename T>
__device__ __forceinline__ void cx_s(T &a, T &b) {
	if constexpr (std::is_integral<T>::value) {
		const T lo = a < b ? a : b, hi = a < b ? b : a;
		a = DESC ? hi : lo;
		b = DESC ? lo : hi;
	} else {
		cmpxchg(a, b, DESC);
	}
}

// Steps on bits HI .. LO (within B0 .. B0 + 4) in layout L(B0); dir(a, b, m)
// compare-exchanges registers m and m | stride.
template <int B0, int HI, int LO, typename T, typename Dir>
__device__ __forceinline__ void rphase(T (&r)[kRN], Dir dir) {
#pragma unroll
	for (int b = HI; b >= LO; --b) {
		const int sb = 1 << (b - B0);
#pragma unroll
		for (int m = 0; m < kRN; ++m)
			if (!(m & sb)) dir(r[m], r[m | sb], m);
	}
}

// Padded shared-memory slot of element (tid, m) of L(B0), split as a
// per-thread base plus a per-register constant: the register bits never
// carry into the padding term, so
//   spad(lidx(tid, m)) = spad(lidx(tid, 0)) + (m << B0) + ((m << B0) >> 5).
template <int B0>
__device__ __forceinline__ uint32_t lbase(uint32_t tid) {
	return spad(lidx<B0>(tid, 0));
}
template <int B0>
__host__ __device__ constexpr uint32_t loff(int m) {
	return ((uint32_t)m << B0) + (((uint32_t)m << B0) >> 5);
}

template <int FROM, int TO, typename T>
__device__ __forceinline__ void rtranspose(T (&r)[kRN], T *s, uint32_t tid) {
	// L(0) and L(4) give a half-warp the same 512 consecutive elements
	// (index bits 9..13 are its thread bits 4..8), so a transpose between
	// them stays inside the warp's own part of the tile and needs only the
	// warp to synchronise; the part's previous readers were this warp's
	// threads (a transpose into L(0) or L(4) reads only the reader's part,
	// and one into L(9) is always followed by one out of it, which starts
	// with a CTA barrier).
	constexpr bool kLocal = (FROM == 0 || FROM == 4) && (TO == 0 || TO == 4);
	if constexpr (kLocal) __syncwarp();
	else __syncthreads();
	T *sf = s + lbase<FROM>(tid);
#pragma unroll
	for (int m = 0; m < kRN; ++m) sf[loff<FROM>(m)] = r[m];
	if constexpr (kLocal) __syncwarp();
	else __syncthreads();
	const T *st = s + lbase<TO>(tid);
#pragma unroll
	for (int m = 0; m < kRN; ++m) r[m] = st[loff<TO>(m)];
}

// One phase of stage S (< kRLog) in layout L(B0): the direction of a pair
// is bit S of its lower element's tile index, which is a register bit
// (fixed per register) or a thread bit (fixed per thread).
template <int S, int B0, int HI, int LO, typename T>
__device__ __forceinline__ void sort_phase(T (&r)[kRN], uint32_t tid) {
	if constexpr (S >= B0 && S < B0 + kRE) {
		rphase<B0, HI, LO>(r, [](T &a, T &b, int m) {
			if ((m >> (S - B0)) & 1) cx_s<true>(a, b);
			else cx_s<false>(a, b);
		});
	} else {
		const bool d = (tid >> (S < B0 ? S : S - kRE)) & 1u;
		rphase<B0, HI, LO>(r, [d](T &a, T &b, int) { cmpxchg(a, b, d); });
	}
}

// Stage S (< kRLog) of the tile sort; the registers are in L(0) before and
// after.
template <int S, typename T>
__device__ __forceinline__ void sort_stage(T (&r)[kRN], T *s, uint32_t tid) {
	constexpr int top = S - 1;
	if constexpr (top >= 9) {
		rtranspose<0, 9>(r, s, tid);
		sort_phase<S, 9, top, 9>(r, tid);
		rtranspose<9, 4>(r, s, tid);
		sort_phase<S, 4, 8, 5>(r, tid);
		rtranspose<4, 0>(r, s, tid);
		sort_phase<S, 0, 4, 0>(r, tid);
	} else if constexpr (top >= 5) {
		rtranspose<0, 4>(r, s, tid);
		sort_phase<S, 4, top, 5>(r, tid);
		rtranspose<4, 0>(r, s, tid);
		sort_phase<S, 0, 4, 0>(r, tid);
	} else {
		sort_phase<S, 0, top, 0>(r, tid);
	}
}

template <int S, typename T>
__device__ __forceinline__ void sort_stages(T (&r)[kRN], T *s, uint32_t tid) {
	sort_stage<S>(r, s, tid);
	if constexpr (S + 1 < kRLog) sort_stages<S + 1>(r, s, tid);
}

// All 14 steps of a stage with one direction for the whole tile, starting
// in L(9) and ending in L(0).
template <bool D, typename T>
__device__ __forceinline__ void full_stage_uniform(T (&r)[kRN], T *s, uint32_t tid) {
	auto dir = [](T &a, T &b, int) { cx_s<D>(a, b); };
	rphase<9, 13, 9>(r, dir);
	rtranspose<9, 4>(r, s, tid);
	rphase<4, 8, 5>(r, dir);
	rtranspose<4, 0>(r, s, tid);
	rphase<0, 4, 0>(r, dir);
}

// A thread's 32 consecutive 4-byte elements move as 32-byte vectors when
// the tile is 32-byte aligned (half the requests of 16-byte vectors, whose
// lanes 128 bytes apart each touch a line of their own), else as 16-byte
// vectors.
template <typename T>
__device__ __forceinline__ void rload_l0(T (&r)[kRN], const T *g, T *s, uint32_t tid) {
	if constexpr (sizeof(T) == 4) {
		const T *src = g + ((size_t)tid << kRE);
		if (((uintptr_t)g % 32) == 0) {
#pragma unroll
			for (int q = 0; q < kRN / 8; ++q) {
				uint32_t w[8];
				dev::ld_v8(src + 8 * q, w);
#pragma unroll
				for (int e = 0; e < 8; ++e) r[8 * q + e] = __builtin_bit_cast(T, w[e]);
			}
		} else {
			const uint4 *src4 = reinterpret_cast<const uint4 *>(src);
#pragma unroll
			for (int q = 0; q < kRN / 4; ++q) {
				const uint4 v = src4[q];
				r[4 * q + 0] = __builtin_bit_cast(T, v.x);
				r[4 * q + 1] = __builtin_bit_cast(T, v.y);
				r[4 * q + 2] = __builtin_bit_cast(T, v.z);
				r[4 * q + 3] = __builtin_bit_cast(T, v.w);
			}
		}
	} else {
#pragma unroll
		for (int m = 0; m < kRN; ++m) r[m] = g[lidx<9>(tid, m)];
		rtranspose<9, 0>(r, s, tid);
	}
}

template <typename T>
__device__ __forceinline__ void rstore_l0(T *g, T (&r)[kRN], T *s, uint32_t tid) {
	if constexpr (sizeof(T) == 4) {
		T *dst = g + ((size_t)tid << kRE);
		if (((uintptr_t)g % 32) == 0) {
#pragma unroll
			for (int q = 0; q < kRN / 8; ++q) {
				uint32_t w[8];
#pragma unroll
				for (int e = 0; e < 8; ++e) w[e] = __builtin_bit_cast(uint32_t, r[8 * q + e]);
				dev::st_v8(dst + 8 * q, w);
			}
		} else {
			uint4 *dst4 = reinterpret_cast<uint4 *>(dst);
#pragma unroll
			for (int q = 0; q < kRN / 4; ++q)
				dst4[q] = make_uint4(__builtin_bit_cast(uint32_t, r[4 * q + 0]),
					__builtin_bit_cast(uint32_t, r[4 * q + 1]),
					__builtin_bit_cast(uint32_t, r[4 * q + 2]),
					__builtin_bit_cast(uint32_t, r[4 * q + 3]));
		}
	} else {
		rtranspose<0, 9>(r, s, tid);
#pragma unroll
		for (int m = 0; m < kRN; ++m) g[lidx<9>(tid, m)] = r[m];
	}
}

// Stages 1..14 of every tile of 2^14 elements.
template <typename T>
__global__ void __launch_bounds__(kRThreads, 2)
abitonic_tile_sort_r(T *data) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *s = reinterpret_cast<T *>(smem_raw);
	const uint32_t tid = threadIdx.x;
	const size_t tile_base = (size_t)blockIdx.x << kRLog;
	T *g = data + tile_base;
	T r[kRN];
	rload_l0(r, g, s, tid);
	sort_stages<1>(r, s, tid);
	// Stage 14: one direction for the tile (bit 14 of its global index).
	rtranspose<0, 9>(r, s, tid);
	if ((tile_base >> kRLog) & 1) full_stage_uniform<true>(r, s, tid);
	else full_stage_uniform<false>(r, s, tid);
	rstore_l0(g, r, s, tid);
}

// Steps 14..1 of `stage` (> 14) for every tile.
template <typename T>
__global__ void __launch_bounds__(kRThreads, 2)
abitonic_tile_finish_r(T *data, int stage) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	T *s = reinterpret_cast<T *>(smem_raw);
	const uint32_t tid = threadIdx.x;
	const size_t tile_base = (size_t)blockIdx.x << kRLog;
	T *g = data + tile_base;
	T r[kRN];
#pragma unroll
	for (int m = 0; m < kRN; ++m) r[m] = g[lidx<9>(tid, m)];
	if ((tile_base >> stage) & 1) full_stage_uniform<true>(r, s, tid);
	else full_stage_uniform<false>(r, s, tid);
	rstore_l0(g, r, s, tid);
}

template <typename T>
__global__ void fill_value(T *p, size_t n, T v) {
	size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (i < n) p[i] = v;
}

template <typename T> T max_value();
template <> int8_t max_value<int8_t>() { return INT8_MAX; }
template <> uint8_t max_value<uint8_t>() { return UINT8_MAX; }
template <> int16_t max_value<int16_t>() { return INT16_MAX; }
template <> uint16_t max_value<uint16_t>() { return UINT16_MAX; }
template <> int32_t max_value<int32_t>() { return INT32_MAX; }
template <> uint32_t max_value<uint32_t>() { return UINT32_MAX; }
template <> int64_t max_value<int64_t>() { return INT64_MAX; }
template <> uint64_t max_value<uint64_t>() { return UINT64_MAX; }
template <> Half16 max_value<Half16>() { return Half16{0x7c00}; }  // +inf
template <> float max_value<float>() { return __builtin_huge_valf(); }
template <> double max_value<double>() { return __builtin_huge_val(); }

int ilog2(size_t v) {
	int r = 0;
	while (((size_t)1 << r) < v) ++r;
	return r;
}

// Tile exponent: 2^14 elements (<= 4-byte types) or 2^13 (8-byte), so a
// tile takes 64 KB of shared memory; capped by the abitonic maxsfs option.
template <typename T>
int default_tile_log2() {
	return sizeof(T) >= 8 ? 13 : 14;
}

template <typename T>
cudaError_t run_abitonic(T *d, size_t N, int max_ps, int max_sfs,
	cudaStream_t s, unsigned &launches) {
	const int logN = ilog2(N);
	int t = std::min(default_tile_log2<T>(), logN);
	if (max_sfs >= 1 && max_sfs < t) t = max_sfs;
	// Steps per register round: at most 4 (16 elements per thread) in the
	// shared-memory tiles; in the global passes 7 (128) for 4-byte types,
	// 6 (64) for 2-byte types and 5 (32) for 1-byte types (which spill at
	// 64) when the maxps option allows the most grouping (the network,
	// hence the result, is the same for any grouping; 5 in the tiles would
	// leave one 512-thread CTA per SM). A global pass moves the whole array
	// whatever its step count, so fewer, longer passes cut the bytes.
	const int maxg = std::max(1, std::min(4, max_ps));
	const int gmaxg = max_ps >= 4 && sizeof(T) <= 4
		? (sizeof(T) == 4 ? 7 : sizeof(T) == 2 ? 6 : 5) : maxg;
	const uint32_t tile_n = 1u << t;
	const size_t smem = (size_t)(tile_n + tile_n / 32 + 1) * sizeof(T);
	const int threads = (int)std::min<uint32_t>(kTileThreads, std::max<uint32_t>(tile_n / 2, 32));
	cudaError_t e = cudaFuncSetAttribute(abitonic_tile_sort<T>,
		cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e == cudaSuccess)
		e = cudaFuncSetAttribute(abitonic_tile_finish<T>,
			cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	const size_t tiles = N >> t;
	const double pass_bytes = 2.0 * (double)N * sizeof(T);
	// Register-phase tile kernels for full 2^14 tiles of up to 4-byte types
	// with the default grouping.
	bool rtiles = false;
	if constexpr (sizeof(T) <= 4) {
		// (16-byte vector accesses need an aligned array.)
		rtiles = t == kRLog && maxg == 4 && ((uintptr_t)d % 16) == 0;
		if (rtiles) {
			e = cudaFuncSetAttribute(abitonic_tile_sort_r<T>,
				cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e == cudaSuccess)
				e = cudaFuncSetAttribute(abitonic_tile_finish_r<T>,
					cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e != cudaSuccess) return e;
		}
	}
	{
		KernelTimer tm("abitonic_tile_sort", s, pass_bytes);
		if constexpr (sizeof(T) <= 4) {
			if (rtiles) abitonic_tile_sort_r<T><<<(unsigned)tiles, kRThreads, smem, s>>>(d);
		}
		if (!rtiles) abitonic_tile_sort<T><<<(unsigned)tiles, threads, smem, s>>>(d, t, maxg);
		tm.stop();
	}
	launches++;
	for (int stage = t + 1; stage <= logN && e == cudaSuccess; ++stage) {
		int j = stage;
		while (j > t) {
			// Balanced groups (6 steps as 3 + 3, not 5 + 1): a pass of few
			// steps per thread is the slowest per byte.
			const int rem = j - t;
			const int npass = (rem + gmaxg - 1) / gmaxg;
			int g = (rem + npass - 1) / npass;
			size_t groups = N >> g;
			unsigned blocks = (unsigned)((groups + 255) / 256);
			const unsigned blocks7 = (unsigned)((groups + 127) / 128);
			KernelTimer tm("abitonic_global_steps", s, pass_bytes);
			switch (g) {
			case 7:
				if constexpr (sizeof(T) == 4)
					abitonic_global_steps<T, 7><<<blocks7, gs_threads<7>(), 0, s>>>(d, groups, stage, j);
				break;
			case 6:
				if constexpr (sizeof(T) == 2 || sizeof(T) == 4)
					abitonic_global_steps<T, 6><<<blocks, 256, 0, s>>>(d, groups, stage, j);
				break;
			case 5: abitonic_global_steps<T, 5><<<blocks, 256, 0, s>>>(d, groups, stage, j); break;
			case 4: abitonic_global_steps<T, 4><<<blocks, 256, 0, s>>>(d, groups, stage, j); break;
			case 3: abitonic_global_steps<T, 3><<<blocks, 256, 0, s>>>(d, groups, stage, j); break;
			case 2: abitonic_global_steps<T, 2><<<blocks, 256, 0, s>>>(d, groups, stage, j); break;
			default: abitonic_global_steps<T, 1><<<blocks, 256, 0, s>>>(d, groups, stage, j); break;
			}
			tm.stop();
			launches++;
			j -= g;
		}
		KernelTimer tf("abitonic_tile_finish", s, pass_bytes);
		if constexpr (sizeof(T) <= 4) {
			if (rtiles) abitonic_tile_finish_r<T><<<(unsigned)tiles, kRThreads, smem, s>>>(d, stage);
		}
		if (!rtiles) abitonic_tile_finish<T><<<(unsigned)tiles, threads, smem, s>>>(d, t, stage, maxg);
		tf.stop();
		launches++;
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaGetLastError();
	return e;
}

template <typename T>
cudaError_t run_sbitonic(T *d, size_t N, cudaStream_t s, unsigned &launches) {
	const int logN = ilog2(N);
	const size_t half = N / 2;
	const unsigned blocks = (unsigned)((half + 255) / 256);
	for (int stage = 1; stage <= logN; ++stage)
		for (int step = stage; step >= 1; --step) {
			sbitonic_step<T><<<blocks, 256, 0, s>>>(d, half, stage, step);
			launches++;
		}
	return cudaGetLastError();
}

template <typename T>
cudaError_t bitonic_typed(void *data, size_t n, bool simple, int max_ps,
	int max_sfs, CCLContext *ctx, cudaStream_t s, GError **err) {
	if (n < 2) return cudaSuccess;
	size_t N = (size_t)1 << ilog2(n);
	T *d = (T *)data;
	T *tmp = nullptr;
	unsigned launches = 0;
	cudaError_t e = cudaSuccess;
	if (N != n) {
		tmp = (T *)tmp_alloc(ctx, N * sizeof(T), s, err);
		if (!tmp) return cudaErrorMemoryAllocation;
		e = cudaMemcpyAsync(tmp, data, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
		if (e == cudaSuccess) {
			size_t pad = N - n;
			fill_value<T><<<(unsigned)((pad + 255) / 256), 256, 0, s>>>(tmp + n, pad,
				max_value<T>());
			launches++;
			e = cudaGetLastError();
		}
		d = tmp;
	}
	if (e == cudaSuccess)
		e = simple ? run_sbitonic<T>(d, N, s, launches)
				   : run_abitonic<T>(d, N, max_ps, max_sfs, s, launches);
	if (tmp) {
		if (e == cudaSuccess)
			e = cudaMemcpyAsync(data, tmp, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
		tmp_free(tmp, s);
	}
	count_launches(launches);
	if (e != cudaSuccess) cuda_ok(e, err, simple ? "sbitonic" : "abitonic");
	return e;
}

cudaError_t bitonic_dispatch(void *data, size_t n, CloType type, bool simple,
	int max_ps, int max_sfs, CCLContext *ctx, cudaStream_t s, GError **err) {
	switch (type) {
	case CLO_CHAR: return bitonic_typed<int8_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_UCHAR: return bitonic_typed<uint8_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_SHORT: return bitonic_typed<int16_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_USHORT: return bitonic_typed<uint16_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_INT: return bitonic_typed<int32_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_UINT: return bitonic_typed<uint32_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_LONG: return bitonic_typed<int64_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_ULONG: return bitonic_typed<uint64_t>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_HALF: return bitonic_typed<Half16>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_FLOAT: return bitonic_typed<float>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	case CLO_DOUBLE: return bitonic_typed<double>(data, n, simple, max_ps, max_sfs, ctx, s, err);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported element type %d", (int)type);
	return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t bitonic_sort(void *data, size_t n, CloType type, CCLContext *ctx,
	cudaStream_t s, GError **err) {
	return bitonic_dispatch(data, n, type, false, 4, 0, ctx, s, err);
}

cudaError_t bitonic_sort_tuned(void *data, size_t n, CloType type, int max_ps,
	int max_sfs, CCLContext *ctx, cudaStream_t s, GError **err) {
	return bitonic_dispatch(data, n, type, false, max_ps, max_sfs, ctx, s, err);
}

cudaError_t bitonic_sort_simple(void *data, size_t n, CloType type,
	CCLContext *ctx, cudaStream_t s, GError **err) {
	return bitonic_dispatch(data, n, type, true, 1, 0, ctx, s, err);
}

}  // namespace clo
