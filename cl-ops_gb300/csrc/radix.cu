// "satradix": stable LSD radix sort, onesweep style, 8-bit digits.
//
// Result contract (src/cl_ops/sort/clo_sort_satradix.c:117-335 with the
// kernels of clo_sort_satradix.cl:34-258): a stable sort, ascending by the
// unsigned bit pattern of the key. The reference sorts with
// log2(radix)-bit digits; any digit width gives the same stable order, so
// the width here is a tuning choice (8 bits: 4 passes for 32-bit keys).
//
// Per sort:
//   1. radix_upsweep: one read of the keys builds the 256-bin histogram
//      of every digit position at once.
//   2. per digit position, radix_pass_chunked (one launch per pass), one
//      CTA per contiguous chunk of 4096-key tiles (2048 for 64-bit keys):
//      a. the CTA counts its chunk's digits, publishes the counts and looks
//         back over the preceding chunks once (decoupled lookback, one
//         thread per digit, bounded waits) for its digits' global offsets;
//      b. per tile, keys are loaded warp-striped (a warp's keys are in
//         index order) and ranked among equal digits of their warp, stably
//         (lanes in order, rounds in order): peers found through a
//         shared-memory OR mask, the lowest advancing the warp's counter;
//      c. keys (then values) are staged in shared memory in tile-sorted
//         order and written out so that consecutive threads write
//         consecutive addresses of a digit's run, each digit's run
//         continuing where the previous tile's ended.
// Passes whose digit has a single populated bin are skipped (the order of
// a stable sort by a constant digit is the identity).
//
// HBM roofline per 32-bit key: 4 B (upsweep) + P x 8 B (passes), i.e.
// 36 B/key for P = 4.
#include <algorithm>
#include <vector>

#include "clo_internal.h"
#include "dev_common.cuh"
#include "timing.h"

namespace clo {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;

// Tile status word: 2-bit flag | 30-bit count.
constexpr uint32_t kStAgg = 1u << 30;
constexpr uint32_t kStPrefix = 2u << 30;
constexpr uint32_t kStValue = (1u << 30) - 1u;

template <typename K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift) {
	return (uint32_t)(k >> shift) & (kRadix - 1);
}

// ----------------------------------------------------------- upsweep
// Histograms of all `passes` digit positions in one read: one shared-memory
// atomic per key and digit position, except when all 32 x PER keys of a
// warp step share the digit (sorted or constant input), which the warp
// detects with one AND/OR reduction and adds once.
template <typename K, int PASSES>
__global__ void __launch_bounds__(256)
radix_upsweep(const K *__restrict__ keys, size_t n, uint32_t *__restrict__ hist,
	int base_shift) {
	constexpr int passes = PASSES;
	__shared__ uint32_t h[PASSES][kRadix];
	for (int i = threadIdx.x; i < PASSES * kRadix; i += blockDim.x) (&h[0][0])[i] = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31;
	const size_t warp_global = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
	const size_t warps_total = ((size_t)gridDim.x * blockDim.x) >> 5;
	constexpr int PER = 16 / sizeof(K);  // keys per 16-byte load
	const bool aligned = ((uintptr_t)keys % 16) == 0;
	// Full 16-byte chunks, processed 32 per warp step with the fast path.
	const size_t full_chunks = aligned ? n / PER : 0;
	const size_t full_steps = full_chunks / 32;
	const uint4 *kv4 = reinterpret_cast<const uint4 *>(keys);
	for (size_t step = warp_global; step < full_steps; step += warps_total) {
		uint4 v = dev::ld_stream_v4(kv4 + step * 32 + lane);
		const K *e = reinterpret_cast<const K *>(&v);
#pragma unroll
		for (int p = 0; p < passes; ++p) {
			uint32_t dd[PER];
			uint32_t a = 0xffffffffu, o = 0u;
#pragma unroll
			for (int q = 0; q < PER; ++q) {
				dd[q] = digit_of(e[q], base_shift + p * kRadixBits);
				a &= dd[q];
				o |= dd[q];
			}
			uint32_t wa = __reduce_and_sync(0xffffffffu, a);
			uint32_t wo = __reduce_or_sync(0xffffffffu, o);
			if (wa == wo) {
				if (lane == 0) atomicAdd(&h[p][wa], 32u * PER);
			} else {
#pragma unroll
				for (int q = 0; q < PER; ++q) atomicAdd(&h[p][dd[q]], 1u);
			}
		}
	}
	// Remaining keys (and unaligned inputs): one key per thread.
	const size_t done = full_steps * 32 * PER;
	const size_t tid_global = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	const size_t threads_total = (size_t)gridDim.x * blockDim.x;
	for (size_t i = done + tid_global; i < n; i += threads_total) {
		K key = keys[i];
		for (int p = 0; p < passes; ++p)
			atomicAdd(&h[p][digit_of(key, base_shift + p * kRadixBits)], 1u);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) {
		uint32_t v = (&h[0][0])[i];
		if (v) atomicAdd(hist + i, v);
	}
}

// ----------------------------------------------------------- onesweep pass
struct PassArgs {
	const uint32_t *hist;   // 256 bins of this digit position
	uint32_t *status;       // num_tiles * 256 words used by this pass
	uint32_t *status_next;  // the other buffer, cleared for the next pass
	uint32_t *tile_counter;
	int *dev_status;
	size_t n;
	int shift;
};

// Lookback window: predecessor statuses read per round trip per digit.
constexpr int kLookWindow = 32;

// Threads per CTA of the chunked pass.
constexpr int kChunkThreads = 256;

// Reads the statuses of tiles base, base-1, ..., base-W+1 for one digit
// (independent loads, one round trip), adds them in order to `excl` up to
// and including the first inclusive prefix. Returns true when a prefix was
// reached; otherwise moves `base` to the first unpublished predecessor
// (or past the window).
template <int W>
__device__ __forceinline__ bool lookback_window(const uint32_t *status, int digit,
	long long &base, uint32_t &excl) {
	uint32_t sv[W];
#pragma unroll
	for (int i = 0; i < W; ++i) {
		long long j = base - i;
		sv[i] = j >= 0 ? dev::ld_relaxed_u32(status + (size_t)j * kRadix + digit)
					   : kStPrefix;
	}
	int consumed = W;
	bool done = false;
#pragma unroll
	for (int i = 0; i < W; ++i) {
		if (!done && consumed == W) {
			if ((sv[i] & ~kStValue) == 0) {
				consumed = i;
			} else {
				excl += sv[i] & kStValue;
				if (sv[i] & kStPrefix) done = true;
			}
		}
	}
	if (!done) base -= consumed;
	return done;
}


// ------------------------------------------------------- chunked pass
// One CTA per contiguous chunk of tiles (chunks claimed in order from an
// atomic counter). The CTA first counts the digit over its whole chunk
// with streaming 16-byte loads, publishes the chunk's counts and looks
// back over the preceding chunks -- one decoupled lookback per CTA and
// pass instead of one per tile, so no tile ever waits on another CTA --
// then ranks and scatters its tiles in order, each digit's run continuing
// where the previous tile's ended. The counting read costs key-size bytes
// per key on top of the pass's read and write. THREADS is 256 or 512;
// with 256 threads (4096-key tiles) four CTAs share an SM and hide each
// other's per-tile latency.
template <typename K, int THREADS>
struct ChunkCfg {
	static constexpr int kWarps = THREADS / 32;
	static constexpr int kKpt = sizeof(K) <= 4 ? 16 : 8;
	static constexpr int kTile = THREADS * kKpt;
	static constexpr int kHalves = THREADS / kRadix;          // 1 or 2
	static constexpr int kWarpsPerHalf = kWarps / kHalves;    // 8
	static constexpr int kMinBlocks = THREADS == 256 ? 4 : 2;
};

template <typename K, int THREADS>
__device__ __forceinline__ void chunk_load_keys(K (&k)[ChunkCfg<K, THREADS>::kKpt],
	const K *__restrict__ kin, size_t n, uint32_t tile, int warp, int lane) {
	constexpr int KPT = ChunkCfg<K, THREADS>::kKpt;
	const size_t wbase = (size_t)tile * ChunkCfg<K, THREADS>::kTile +
		(size_t)warp * (KPT * 32);
#pragma unroll
	for (int j = 0; j < KPT; ++j) {
		size_t idx = wbase + (size_t)j * 32 + lane;
		k[j] = idx < n ? kin[idx] : (K)~(K)0;
	}
}

template <typename K, typename V, bool HAS_V, int THREADS>
__global__ void __launch_bounds__(THREADS, ChunkCfg<K, THREADS>::kMinBlocks)
radix_pass_chunked(const K *__restrict__ kin, K *__restrict__ kout,
	const V *__restrict__ vin, V *__restrict__ vout, PassArgs a,
	uint32_t num_tiles, uint32_t num_chunks) {
	using Cfg = ChunkCfg<K, THREADS>;
	constexpr int KPT = Cfg::kKpt;
	constexpr int TILE = Cfg::kTile;
	constexpr int WARPS = Cfg::kWarps;
	constexpr int WPH = Cfg::kWarpsPerHalf;
	constexpr int kWin = kLookWindow / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	uint32_t *s_hist = reinterpret_cast<uint32_t *>(smem);   // [WARPS][256]
	uint32_t *s_match = s_hist + WARPS * kRadix;             // [WARPS][256]
	uint32_t *s_tile_off = s_match + WARPS * kRadix;         // [256]
	uint32_t *s_tile_cnt = s_tile_off + kRadix;              // [256]
	uint32_t *s_run = s_tile_cnt + kRadix;                   // [256]
	uint32_t *s_half = s_run + kRadix;                       // [2][256]
	uint32_t *s_part = s_half + 2 * kRadix;                  // [256]
	uint32_t *s_misc = s_part + kRadix;                      // [64]
	unsigned char *s_stage = reinterpret_cast<unsigned char *>(s_misc + 64);

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	uint32_t *my_hist = s_hist + warp * kRadix;
	uint32_t *my_match = s_match + warp * kRadix;
	const int shift = a.shift;
	const uint32_t lt = dev::lanemask_lt();
	const int pd = tid & (kRadix - 1), ph = tid >> 8;
	const int dw = pd >> 5;  // warp (within a half) that owns digit pd

	if (tid == 0) s_misc[0] = atomicAdd(a.tile_counter, 1u);
	for (int i = lane; i < kRadix; i += 32) {
		my_hist[i] = 0;
		my_match[i] = 0;
	}
	// Global digit base of this pass: exclusive scan of its histogram.
	if (ph == 0) {
		const uint32_t hv = a.hist[pd];
		uint32_t inc = hv;
#pragma unroll
		for (int s = 1; s < 32; s <<= 1) {
			uint32_t t = __shfl_up_sync(0xffffffffu, inc, s);
			if (lane >= s) inc += t;
		}
		if (lane == 31) s_misc[16 + dw] = inc;
		s_part[pd] = inc - hv;
	}
	__syncthreads();
	const uint32_t c = s_misc[0];
	if (c >= num_chunks) return;
	uint32_t run_init = 0;
	if (ph == 0) {
		uint32_t goff = 0;
#pragma unroll
		for (int w = 0; w < 8; ++w)
			if (w < dw) goff += s_misc[16 + w];
		run_init = s_part[pd] + goff;
	}
	const uint32_t t0 = (uint32_t)((uint64_t)c * num_tiles / num_chunks);
	const uint32_t t1 = (uint32_t)((uint64_t)(c + 1) * num_tiles / num_chunks);
	const size_t k_lo = (size_t)t0 * TILE;
	const size_t k_hi = (size_t)t1 * TILE < a.n ? (size_t)t1 * TILE : a.n;

	// Phase 1: digit counts of the whole chunk.
	{
		constexpr int PER = 16 / sizeof(K);
		const bool vec = ((uintptr_t)(kin + k_lo) % 16) == 0;
		const size_t nvec = vec ? (k_hi - k_lo) / PER : 0;
		const uint4 *src = reinterpret_cast<const uint4 *>(kin + k_lo);
#pragma unroll 4
		for (size_t i = tid; i < nvec; i += THREADS) {
			uint4 v = dev::ld_stream_v4(src + i);
			const K *e = reinterpret_cast<const K *>(&v);
#pragma unroll
			for (int q = 0; q < PER; ++q) atomicAdd(my_hist + digit_of(e[q], shift), 1u);
		}
		for (size_t i = k_lo + nvec * PER + tid; i < k_hi; i += THREADS)
			atomicAdd(my_hist + digit_of(kin[i], shift), 1u);
	}
	__syncthreads();
	if (ph == 0) {
		uint32_t cnt = 0;
#pragma unroll
		for (int w = 0; w < WARPS; ++w) cnt += s_hist[w * kRadix + pd];
		uint32_t *st = a.status + (size_t)c * kRadix + pd;
		if (c == 0) dev::st_relaxed_u32(st, kStPrefix | cnt);
		else dev::st_relaxed_u32(st, kStAgg | cnt);
		a.status_next[(size_t)c * kRadix + pd] = 0;
		uint32_t excl = 0;
		if (c > 0) {
			long long base = (long long)c - 1;
			uint32_t iter = 0;
			bool done = lookback_window<4>(a.status, pd, base, excl);
			while (!done && base >= 0) {
				uint32_t sv = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
				while ((sv & ~kStValue) == 0) {
					if (++iter >= dev::kSpinLimit) break;
					dev::backoff(iter);
					sv = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
				}
				if ((sv & ~kStValue) == 0) {
					dev::report_timeout(a.dev_status, DEV_ERR_LOOKBACK_TIMEOUT, (int)c);
					break;
				}
				done = lookback_window<kWin>(a.status, pd, base, excl);
			}
			dev::st_relaxed_u32(st, kStPrefix | (excl + cnt));
		}
		s_run[pd] = run_init;
		s_tile_cnt[pd] = excl;  // the first tile's run starts after excl
	}
	__syncthreads();

	// Phase 2: tiles of the chunk in order.
	K k[KPT];
	if (t0 < t1) chunk_load_keys<K, THREADS>(k, kin, a.n, t0, warp, lane);
	for (uint32_t t = t0; t < t1; ++t) {
		for (int i = lane; i < kRadix; i += 32) my_hist[i] = 0;
		__syncwarp();
#pragma unroll
		for (int j = 0; j < KPT; ++j) atomicAdd(my_hist + digit_of(k[j], shift), 1u);
		__syncthreads();
		// Warp prefixes per digit: thread (pd, ph) takes warps
		// WPH*ph .. WPH*ph + WPH - 1 with independent loads.
		uint32_t cw[WPH];
#pragma unroll
		for (int i = 0; i < WPH; ++i) cw[i] = s_hist[(WPH * ph + i) * kRadix + pd];
		uint32_t run = 0;
#pragma unroll
		for (int i = 0; i < WPH; ++i) {
			uint32_t tmp = cw[i];
			cw[i] = run;
			run += tmp;
		}
		uint32_t sum = run;
		if (Cfg::kHalves == 2) {
			s_half[ph * kRadix + pd] = run;
			__syncthreads();
			const uint32_t lo = s_half[pd];
			sum = lo + s_half[kRadix + pd];
			if (ph == 1) {
#pragma unroll
				for (int i = 0; i < WPH; ++i) cw[i] += lo;
			}
		}
		if (ph == 0) {
			// Advance the run by the previous tile's count (or the lookback).
			s_run[pd] += s_tile_cnt[pd];
			s_tile_cnt[pd] = sum;
			uint32_t inc = sum;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				uint32_t tt = __shfl_up_sync(0xffffffffu, inc, d);
				if (lane >= d) inc += tt;
			}
			if (lane == 31) s_misc[8 + dw] = inc;
			s_part[pd] = inc - sum;
		}
		__syncthreads();
		{
			uint32_t woff = 0;
#pragma unroll
			for (int w = 0; w < 8; ++w)
				if (w < dw) woff += s_misc[8 + w];
			const uint32_t to = s_part[pd] + woff;
#pragma unroll
			for (int i = 0; i < WPH; ++i) s_hist[(WPH * ph + i) * kRadix + pd] = to + cw[i];
			// Output index of staged position q of digit d is q + G[d]
			// (modulo 2^32), G[d] = global run start - tile offset.
			if (ph == 0) s_tile_off[pd] = s_run[pd] - to;
		}
		__syncthreads();
		K *sk = reinterpret_cast<K *>(s_stage);
		uint32_t tpos[HAS_V ? KPT : 1];
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			const uint32_t pos = dev::warp_rank_digit(my_match, my_hist,
				digit_of(k[j], shift), lane, lt);
			if (pos < (uint32_t)TILE) sk[pos] = k[j];
			if (HAS_V) tpos[j] = pos;
		}
		__syncthreads();
		if (!HAS_V && t + 1 < t1) chunk_load_keys<K, THREADS>(k, kin, a.n, t + 1, warp, lane);
		uint32_t outpos[HAS_V ? KPT : 1];
#pragma unroll
		for (int i = 0; i < KPT; ++i) {
			const int q = i * THREADS + tid;
			const K key = sk[q];
			const size_t o = (uint32_t)(s_tile_off[digit_of(key, shift)] + (uint32_t)q);
			if (o < a.n) kout[o] = key;
			if (HAS_V) outpos[i] = (uint32_t)o;
		}
		if (HAS_V) {
			V v[KPT];
			const size_t wbase = (size_t)t * TILE + (size_t)warp * (KPT * 32);
#pragma unroll
			for (int j = 0; j < KPT; ++j) {
				size_t idx = wbase + (size_t)j * 32 + lane;
				v[j] = idx < a.n ? vin[idx] : (V)0;
			}
			__syncthreads();
			V *sv = reinterpret_cast<V *>(s_stage);
#pragma unroll
			for (int j = 0; j < KPT; ++j)
				if (tpos[j] < (uint32_t)TILE) sv[tpos[j]] = v[j];
			__syncthreads();
#pragma unroll
			for (int i = 0; i < KPT; ++i) {
				const int q = i * THREADS + tid;
				if (outpos[i] < a.n) vout[outpos[i]] = sv[q];
			}
			if (t + 1 < t1) chunk_load_keys<K, THREADS>(k, kin, a.n, t + 1, warp, lane);
			__syncthreads();
		}
	}
}

template <typename K, typename V, bool HAS_V, int THREADS>
size_t chunked_smem() {
	constexpr int TILE = ChunkCfg<K, THREADS>::kTile;
	size_t stage = (size_t)TILE * (sizeof(K) > sizeof(V) || !HAS_V ? sizeof(K) : sizeof(V));
	return (2 * ChunkCfg<K, THREADS>::kWarps * kRadix + 7 * kRadix + 64) * sizeof(uint32_t) +
		stage;
}

template <typename K>
void launch_upsweep(int passes, int grid, cudaStream_t s, const K *keys, size_t n,
	uint32_t *hist, int base_shift = 0) {
	switch (passes) {
	case 1: radix_upsweep<K, 1><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 2: radix_upsweep<K, 2><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 3: radix_upsweep<K, 3><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 4: radix_upsweep<K, 4><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 5: radix_upsweep<K, 5><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 6: radix_upsweep<K, 6><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	case 7: radix_upsweep<K, 7><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	default: radix_upsweep<K, 8><<<grid, 256, 0, s>>>(keys, n, hist, base_shift); break;
	}
}

template <typename K, typename V, bool HAS_V>
cudaError_t sort_typed(void *keys, void *vals, size_t n, int sort_bits,
	CCLContext *ctx, cudaStream_t s, bool allow_skip, GError **err) {
	const int passes = sort_bits / kRadixBits;
	if (n < 2 || passes == 0) return cudaSuccess;
	if (n >= (size_t)kStValue) {
		set_error(err, CLO_ERROR_ARGS,
			"satradix: %zu elements exceed the single-sort limit of 2^30 - 1", n);
		return cudaErrorInvalidValue;
	}
	// The chunked pass: tiles of ChunkCfg size, one chunk per CTA.
	constexpr int CT = kChunkThreads;
	constexpr int CTILE = ChunkCfg<K, CT>::kTile;
	const size_t ctiles = (n + CTILE - 1) / CTILE;
	const uint32_t chunks = (uint32_t)std::min<size_t>(ctiles,
		(size_t)ChunkCfg<K, CT>::kMinBlocks * ctx->sm_count);
	// Status slots: one per chunk.
	const size_t status_words = (size_t)chunks * kRadix;
	// Scratch: [hist passes*256][counters 8][status0][status1][alt keys][alt vals]
	size_t off_hist = 0;
	size_t off_cnt = off_hist + (size_t)passes * kRadix * 4;
	size_t off_st0 = off_cnt + 8 * 4;
	size_t off_st1 = off_st0 + status_words * 4;
	size_t off_keys = (off_st1 + status_words * 4 + 255) / 256 * 256;
	size_t off_vals = (off_keys + n * sizeof(K) + 255) / 256 * 256;
	size_t total = off_vals + (HAS_V ? n * sizeof(V) : 0);
	char *tmp = (char *)tmp_alloc(ctx, total, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	uint32_t *hist = (uint32_t *)(tmp + off_hist);
	uint32_t *cnt = (uint32_t *)(tmp + off_cnt);
	uint32_t *st[2] = {(uint32_t *)(tmp + off_st0), (uint32_t *)(tmp + off_st1)};
	K *alt_k = (K *)(tmp + off_keys);
	V *alt_v = (V *)(tmp + off_vals);
	cudaError_t e = cudaMemsetAsync(tmp, 0, off_st1, s);
	unsigned launches = 0;
	if (e == cudaSuccess) {
		int grid = ctx->sm_count * 4;
		size_t chunks = (n * sizeof(K) + 15) / 16;
		size_t need = (chunks + 255) / 256;
		if ((size_t)grid > need) grid = (int)std::max<size_t>(need, 1);
		KernelTimer t("satradix_upsweep", s, (double)n * sizeof(K));
		launch_upsweep<K>(passes, grid, s, (const K *)keys, n, hist);
		t.stop();
		launches++;
		e = cudaGetLastError();
	}
	std::vector<int> active;
	if (e == cudaSuccess) {
		if (allow_skip && n >= (1u << 16)) {
			std::vector<uint32_t> h((size_t)passes * kRadix);
			e = cudaMemcpyAsync(h.data(), hist, h.size() * 4, cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaStreamSynchronize(s);
			for (int p = 0; p < passes && e == cudaSuccess; ++p) {
				bool trivial = false;
				for (int d = 0; d < kRadix; ++d)
					if (h[(size_t)p * kRadix + d] == n) trivial = true;
				if (!trivial) active.push_back(p);
			}
		} else {
			for (int p = 0; p < passes; ++p) active.push_back(p);
		}
	}
	if (e == cudaSuccess) {
		const size_t smem = chunked_smem<K, V, HAS_V, CT>();
		auto kern = radix_pass_chunked<K, V, HAS_V, CT>;
		e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
			(int)smem);
		K *src_k = (K *)keys, *dst_k = alt_k;
		V *src_v = (V *)vals, *dst_v = alt_v;
		for (size_t q = 0; q < active.size() && e == cudaSuccess; ++q) {
			PassArgs pa;
			pa.hist = hist + (size_t)active[q] * kRadix;
			pa.status = st[q & 1];
			pa.status_next = st[(q + 1) & 1];
			pa.tile_counter = cnt + active[q];
			pa.dev_status = ctx->d_status;
			pa.n = n;
			pa.shift = active[q] * kRadixBits;
			KernelTimer t("satradix_onesweep", s,
				2.0 * (double)n * (sizeof(K) + (HAS_V ? sizeof(V) : 0)));
			kern<<<chunks, CT, smem, s>>>(src_k, dst_k, src_v, dst_v, pa,
				(uint32_t)ctiles, chunks);
			t.stop();
			launches++;
			e = cudaGetLastError();
			std::swap(src_k, dst_k);
			std::swap(src_v, dst_v);
		}
		if (e == cudaSuccess && (active.size() & 1)) {
			e = cudaMemcpyAsync(keys, alt_k, n * sizeof(K), cudaMemcpyDeviceToDevice, s);
			if (e == cudaSuccess && HAS_V)
				e = cudaMemcpyAsync(vals, alt_v, n * sizeof(V), cudaMemcpyDeviceToDevice, s);
		}
	}
	count_launches(launches);
	tmp_free(tmp, s);
	if (e != cudaSuccess) cuda_ok(e, err, "satradix");
	return e;
}

// Stable partition of n keys by the top 8 of their sort_bits low bits:
// keys_out receives the keys grouped by that digit, in input order within a
// digit; counts (host) receives the 256 group sizes. One histogram kernel
// for the digit, a host readback of its 256 counts, one chunked pass.
template <typename K>
cudaError_t msd_partition_typed(const K *keys_in, K *keys_out, size_t n, int sort_bits,
	uint32_t *counts, CCLContext *ctx, cudaStream_t s, GError **err) {
	constexpr int CT = kChunkThreads;
	constexpr int CTILE = ChunkCfg<K, CT>::kTile;
	const int shift = sort_bits - kRadixBits;
	const size_t ctiles = (n + CTILE - 1) / CTILE;
	const uint32_t chunks = (uint32_t)std::min<size_t>(ctiles,
		(size_t)ChunkCfg<K, CT>::kMinBlocks * ctx->sm_count);
	const size_t status_words = (size_t)chunks * kRadix;
	const size_t off_cnt = kRadix * 4, off_st0 = off_cnt + 64;
	const size_t off_st1 = off_st0 + status_words * 4;
	char *tmp = (char *)tmp_alloc(ctx, off_st1 + status_words * 4, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	uint32_t *hist = (uint32_t *)tmp;
	uint32_t *cnt = (uint32_t *)(tmp + off_cnt);
	cudaError_t e = cudaMemsetAsync(tmp, 0, off_st1, s);
	if (e == cudaSuccess) {
		int grid = ctx->sm_count * 4;
		const size_t need = ((n * sizeof(K) + 15) / 16 + 255) / 256;
		if ((size_t)grid > need) grid = (int)std::max<size_t>(need, 1);
		KernelTimer t("satradix_upsweep", s, (double)n * sizeof(K));
		launch_upsweep<K>(1, grid, s, keys_in, n, hist, shift);
		t.stop();
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(counts, hist, kRadix * 4, cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	bool trivial = false;
	for (int d = 0; d < kRadix && e == cudaSuccess; ++d) trivial = trivial || counts[d] == n;
	if (e == cudaSuccess && trivial) {
		e = cudaMemcpyAsync(keys_out, keys_in, n * sizeof(K), cudaMemcpyDeviceToDevice, s);
	} else if (e == cudaSuccess) {
		const size_t smem = chunked_smem<K, uint32_t, false, CT>();
		auto kern = radix_pass_chunked<K, uint32_t, false, CT>;
		e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		PassArgs pa;
		pa.hist = hist;
		pa.status = (uint32_t *)(tmp + off_st0);
		pa.status_next = (uint32_t *)(tmp + off_st1);
		pa.tile_counter = cnt;
		pa.dev_status = ctx->d_status;
		pa.n = n;
		pa.shift = shift;
		if (e == cudaSuccess) {
			KernelTimer t("satradix_onesweep", s, 2.0 * (double)n * sizeof(K));
			kern<<<chunks, CT, smem, s>>>(keys_in, keys_out, nullptr, nullptr, pa,
				(uint32_t)ctiles, chunks);
			t.stop();
			e = cudaGetLastError();
		}
	}
	count_launches(trivial ? 1 : 2);
	tmp_free(tmp, s);
	if (e != cudaSuccess) cuda_ok(e, err, "satradix partition");
	return e;
}

template <typename K>
cudaError_t sort_keys_vals(void *keys, void *vals, size_t n, int val_bytes,
	int sort_bits, CCLContext *ctx, cudaStream_t s, bool skip, GError **err) {
	switch (val_bytes) {
	case 0: return sort_typed<K, uint32_t, false>(keys, nullptr, n, sort_bits, ctx, s, skip, err);
	case 4: return sort_typed<K, uint32_t, true>(keys, vals, n, sort_bits, ctx, s, skip, err);
	case 8: return sort_typed<K, uint64_t, true>(keys, vals, n, sort_bits, ctx, s, skip, err);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported value width %d", val_bytes);
	return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t radix_msd_partition(const void *keys_in, void *keys_out, size_t n, int key_bytes,
	int sort_bits, uint32_t *counts, CCLContext *ctx, cudaStream_t s, GError **err) {
	if (sort_bits < kRadixBits || n >= (size_t)kStValue) {
		set_error(err, CLO_ERROR_ARGS, "satradix partition: %d sort bits, %zu keys", sort_bits, n);
		return cudaErrorInvalidValue;
	}
	switch (key_bytes) {
	case 2: return msd_partition_typed<uint16_t>((const uint16_t *)keys_in, (uint16_t *)keys_out, n, sort_bits, counts, ctx, s, err);
	case 4: return msd_partition_typed<uint32_t>((const uint32_t *)keys_in, (uint32_t *)keys_out, n, sort_bits, counts, ctx, s, err);
	case 8: return msd_partition_typed<uint64_t>((const uint64_t *)keys_in, (uint64_t *)keys_out, n, sort_bits, counts, ctx, s, err);
	}
	set_error(err, CLO_ERROR_ARGS, "satradix partition: key width %d", key_bytes);
	return cudaErrorInvalidValue;
}

cudaError_t radix_sort(void *keys, void *vals, size_t n, int key_bytes,
	int val_bytes, int sort_bits, CCLContext *ctx, cudaStream_t s,
	bool allow_skip, GError **err) {
	switch (key_bytes) {
	case 1: return sort_keys_vals<uint8_t>(keys, vals, n, val_bytes, sort_bits, ctx, s, allow_skip, err);
	case 2: return sort_keys_vals<uint16_t>(keys, vals, n, val_bytes, sort_bits, ctx, s, allow_skip, err);
	case 4: return sort_keys_vals<uint32_t>(keys, vals, n, val_bytes, sort_bits, ctx, s, allow_skip, err);
	case 8: return sort_keys_vals<uint64_t>(keys, vals, n, val_bytes, sort_bits, ctx, s, allow_skip, err);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported key width %d", key_bytes);
	return cudaErrorInvalidValue;
}

}  // namespace clo
