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
//      b. per tile, keys are loaded in half-warp units (a unit's keys are
//         in index order) and ranked among equal digits of their unit,
//         stably (lanes in order, rounds in order): peers found through a
//         shared-memory OR mask in the low half of the unit's word for the
//         digit, whose high half holds the unit's next position;
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
// Histograms of all `passes` digit positions in one read. Up to four
// positions count into lane columns: the (d & 1) 16-bit half of word
// (d >> 1) * 32 + lane per position, shared by the CTA's warps through
// atomics, so a warp's 32 increments hit 32 different banks; more positions
// count into one 256-bin row per warp and position. Each thread keeps
// kUpsweepInFlight 16-byte loads in flight.
//
// A column half receives at most kWarps x (keys per thread) increments;
// the grid is sized so that a thread sees at most kUpsweepKeysPerThread
// keys (8 x (4096 + 16) < 2^16).
constexpr int kUpsweepThreads = 256;
constexpr size_t kUpsweepKeysPerThread = 4096;
constexpr int kUpsweepColumnPasses = 4;  // most positions counted in columns
constexpr int kUpsweepInFlight = 8;

template <int PASSES>
constexpr size_t upsweep_smem() {
	return PASSES <= kUpsweepColumnPasses ? (size_t)PASSES * (kRadix / 2) * 32 * 4
										  : (size_t)PASSES * (kUpsweepThreads / 32) * kRadix * 4;
}

template <typename K, int PASSES>
__global__ void __launch_bounds__(kUpsweepThreads)
radix_upsweep(const K *__restrict__ keys, size_t n, uint32_t *__restrict__ hist,
	int base_shift) {
	constexpr bool COLS = PASSES <= kUpsweepColumnPasses;
	constexpr int kWarps = kUpsweepThreads / 32;
	constexpr int kPosWords = COLS ? (kRadix / 2) * 32 : kWarps * kRadix;
	extern __shared__ __align__(16) uint32_t up_smem[];
	for (int i = threadIdx.x; i < PASSES * kPosWords; i += kUpsweepThreads) up_smem[i] = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t *base = COLS ? up_smem + lane : up_smem + warp * kRadix;
	auto count = [&](int p, K key) {
		const uint32_t d = digit_of(key, base_shift + p * kRadixBits);
		if (COLS) atomicAdd(base + p * kPosWords + (d >> 1) * 32, 1u << ((d & 1) << 4));
		else atomicAdd(base + p * kPosWords + d, 1u);
	};
	// 32-bit keys at shift 0 with four positions: the four column rows
	// (d >> 1) and half selectors (d & 1) come out of two word-wide masks,
	// then one byte extract, one address add and the atomic per position.
	auto count4 = [&](uint32_t key) {
		const uint32_t rows = (key >> 1) & 0x7F7F7F7Fu;
		const uint32_t halves = (key & 0x01010101u) << 4;  // 0 or 16 per byte
#pragma unroll
		for (int p = 0; p < 4; ++p) {
			const uint32_t row = __byte_perm(rows, 0, 0x4440 + p);
			const uint32_t sh = __byte_perm(halves, 0, 0x4440 + p);
			atomicAdd(base + p * kPosWords + row * 32, 1u << sh);
		}
	};
	constexpr bool kFast4 = COLS && PASSES == 4 && sizeof(K) == 4;
	constexpr int PER = 16 / sizeof(K);  // keys per 16-byte load
	const bool aligned = ((uintptr_t)keys % 16) == 0;
	const size_t nvec = aligned ? n / PER : 0;
	const uint4 *kv4 = reinterpret_cast<const uint4 *>(keys);
	const size_t stride = (size_t)gridDim.x * kUpsweepThreads;
	size_t i = blockIdx.x * (size_t)kUpsweepThreads + threadIdx.x;
	for (; i + (kUpsweepInFlight - 1) * stride < nvec; i += kUpsweepInFlight * stride) {
		uint4 v[kUpsweepInFlight];
#pragma unroll
		for (int u = 0; u < kUpsweepInFlight; ++u) v[u] = dev::ld_stream_v4(kv4 + i + u * stride);
#pragma unroll
		for (int u = 0; u < kUpsweepInFlight; ++u) {
			const K *e = reinterpret_cast<const K *>(&v[u]);
			if (kFast4 && base_shift == 0) {
#pragma unroll
				for (int q = 0; q < PER; ++q) count4((uint32_t)e[q]);
			} else {
#pragma unroll
				for (int p = 0; p < PASSES; ++p)
#pragma unroll
					for (int q = 0; q < PER; ++q) count(p, e[q]);
			}
		}
	}
	for (; i < nvec; i += stride) {
		uint4 v = dev::ld_stream_v4(kv4 + i);
		const K *e = reinterpret_cast<const K *>(&v);
#pragma unroll
		for (int p = 0; p < PASSES; ++p)
#pragma unroll
			for (int q = 0; q < PER; ++q) count(p, e[q]);
	}
	// Remaining keys (and unaligned inputs): one key per thread.
	for (size_t j = nvec * PER + blockIdx.x * (size_t)kUpsweepThreads + threadIdx.x; j < n;
		 j += stride) {
		const K key = keys[j];
#pragma unroll
		for (int p = 0; p < PASSES; ++p) count(p, key);
	}
	__syncthreads();
	for (int b = threadIdx.x; b < PASSES * kRadix; b += kUpsweepThreads) {
		const int p = b / kRadix, d = b % kRadix;
		uint32_t v = 0;
		if (COLS) {
			// Digit d's 32 column halves, from a rotated start (no conflicts).
			const uint32_t *row = up_smem + p * kPosWords + (d >> 1) * 32;
			const int hs = (d & 1) << 4;
#pragma unroll 8
			for (int c = 0; c < 32; ++c) v += (row[(c + lane) & 31] >> hs) & 0xFFFFu;
		} else {
#pragma unroll
			for (int w = 0; w < kWarps; ++w) v += up_smem[p * kPosWords + w * kRadix + d];
		}
		if (v) atomicAdd(hist + b, v);
	}
}

// ----------------------------------------------------------- onesweep pass
struct PassArgs {
	const uint32_t *hist;   // 256 bins of this digit position
	uint32_t *status;       // chunks * 256 words used by this pass
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
// per key on top of the pass's read and write. With 256 threads
// (4096-key tiles) four CTAs share an SM and hide each other's per-tile
// latency.
//
// Shared-memory work per key is what bounds the pass, so both counting
// steps and the ranking are built to touch few shared words:
//  - phase 1 counts into lane columns: digit d of lane l is the (d & 1)
//    16-bit half of word (d >> 1) * 32 + l, shared by the CTA's warps
//    through atomics. A warp's 32 increments hit 32 different banks.
//  - phase 2 ranks in half-warp units (16 lanes, KPT rounds): the unit's
//    word for digit d holds the unit's next tile position for d in its
//    upper half and the round's peer mask in its lower half, so a round is
//    one OR, one read and one store by the lowest peer.
template <typename K, int THREADS>
struct ChunkCfg {
	static_assert(THREADS == kRadix, "one thread per digit in the per-tile scans");
	static constexpr int kWarps = THREADS / 32;
	static constexpr int kUnits = 2 * kWarps;          // half-warp ranking units
	static constexpr int kKpt = sizeof(K) <= 4 ? 16 : 8;
	static constexpr int kUnitKeys = 16 * kKpt;        // a unit's keys in one tile
	static constexpr int kTile = THREADS * kKpt;
	// Largest chunk: a lane-column counter half receives at most kWarps x
	// (keys per thread) = kWarps x (2^20 / THREADS + 4) < 2^16 increments.
	static constexpr size_t kMaxChunkKeys = (size_t)1 << 20;
};

// Chunks (CTAs) of a pass over ctiles tiles: one per resident CTA
// (per_sm x SMs), more when the chunks would exceed kMaxChunkKeys.
template <typename K>
uint32_t chunk_count(size_t ctiles, int sm_count, int per_sm) {
	using Cfg = ChunkCfg<K, kChunkThreads>;
	constexpr size_t kMaxTiles = Cfg::kMaxChunkKeys / Cfg::kTile;
	const size_t c = std::max<size_t>((size_t)std::max(per_sm, 1) * sm_count,
		(ctiles + kMaxTiles - 1) / kMaxTiles);
	return (uint32_t)std::max<size_t>(std::min(c, ctiles), 1);
}

// Ranking and count rows: 256 digits each, 264 words apart, odd rows 8
// words later, so rows 2w and 2w + 1 (the two units of warp w) hold a digit
// 16 banks apart and a digit both halves of a warp hold does not conflict.
constexpr int kRowWords = kRadix + 8;
__device__ __forceinline__ int row_of(int r) { return r * kRowWords + (r & 1) * 8; }

// Keys of one unit in a tile, round-major: round j of lane l holds key
// ubase + 16 j + l, so the unit's (round, lane) order is index order.
template <typename K, int THREADS>
__device__ __forceinline__ void chunk_load_keys(K (&k)[ChunkCfg<K, THREADS>::kKpt],
	const K *__restrict__ kin, size_t n, uint32_t tile, int unit, int l16) {
	using Cfg = ChunkCfg<K, THREADS>;
	const size_t ubase = (size_t)tile * Cfg::kTile + (size_t)unit * Cfg::kUnitKeys;
#pragma unroll
	for (int j = 0; j < Cfg::kKpt; ++j) {
		size_t idx = ubase + (size_t)j * 16 + l16;
		k[j] = idx < n ? kin[idx] : (K)~(K)0;
	}
}

// Values of one unit in a tile, in the keys' layout.
template <typename K, typename V, int THREADS>
__device__ __forceinline__ void chunk_load_vals(V (&v)[ChunkCfg<K, THREADS>::kKpt],
	const V *__restrict__ vin, size_t n, uint32_t tile, int unit, int l16) {
	using Cfg = ChunkCfg<K, THREADS>;
	const size_t ubase = (size_t)tile * Cfg::kTile + (size_t)unit * Cfg::kUnitKeys;
#pragma unroll
	for (int j = 0; j < Cfg::kKpt; ++j) {
		size_t idx = ubase + (size_t)j * 16 + l16;
		v[j] = idx < n ? vin[idx] : (V)0;
	}
}

template <typename K, typename V, bool HAS_V, int THREADS>
constexpr size_t chunked_smem() {
	using Cfg = ChunkCfg<K, THREADS>;
	return ((Cfg::kUnits + Cfg::kUnits / 2) * kRowWords + 4 * kRadix + 64) * sizeof(uint32_t) +
		(size_t)Cfg::kTile * (sizeof(K) + (HAS_V ? sizeof(V) : 0));
}

// Resident CTAs per SM the pass is compiled for: four for keys only, three
// with values (keys and values of a tile stay in registers), fewer when
// the shared memory (228 KB per SM, 1 KB reserved per CTA) allows fewer.
template <typename K, typename V, bool HAS_V, int THREADS>
constexpr int chunked_min_blocks() {
	constexpr int by_smem = (int)((228 * 1024) / (chunked_smem<K, V, HAS_V, THREADS>() + 1024));
	constexpr int want = HAS_V ? 3 : 4;
	return by_smem < want ? by_smem : want;
}

template <typename K, typename V, bool HAS_V, int THREADS>
__global__ void __launch_bounds__(THREADS, (chunked_min_blocks<K, V, HAS_V, THREADS>()))
radix_pass_chunked(const K *__restrict__ kin, K *__restrict__ kout,
	const V *__restrict__ vin, V *__restrict__ vout, PassArgs a,
	uint32_t num_tiles, uint32_t num_chunks) {
	using Cfg = ChunkCfg<K, THREADS>;
	constexpr int KPT = Cfg::kKpt;
	constexpr int TILE = Cfg::kTile;
	constexpr int UNITS = Cfg::kUnits;
	constexpr int HALF = UNITS / 2;
	constexpr int kWin = kLookWindow / 2;
	extern __shared__ __align__(16) unsigned char smem[];
	// Ranking rows of units and count rows, kRowWords apart (row_of).
	uint32_t *s_rank = reinterpret_cast<uint32_t *>(smem);   // [UNITS] rows
	uint32_t *s_cnt = s_rank + UNITS * kRowWords;            // [HALF] rows
	uint32_t *s_tile_off = s_cnt + HALF * kRowWords;         // [256]
	uint32_t *s_tile_cnt = s_tile_off + kRadix;              // [256]
	uint32_t *s_run = s_tile_cnt + kRadix;                   // [256]
	uint32_t *s_part = s_run + kRadix;                       // [256]
	uint32_t *s_misc = s_part + kRadix;                      // [64]
	unsigned char *s_stage = reinterpret_cast<unsigned char *>(s_misc + 64);
	// Phase 1 only: [128][32] lane-column counters over s_rank.
	uint32_t *s_col = s_rank;
	static_assert(UNITS * kRowWords >= (kRadix / 2) * 32, "column counters fit");

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int unit = 2 * warp + (lane >> 4);
	const uint32_t l16 = lane & 15;
	const uint32_t lt16 = (1u << l16) - 1u;
	uint32_t *my_rank = s_rank + row_of(unit);
	// Tile counts: units u and u + HALF share row u % HALF (16-bit halves).
	uint32_t *my_cnt = s_cnt + row_of(unit % HALF);
	const uint32_t cnt_inc = 1u << ((unit / HALF) * 16);
	const int shift = a.shift;
	const int pd = tid;        // the digit this thread scans
	const int dw = pd >> 5;    // the warp that owns digit pd

	if (tid == 0) s_misc[0] = atomicAdd(a.tile_counter, 1u);
	for (int i = tid; i < (kRadix / 2) * 32; i += THREADS) s_col[i] = 0;
#pragma unroll
	for (int i = 0; i < HALF; ++i) s_cnt[row_of(i) + pd] = 0;
	// Global digit base of this pass: exclusive scan of its histogram.
	{
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
	uint32_t run_init;
	{
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

	// Phase 1: digit counts of the whole chunk, in lane columns.
	{
		constexpr int PER = 16 / sizeof(K);
		uint32_t *col = s_col + lane;
		const bool vec = ((uintptr_t)(kin + k_lo) % 16) == 0;
		const size_t nvec = vec ? (k_hi - k_lo) / PER : 0;
		const uint4 *src = reinterpret_cast<const uint4 *>(kin + k_lo);
		constexpr int kIn = 4;  // 16-byte loads in flight per thread
		size_t i = tid;
		for (; i + (kIn - 1) * THREADS < nvec; i += kIn * THREADS) {
			uint4 v[kIn];
#pragma unroll
			for (int u = 0; u < kIn; ++u) v[u] = dev::ld_stream_v4(src + i + u * THREADS);
#pragma unroll
			for (int u = 0; u < kIn; ++u) {
				const K *e = reinterpret_cast<const K *>(&v[u]);
#pragma unroll
				for (int q = 0; q < PER; ++q) {
					const uint32_t d = digit_of(e[q], shift);
					atomicAdd(col + (d >> 1) * 32, 1u << ((d & 1) << 4));
				}
			}
		}
		for (; i < nvec; i += THREADS) {
			uint4 v = dev::ld_stream_v4(src + i);
			const K *e = reinterpret_cast<const K *>(&v);
#pragma unroll
			for (int q = 0; q < PER; ++q) {
				const uint32_t d = digit_of(e[q], shift);
				atomicAdd(col + (d >> 1) * 32, 1u << ((d & 1) << 4));
			}
		}
		for (size_t i = k_lo + nvec * PER + tid; i < k_hi; i += THREADS) {
			const uint32_t d = digit_of(kin[i], shift);
			atomicAdd(col + (d >> 1) * 32, 1u << ((d & 1) << 4));
		}
	}
	__syncthreads();
	{
		// Sum digit pd's 32 column halves (rotated start: no bank conflicts).
		const uint32_t *row = s_col + (pd >> 1) * 32;
		const int hs = (pd & 1) << 4;
		uint32_t cnt = 0;
#pragma unroll 8
		for (int i = 0; i < 32; ++i) cnt += (row[(i + lane) & 31] >> hs) & 0xFFFFu;
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
	V v[HAS_V ? KPT : 1];
	if (t0 < t1) {
		chunk_load_keys<K, THREADS>(k, kin, a.n, t0, unit, l16);
		if constexpr (HAS_V) chunk_load_vals<K, V, THREADS>(v, vin, a.n, t0, unit, l16);
	}
	for (uint32_t t = t0; t < t1; ++t) {
#pragma unroll
		for (int j = 0; j < KPT; ++j) atomicAdd(my_cnt + digit_of(k[j], shift), cnt_inc);
		__syncthreads();
		// Unit prefixes of digit pd in unit order (rows' low halves are
		// units 0..HALF-1, high halves units HALF..UNITS-1); the rows are
		// cleared for the next tile as they are read.
		uint32_t c2[HALF];
#pragma unroll
		for (int i = 0; i < HALF; ++i) {
			c2[i] = s_cnt[row_of(i) + pd];
			s_cnt[row_of(i) + pd] = 0;
		}
		uint32_t run = 0;
#pragma unroll
		for (int i = 0; i < HALF; ++i) {
			const uint32_t lo = c2[i] & 0xFFFFu;
			c2[i] = (c2[i] & 0xFFFF0000u) | run;
			run += lo;
		}
#pragma unroll
		for (int i = 0; i < HALF; ++i) {
			const uint32_t hi = c2[i] >> 16;
			c2[i] = (c2[i] & 0xFFFFu) | (run << 16);
			run += hi;
		}
		const uint32_t sum = run;
		// Advance the run by the previous tile's count (or the lookback).
		s_run[pd] += s_tile_cnt[pd];
		s_tile_cnt[pd] = sum;
		{
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
			for (int i = 0; i < HALF; ++i) {
				s_rank[row_of(i) + pd] = (to + (c2[i] & 0xFFFFu)) << 16;
				s_rank[row_of(i + HALF) + pd] = (to + (c2[i] >> 16)) << 16;
			}
			// Output index of staged position q of digit d is q + G[d]
			// (modulo 2^32), G[d] = global run start - tile offset.
			s_tile_off[pd] = s_run[pd] - to;
		}
		__syncthreads();
		K *sk = reinterpret_cast<K *>(s_stage);
		V *sv = reinterpret_cast<V *>(s_stage + (size_t)TILE * sizeof(K));
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			const uint32_t pos = dev::unit_rank_digit(my_rank + digit_of(k[j], shift), l16, lt16);
			if (pos < (uint32_t)TILE) {
				sk[pos] = k[j];
				if (HAS_V) sv[pos] = v[j];
			}
		}
		__syncthreads();
		if (t + 1 < t1) {
			chunk_load_keys<K, THREADS>(k, kin, a.n, t + 1, unit, l16);
			if constexpr (HAS_V) chunk_load_vals<K, V, THREADS>(v, vin, a.n, t + 1, unit, l16);
		}
#pragma unroll
		for (int i = 0; i < KPT; ++i) {
			const int q = i * THREADS + tid;
			const K key = sk[q];
			const size_t o = (uint32_t)(s_tile_off[digit_of(key, shift)] + (uint32_t)q);
			if (o < a.n) {
				kout[o] = key;
				if (HAS_V) vout[o] = sv[q];
			}
		}
	}
}


template <typename K, int PASSES>
void launch_upsweep_p(cudaStream_t s, const K *keys, size_t n, uint32_t *hist,
	int base_shift, int sm_count) {
	constexpr size_t smem = upsweep_smem<PASSES>();
	auto kern = radix_upsweep<K, PASSES>;
	if (smem > 48 * 1024)
		cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	// Resident CTAs per SM by shared memory (228 KB per SM, 1 KB reserved
	// per CTA), at most 4; at least enough CTAs for the per-thread key cap.
	const int per_sm = (int)std::min<size_t>(4, (228 * 1024) / (smem + 1024));
	size_t grid = (size_t)sm_count * std::max(per_sm, 1);
	const size_t need = ((n * sizeof(K) + 15) / 16 + kUpsweepThreads - 1) / kUpsweepThreads;
	if (grid > need) grid = std::max<size_t>(need, 1);
	const size_t cap = kUpsweepThreads * kUpsweepKeysPerThread;
	grid = std::max(grid, (n + cap - 1) / cap);
	kern<<<(unsigned)grid, kUpsweepThreads, smem, s>>>(keys, n, hist, base_shift);
}

template <typename K>
void launch_upsweep(int passes, cudaStream_t s, const K *keys, size_t n, uint32_t *hist,
	int sm_count, int base_shift = 0) {
	switch (passes) {
	case 1: launch_upsweep_p<K, 1>(s, keys, n, hist, base_shift, sm_count); break;
	case 2: launch_upsweep_p<K, 2>(s, keys, n, hist, base_shift, sm_count); break;
	case 3: launch_upsweep_p<K, 3>(s, keys, n, hist, base_shift, sm_count); break;
	case 4: launch_upsweep_p<K, 4>(s, keys, n, hist, base_shift, sm_count); break;
	case 5: launch_upsweep_p<K, 5>(s, keys, n, hist, base_shift, sm_count); break;
	case 6: launch_upsweep_p<K, 6>(s, keys, n, hist, base_shift, sm_count); break;
	case 7: launch_upsweep_p<K, 7>(s, keys, n, hist, base_shift, sm_count); break;
	default: launch_upsweep_p<K, 8>(s, keys, n, hist, base_shift, sm_count); break;
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
	const size_t smem = chunked_smem<K, V, HAS_V, CT>();
	auto kern = radix_pass_chunked<K, V, HAS_V, CT>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	int per_sm = 0;
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CT, smem);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "satradix");
		return e;
	}
	const uint32_t chunks = chunk_count<K>(ctiles, ctx->sm_count, per_sm);
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
	e = cudaMemsetAsync(tmp, 0, off_st1, s);
	unsigned launches = 0;
	if (e == cudaSuccess) {
		KernelTimer t("satradix_upsweep", s, (double)n * sizeof(K));
		launch_upsweep<K>(passes, s, (const K *)keys, n, hist, ctx->sm_count);
		t.stop();
		launches++;
		e = cudaGetLastError();
	}
	std::vector<int> active;
	if (e == cudaSuccess) {
		// Below 2^22 keys the readback's host round trip (the GPU idles
		// while the host decides) costs about what a skipped pass saves.
		if (allow_skip && n >= ((size_t)1 << 22)) {
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
	const size_t smem = chunked_smem<K, uint32_t, false, CT>();
	auto kern = radix_pass_chunked<K, uint32_t, false, CT>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	int per_sm = 0;
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CT, smem);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "satradix partition");
		return e;
	}
	const uint32_t chunks = chunk_count<K>(ctiles, ctx->sm_count, per_sm);
	const size_t status_words = (size_t)chunks * kRadix;
	const size_t off_cnt = kRadix * 4, off_st0 = off_cnt + 64;
	const size_t off_st1 = off_st0 + status_words * 4;
	char *tmp = (char *)tmp_alloc(ctx, off_st1 + status_words * 4, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	uint32_t *hist = (uint32_t *)tmp;
	uint32_t *cnt = (uint32_t *)(tmp + off_cnt);
	e = cudaMemsetAsync(tmp, 0, off_st1, s);
	if (e == cudaSuccess) {
		KernelTimer t("satradix_upsweep", s, (double)n * sizeof(K));
		launch_upsweep<K>(1, s, keys_in, n, hist, ctx->sm_count, shift);
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
