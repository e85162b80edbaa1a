// "satradix": stable LSD radix sort, onesweep style, 8-bit digits.
//
// Result contract (src/cl_ops/sort/clo_sort_satradix.c:117-335 with the
// kernels of clo_sort_satradix.cl:34-258): a stable sort, ascending by the
// unsigned bit pattern of the key. The reference sorts with
// log2(radix)-bit digits; any digit width gives the same stable order, so
// the width here is a tuning choice (8 bits: 4 passes for 32-bit keys).
//
// Per sort:
//   1. radix_upsweep_w: one read of the keys builds the 256-bin histogram
//      of every digit position at once.
//   2. per digit position, radix_pass_tiles (one launch per pass), one CTA
//      per tile (15360 32-bit keys; 7168 pairs of a 64-bit key and a
//      32-bit value), tiles claimed in order from a counter:
//      a. keys are loaded in half-warp units (a unit's keys are in index
//         order; full tiles of 32-bit keys arrive by bulk copy into shared
//         memory), the tile's digit counts are published for the decoupled
//         lookback before the tile is ranked;
//      b. keys are ranked among equal digits of their unit, stably (lanes
//         in order, rounds in order): peers found through a shared-memory
//         OR mask in the low half of the unit's word for the digit, whose
//         high half holds the unit's next position; keys (and values) are
//         staged in shared memory in tile-sorted order;
//      c. one thread per digit looks back over the preceding tiles
//         (bounded waits) for the digit's global offset;
//      d. the staged tile is written out so that consecutive threads write
//         consecutive addresses of a digit's run.
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
// Histograms of all `passes` digit positions in one read, counted into
// lane columns shared by the CTA's warps through shared-memory adds: the
// counter of digit d of lane l lives in bank l, so a warp's 32 adds hit 32
// different banks whatever the digits. Each thread keeps kUpsweepInFlight
// 16-byte loads in flight.
constexpr int kUpsweepInFlight = 8;

// 1024-thread CTAs. The first four digit positions count into full 32-bit
// words (digit d of lane l at word d * 32 + l per position: one byte
// extract, one address computation and one shared add per key and
// position, and no overflow bound, 32 KB a position); positions five to
// eight (64-bit keys) into 16-bit halves of word (d >> 1) * 32 + l, 16 KB
// per position, with the grid keeping a thread at kUpwHalfKeysPerThread
// keys so that a half, which all 32 warps of a CTA add to, stays below
// 2^16 (eight positions: 192 KB, one CTA per SM).
constexpr int kUpwThreads = 1024;
constexpr size_t kUpwHalfKeysPerThread = 2000;

template <int PASSES>
constexpr size_t upw_smem() {
	return (size_t)(PASSES < 4 ? PASSES : 4) * kRadix * 32 * 4 +
		(size_t)(PASSES > 4 ? PASSES - 4 : 0) * (kRadix / 2) * 32 * 4;
}
// Word offset of position p's columns.
__host__ __device__ constexpr int upw_pos_base(int p) {
	return p <= 4 ? p * kRadix * 32 : 4 * kRadix * 32 + (p - 4) * (kRadix / 2) * 32;
}

template <typename K, int PASSES>
__global__ void __launch_bounds__(kUpwThreads, 1)
radix_upsweep_w(const K *__restrict__ keys, size_t n, uint32_t *__restrict__ hist,
	int base_shift) {
	extern __shared__ __align__(16) uint32_t up_smem[];
	for (int i = threadIdx.x; i < upw_pos_base(PASSES); i += kUpwThreads) up_smem[i] = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31;
	uint32_t *col = up_smem + lane;
	auto count = [&](int p, K key) {
		const uint32_t d = digit_of(key, base_shift + p * kRadixBits);
		if (p >= 4) atomicAdd(col + upw_pos_base(p) + (d >> 1) * 32, 1u << ((d & 1) << 4));
		else atomicAdd(col + upw_pos_base(p) + d * 32, 1u);
	};
	constexpr int PER = 16 / sizeof(K);  // keys per 16-byte load
	const bool aligned = ((uintptr_t)keys % 16) == 0;
	const size_t nvec = aligned ? n / PER : 0;
	const uint4 *kv4 = reinterpret_cast<const uint4 *>(keys);
	const size_t stride = (size_t)gridDim.x * kUpwThreads;
	size_t i = blockIdx.x * (size_t)kUpwThreads + threadIdx.x;
	for (; i + (kUpsweepInFlight - 1) * stride < nvec; i += kUpsweepInFlight * stride) {
		uint4 v[kUpsweepInFlight];
#pragma unroll
		for (int u = 0; u < kUpsweepInFlight; ++u) v[u] = dev::ld_stream_v4(kv4 + i + u * stride);
#pragma unroll
		for (int u = 0; u < kUpsweepInFlight; ++u) {
			const K *e = reinterpret_cast<const K *>(&v[u]);
#pragma unroll
			for (int q = 0; q < PER; ++q)
#pragma unroll
				for (int p = 0; p < PASSES; ++p) count(p, e[q]);
		}
	}
	for (; i < nvec; i += stride) {
		uint4 v = dev::ld_stream_v4(kv4 + i);
		const K *e = reinterpret_cast<const K *>(&v);
#pragma unroll
		for (int q = 0; q < PER; ++q)
#pragma unroll
			for (int p = 0; p < PASSES; ++p) count(p, e[q]);
	}
	for (size_t j = nvec * PER + blockIdx.x * (size_t)kUpwThreads + threadIdx.x; j < n;
		 j += stride) {
		const K key = keys[j];
#pragma unroll
		for (int p = 0; p < PASSES; ++p) count(p, key);
	}
	__syncthreads();
	for (int b = threadIdx.x; b < PASSES * kRadix; b += kUpwThreads) {
		const int p = b / kRadix, d = b % kRadix;
		const bool half = p >= 4;
		// Digit d's 32 columns, from a rotated start (no bank conflicts).
		const uint32_t *row = up_smem + upw_pos_base(p) + (half ? d >> 1 : d) * 32;
		const int hs = half ? (d & 1) << 4 : 0;
		uint32_t v = 0;
#pragma unroll 8
		for (int c = 0; c < 32; ++c) {
			const uint32_t w = row[(c + lane) & 31];
			v += half ? (w >> hs) & 0xFFFFu : w;
		}
		if (v) atomicAdd(hist + b, v);
	}
}

// ------------------------------------------------- pass state and lookback
struct PassArgs {
	const uint32_t *hist;   // 256 bins of this digit position
	uint32_t *status;       // tiles * 256 words used by this pass
	uint32_t *status_next;  // the other buffer, cleared for the next pass
	uint32_t *tile_counter;
	int *dev_status;
	size_t n;
	int shift;
};

// Lookback window: predecessor statuses read per round trip per digit. A
// tile's nearest inclusive predecessor is a few tiles back; wider windows
// measured slower.
#ifndef CLO_RADIX_LOOK_WINDOW
#define CLO_RADIX_LOOK_WINDOW 8
#endif
constexpr int kLookWindow = CLO_RADIX_LOOK_WINDOW;

// Threads per CTA of the pass: at least one per digit (threads below 256
// own a digit in the per-tile scans, the lookback and the output bases).
#ifndef CLO_RADIX_PASS_THREADS
#define CLO_RADIX_PASS_THREADS 256
#endif
constexpr int kPassThreads = CLO_RADIX_PASS_THREADS;
static_assert(kPassThreads >= 256 && kPassThreads <= 1024 && kPassThreads % 32 == 0,
	"pass CTA size");
// Keys per thread for one-word keys (0: the 256-thread shape scaled to the
// CTA size).
#ifndef CLO_RADIX_PASS_KPT1
#define CLO_RADIX_PASS_KPT1 0
#endif
// Resident CTAs per SM the pass is compiled for (registers a thread:
// 65536 / (CTAs x threads)).
#ifndef CLO_RADIX_PASS_MINB
#define CLO_RADIX_PASS_MINB 2
#endif

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

// Ranking and count rows: 256 digits each, 264 words apart, odd rows 8
// words later, so rows 2w and 2w + 1 (the two units of warp w) hold a digit
// 16 banks apart and a digit both halves of a warp hold does not conflict.
constexpr int kRowWords = kRadix + 8;
__device__ __forceinline__ int row_of(int r) { return r * kRowWords + (r & 1) * 8; }

// ------------------------------------------------------- onesweep pass
// One tile per CTA, tiles claimed in order from an atomic counter, so every
// tile a CTA waits on belongs to a CTA that is already running. Per tile:
//  1. keys (and values) are loaded in half-warp units: unit u holds the
//     tile's keys u * 16 KPT .. (u + 1) * 16 KPT - 1, round j of lane l the
//     key 16 j + l, so a unit's (round, lane) order is index order;
//  2. the digits are counted into per-unit rows (16-bit halves, units u and
//     u + 8 sharing a row); the thread of digit d turns them into unit
//     prefixes and the tile's count of d, and publishes the count as the
//     tile's lookback status (tile 0: its inclusive prefix) before the
//     tile is ranked;
//  3. ranking: the unit's word for digit d holds the unit's next tile
//     position for d in its upper half and the round's peer mask in its
//     lower half, so a round is one OR, one read and one store by the
//     lowest peer (stable: lanes in order, rounds in order); keys and
//     values are staged in shared memory at their tile-sorted positions;
//  4. the thread of digit d looks back over the preceding tiles' statuses
//     (windows of kLookWindow, bounded waits), publishes the inclusive
//     prefix and sets the digit's output base;
//  5. the staged tile is written out so that consecutive threads write
//     consecutive addresses of a digit's run.
// Consecutive tiles fill consecutive stretches of every digit's output, so
// output lines complete in L2 while they are hot, and the pass moves one
// read and one write of each key (and value). Tiles are large (TilesCfg)
// because each costs one lookback.
//
// Shared memory: a ranking row per half-warp unit and a count row per two
// units (row_of), the tile offsets and a scan array (256 words each), 64
// misc words, the staged tile (keys, then values).
// Full tiles of 32- or 64-bit keys (with 32- or 64-bit values, if any) are
// taken in with bulk copies (per half-warp unit one of its keys and one of
// its values, into the staging area; the copy engine, not the load/store
// pipe) and read from shared memory: a warp round of 32-bit elements is
// one conflict-free wavefront instead of two global ones (the two units
// of a warp are KPT x 64 bytes apart). 32-bit keys: 0.808 -> 0.790 ms a
// pass at 2^28.
#ifndef CLO_RADIX_BULK_LOAD
#define CLO_RADIX_BULK_LOAD 1
#endif
// 64-bit values as well: (u32, u64) pairs at 2^27 4.31 -> 3.26 ms a sort,
// (u64, u64) 10.28 -> 8.30 ms with the larger tiles the freed registers
// allow.
#ifndef CLO_RADIX_BULK_V8
#define CLO_RADIX_BULK_V8 1
#endif
template <typename K, typename V, bool HAS_V>
constexpr bool bulk_tile_load() {
	return CLO_RADIX_BULK_LOAD && (sizeof(K) == 4 || sizeof(K) == 8) &&
		(!HAS_V || sizeof(V) == 4 || (CLO_RADIX_BULK_V8 && sizeof(V) == 8));
}
// Landing-area elements per unit: the unit's elements, plus 16 where 4-byte
// elements of both units of a warp would otherwise fall in the same banks.
template <int KPT, int BYTES>
constexpr int land_unit_elems() {
	return 16 * KPT + (BYTES == 4 && (16 * KPT) % 32 == 0 ? 16 : 0);
}
// Landing-area bytes of the keys (the values follow them).
template <typename K, int THREADS, int KPT>
constexpr size_t land_key_bytes() {
	return (size_t)(THREADS / 16) * land_unit_elems<KPT, (int)sizeof(K)>() * sizeof(K);
}

template <typename K, typename V, bool HAS_V, int THREADS, int KPT>
constexpr size_t tiles_smem() {
	const size_t stage = (size_t)THREADS * KPT * (sizeof(K) + (HAS_V ? sizeof(V) : 0));
	const size_t land = bulk_tile_load<K, V, HAS_V>()
		? land_key_bytes<K, THREADS, KPT>() + (HAS_V
			? (size_t)(THREADS / 16) * land_unit_elems<KPT, (int)sizeof(V)>() * sizeof(V) : 0)
		: 0;
	return ((size_t)(THREADS / 16 + THREADS / 32) * kRowWords + 2 * kRadix + 64) *
		sizeof(uint32_t) + (stage > land ? stage : land);
}

template <typename K, typename V, bool HAS_V, int THREADS, int KPT, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
radix_pass_tiles(const K *__restrict__ kin, K *__restrict__ kout,
	const V *__restrict__ vin, V *__restrict__ vout, PassArgs a, uint32_t num_tiles) {
	constexpr int TILE = THREADS * KPT;
	constexpr int UNITS = THREADS / 16;
	constexpr int HALF = UNITS / 2;
	constexpr int UKEYS = 16 * KPT;  // a unit's keys
	static_assert(UKEYS <= 0xFFFF && TILE <= 0xFFFF, "16-bit unit and tile counts");
	constexpr int kWin = kLookWindow;
	extern __shared__ __align__(16) unsigned char smem[];
	uint32_t *s_rank = reinterpret_cast<uint32_t *>(smem);   // [UNITS] rows
	uint32_t *s_cnt = s_rank + UNITS * kRowWords;            // [HALF] rows
	uint32_t *s_tile_off = s_cnt + HALF * kRowWords;         // [256]
	uint32_t *s_part = s_tile_off + kRadix;                  // [256]
	uint32_t *s_misc = s_part + kRadix;                      // [64]
	unsigned char *s_stage = reinterpret_cast<unsigned char *>(s_misc + 64);

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int unit = 2 * warp + (lane >> 4);
	const uint32_t l16 = lane & 15;
	const uint32_t lt16 = (1u << l16) - 1u;
	uint32_t *my_rank = s_rank + row_of(unit);
	uint32_t *my_cnt = s_cnt + row_of(unit % HALF);
	const uint32_t cnt_inc = 1u << ((unit / HALF) * 16);
	const int shift = a.shift;
	// Threads below 256 (whole warps) own digit pd in the per-digit steps.
	const bool owner = THREADS == kRadix || tid < kRadix;
	const int pd = tid & (kRadix - 1);
	const int dw = pd >> 5;

	constexpr bool BULK = bulk_tile_load<K, V, HAS_V>();
	constexpr int LK = land_unit_elems<KPT, (int)sizeof(K)>();
	constexpr int LV = land_unit_elems<KPT, (int)sizeof(V)>();
	uint64_t *bar = reinterpret_cast<uint64_t *>(s_misc + 32);
	const bool bulk_ok = BULK && ((uintptr_t)kin % 16) == 0 &&
		(!HAS_V || ((uintptr_t)vin % 16) == 0);
	K *land_k = reinterpret_cast<K *>(s_stage);
	V *land_v = reinterpret_cast<V *>(s_stage + land_key_bytes<K, THREADS, KPT>());
	if (tid == 0) {
		const uint32_t tt = atomicAdd(a.tile_counter, 1u);
		s_misc[0] = tt;
		if (bulk_ok && tt < num_tiles && (size_t)(tt + 1) * TILE <= a.n) {
			dev::mbar_init(bar, 1);
			dev::mbar_expect_tx(bar, (uint32_t)(TILE * (sizeof(K) + (HAS_V ? sizeof(V) : 0))));
			const size_t t0 = (size_t)tt * TILE;
#pragma unroll 1
			for (int u = 0; u < UNITS; ++u) {
				dev::bulk_g2s(land_k + u * LK, kin + t0 + u * UKEYS,
					(uint32_t)(UKEYS * sizeof(K)), bar);
				if constexpr (HAS_V)
					dev::bulk_g2s(land_v + u * LV, vin + t0 + u * UKEYS,
						(uint32_t)(UKEYS * sizeof(V)), bar);
			}
		}
	}
	uint32_t hv = 0, hinc = 0;
	if (owner) {
#pragma unroll
		for (int i = 0; i < HALF; ++i) s_cnt[row_of(i) + pd] = 0;
		// Global digit base of this pass: exclusive scan of its histogram.
		hv = a.hist[pd];
		hinc = hv;
#pragma unroll
		for (int s = 1; s < 32; s <<= 1) {
			uint32_t t = __shfl_up_sync(0xffffffffu, hinc, s);
			if (lane >= s) hinc += t;
		}
		if (lane == 31) s_misc[16 + dw] = hinc;
	}
	__syncthreads();
	const uint32_t t = s_misc[0];
	if (t >= num_tiles) return;
	uint32_t gbase = hinc - hv;
#pragma unroll
	for (int w = 0; w < 8; ++w)
		if (w < dw) gbase += s_misc[16 + w];

	// Keys (and values) of this thread's unit, round-major (index order).
	K k[KPT];
	V v[HAS_V ? KPT : 1];
	const size_t ubase = (size_t)t * TILE + (size_t)unit * UKEYS;
	if (bulk_ok && (size_t)(t + 1) * TILE <= a.n) {
		if (!dev::mbar_wait_bounded(bar, 0)) {
			if (tid == 0) dev::report_timeout(a.dev_status, DEV_ERR_COPY_TIMEOUT, (int)t);
			dev::mbar_wait_bounded(bar, 0);  // the copies still in flight
		}
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			k[j] = land_k[unit * LK + j * 16 + l16];
			if constexpr (HAS_V) v[j] = land_v[unit * LV + j * 16 + l16];
		}
	} else {
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			const size_t idx = ubase + (size_t)j * 16 + l16;
			k[j] = idx < a.n ? kin[idx] : (K)~(K)0;
			if constexpr (HAS_V) v[j] = idx < a.n ? vin[idx] : (V)0;
		}
	}
#pragma unroll
	for (int j = 0; j < KPT; ++j) atomicAdd(my_cnt + digit_of(k[j], shift), cnt_inc);
	__syncthreads();
	// Unit prefixes of digit pd in unit order (written to the units' rank
	// words, the tile offset added below) and the tile's count.
	uint32_t sum = 0;
	uint32_t *st = a.status + (size_t)t * kRadix + pd;
	if (owner) {
		uint32_t run = 0;
#pragma unroll
		for (int i = 0; i < HALF; ++i) {
			s_rank[row_of(i) + pd] = run << 16;
			run += s_cnt[row_of(i) + pd] & 0xFFFFu;
		}
#pragma unroll
		for (int i = 0; i < HALF; ++i) {
			s_rank[row_of(i + HALF) + pd] = run << 16;
			run += s_cnt[row_of(i) + pd] >> 16;
		}
		sum = run;
		// Publish the tile's count of digit pd (tile 0: its inclusive prefix).
		dev::st_relaxed_u32(st, (t == 0 ? kStPrefix : kStAgg) | sum);
		a.status_next[(size_t)t * kRadix + pd] = 0;
		// Tile offsets of the digits: exclusive scan of the counts.
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
	if (owner) {
		uint32_t to = s_part[pd];
#pragma unroll
		for (int w = 0; w < 8; ++w)
			if (w < dw) to += s_misc[8 + w];
#pragma unroll
		for (int i = 0; i < UNITS; ++i) s_rank[row_of(i) + pd] += to << 16;
		// Output index of staged position q of digit d is q + G[d] (mod
		// 2^32), G[d] = global base + lookback prefix - tile offset; the
		// prefix is added after the lookback.
		s_tile_off[pd] = gbase - to;
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
	// Lookback over the preceding tiles for digit pd (bounded waits).
	uint32_t excl = 0;
	if (owner && t > 0) {
		long long base = (long long)t - 1;
		uint32_t iter = 0;
		bool done = lookback_window<kWin>(a.status, pd, base, excl);
		while (!done && base >= 0) {
			uint32_t sw = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
			while ((sw & ~kStValue) == 0) {
				if (++iter >= dev::kSpinLimit) break;
				dev::backoff(iter);
				sw = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
			}
			if ((sw & ~kStValue) == 0) {
				dev::report_timeout(a.dev_status, DEV_ERR_LOOKBACK_TIMEOUT, (int)t);
				break;
			}
			done = lookback_window<kWin>(a.status, pd, base, excl);
		}
		dev::st_relaxed_u32(st, kStPrefix | (excl + sum));
	}
	if (owner) s_tile_off[pd] += excl;
	__syncthreads();
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

// Tile shape of the pass by the 32-bit register words a key (and value)
// takes: keys per thread and resident CTAs per SM, each the measured best
// at 2^27 - 2^28 elements (larger tiles spread the per-tile work -- row
// clears and scans, the lookback -- over more keys; the limits are 128
// registers a thread without spills and two CTAs' shared memory per SM).
// 32-bit keys: 15360-key tiles; 64-bit keys or 32-bit pairs: 10240;
// 12-byte pairs (bulk-loaded): 7168, 5120 for those loaded lane by lane
// (8- and 16-bit keys with 64-bit values); 16-byte pairs 5120.
template <typename K, typename V, bool HAS_V>
struct TilesCfg {
	static constexpr int kWords = (int)((sizeof(K) + 3) / 4) + (HAS_V ? (int)((sizeof(V) + 3) / 4) : 0);
	static constexpr int kThreads = kPassThreads;
#ifndef CLO_RADIX_PASS_KPT2
#define CLO_RADIX_PASS_KPT2 40
#endif
#ifndef CLO_RADIX_PASS_KPT3
#define CLO_RADIX_PASS_KPT3 28
#endif
#ifndef CLO_RADIX_PASS_KPT4
#define CLO_RADIX_PASS_KPT4 20
#endif
	static constexpr int kKpt256 = kWords == 1 ? 60 : kWords == 2 ? CLO_RADIX_PASS_KPT2
		: kWords == 3 ? (bulk_tile_load<K, V, HAS_V>() ? CLO_RADIX_PASS_KPT3 : 20)
		: (bulk_tile_load<K, V, HAS_V>() ? CLO_RADIX_PASS_KPT4 : 16);
	static constexpr int kKpt = (kWords == 1 && CLO_RADIX_PASS_KPT1 > 0) ? CLO_RADIX_PASS_KPT1
		: kKpt256 * 256 / kThreads;
	static constexpr int kMinBlocks = CLO_RADIX_PASS_MINB;
	static constexpr int kTile = kThreads * kKpt;
};

// The shape for sorts too small to give every SM a tile of TilesCfg size
// (2^20 32-bit keys make 69 of those for 152 SMs): a quarter of the keys
// per thread, so the tiles spread over the whole GPU.
template <typename K, typename V, bool HAS_V>
struct TilesCfgSmall {
	using Big = TilesCfg<K, V, HAS_V>;
	static constexpr int kThreads = Big::kThreads;
	static constexpr int kKpt = Big::kKpt / 4 < 4 ? 4 : Big::kKpt / 4;
	static constexpr int kMinBlocks = Big::kMinBlocks;
	static constexpr int kTile = kThreads * kKpt;
};

template <typename K, int PASSES>
void launch_upsweep_p(cudaStream_t s, const K *keys, size_t n, uint32_t *hist,
	int base_shift, int sm_count) {
	constexpr size_t smem = upw_smem<PASSES>();
	auto kern = radix_upsweep_w<K, PASSES>;
	if (smem > 48 * 1024)
		cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	// 2048 threads per SM: two CTAs where shared memory allows (228 KB per
	// SM, 1 KB reserved per CTA); at least enough CTAs for the key cap of
	// the 16-bit halves.
	const int per_sm = (int)std::min<size_t>(2, (228 * 1024) / (smem + 1024));
	size_t grid = (size_t)sm_count * std::max(per_sm, 1);
	const size_t need = ((n * sizeof(K) + 15) / 16 + kUpwThreads - 1) / kUpwThreads;
	if (grid > need) grid = std::max<size_t>(need, 1);
	if (PASSES > 4) {
		const size_t cap = kUpwThreads * kUpwHalfKeysPerThread;
		grid = std::max(grid, (n + cap - 1) / cap);
	}
	kern<<<(unsigned)grid, kUpwThreads, smem, s>>>(keys, n, hist, base_shift);
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

template <typename K, typename V, bool HAS_V, typename TC>
cudaError_t sort_tiles(void *keys, void *vals, size_t n, int passes,
	CCLContext *ctx, cudaStream_t s, bool allow_skip, GError **err) {
	// One CTA per tile of TC's size.
	const size_t ctiles = (n + TC::kTile - 1) / TC::kTile;
	const size_t smem = tiles_smem<K, V, HAS_V, TC::kThreads, TC::kKpt>();
	auto kern = radix_pass_tiles<K, V, HAS_V, TC::kThreads, TC::kKpt, TC::kMinBlocks>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "satradix");
		return e;
	}
	// Status slots: one per tile.
	const size_t status_words = ctiles * kRadix;
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
			kern<<<(unsigned)ctiles, TC::kThreads, smem, s>>>(src_k, dst_k, src_v, dst_v, pa,
				(uint32_t)ctiles);
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
	using Big = TilesCfg<K, V, HAS_V>;
	if ((n + Big::kTile - 1) / Big::kTile < (size_t)ctx->sm_count)
		return sort_tiles<K, V, HAS_V, TilesCfgSmall<K, V, HAS_V>>(keys, vals, n, passes, ctx,
			s, allow_skip, err);
	return sort_tiles<K, V, HAS_V, Big>(keys, vals, n, passes, ctx, s, allow_skip, err);
}

// Stable partition of n keys by the top 8 of their sort_bits low bits:
// keys_out receives the keys grouped by that digit, in input order within a
// digit; counts (host) receives the 256 group sizes. One histogram kernel
// for the digit, a host readback of its 256 counts, one pass.
template <typename K>
cudaError_t msd_partition_typed(const K *keys_in, K *keys_out, size_t n, int sort_bits,
	uint32_t *counts, CCLContext *ctx, cudaStream_t s, GError **err) {
	using TC = TilesCfg<K, uint32_t, false>;
	const int shift = sort_bits - kRadixBits;
	const size_t ctiles = (n + TC::kTile - 1) / TC::kTile;
	const size_t smem = tiles_smem<K, uint32_t, false, TC::kThreads, TC::kKpt>();
	auto kern = radix_pass_tiles<K, uint32_t, false, TC::kThreads, TC::kKpt, TC::kMinBlocks>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "satradix partition");
		return e;
	}
	const size_t status_words = ctiles * kRadix;
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
			kern<<<(unsigned)ctiles, TC::kThreads, smem, s>>>(keys_in, keys_out, nullptr, nullptr,
				pa, (uint32_t)ctiles);
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
