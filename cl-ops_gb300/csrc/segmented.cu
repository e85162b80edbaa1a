// Segmented sort and segmented scan: many independent segments of one
// buffer, each handled exactly as a separate clo_sort / clo_scan call on it
// would handle it, in a fixed sequence of launches whatever the number and
// the sizes of the segments (no host readback, so the sequence can be
// captured into a CUDA graph).
//
// Segments are given by a device array of S + 1 non-decreasing 64-bit
// offsets; segment i is [off[i], off[i+1]).
//
// Sort ("satradix" order: stable, ascending by the low sort_bits bits of
// the unsigned element pattern), by segment length:
//   len <= 32           one warp per segment: a 32-lane bitonic network on
//                       (key, index) pairs, which makes it stable;
//   len <= tile A       one CTA per segment (class A tile, e.g. 128 x 8),
//   len <= tile B       one CTA per segment (class B tile, e.g. 512 x 16):
//                       an LSD radix sort in shared memory, 8-bit digits,
//                       stable warp-multisplit ranking, digits that are
//                       constant over the segment skipped;
//   longer              the onesweep pass of the full sort, with tiles that
//                       never straddle segments, per-segment digit
//                       histograms and a decoupled lookback that stops at
//                       the segment's first tile.
// A classification kernel builds one list per class (and the tile counts
// of the long segments, scanned into tile starts) on the device.
//
// Scan ("blelloch" semantics per segment): one decoupled-lookback launch
// over the whole buffer with a bitmap of segment heads; sums restart at
// every head, a tile holding a head publishes its inclusive prefix at once.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>

#include "clo_internal.h"
#include "dev_common.cuh"
#include "scan_status.cuh"
#include "seg_common.cuh"
#include "scan_tile.cuh"
#include "timing.h"

namespace clo {
namespace {

using namespace seg;

__device__ __forceinline__ void report_bad_segment(int *st, uint32_t s) {
	if (atomicCAS(st, 0, DEV_ERR_BAD_SEGMENTS) == 0) atomicExch(st + 1, (int)s);
}

// Length of segment s, or 0 (and an error report) when its offsets are
// invalid: decreasing, past the buffer, or 2^30 elements or more.
__device__ __forceinline__ uint64_t checked_len(const uint64_t *off, uint32_t s,
	uint64_t n_cap, int *st) {
	const uint64_t a = off[s], b = off[s + 1];
	if (a > b || b > n_cap || b - a > kMaxSegLen) {
		report_bad_segment(st, s);
		return 0;
	}
	return b - a;
}

template <typename T>
__device__ __forceinline__ T shfl_xor_any(T v, int m) {
	if (sizeof(T) == 8)
		return (T)__shfl_xor_sync(0xffffffffu, (unsigned long long)v, m);
	return (T)__shfl_xor_sync(0xffffffffu, (uint32_t)v, m);
}

// ------------------------------------------------------ classification
// Class lists: [0] warp, [1] CTA A, [2] CTA B, [3] large; counts[0..3].
// tinfo[s] = (tiles of s << 32) | 1 for a large segment, else 0;
// tinfo[S] = 0 (its exclusive scan gives the tile starts and the large
// ranks, and in entry S the totals).
struct ClassArgs {
	const uint64_t *off;
	uint32_t S;
	uint64_t n_cap;
	uint32_t max_warp, max_a, max_b, large_tile;
	uint32_t *lists;
	uint32_t *counts;
	uint64_t *tinfo;
	int *dev_status;
};

__global__ void __launch_bounds__(256) seg_classify(ClassArgs a) {
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t lt = dev::lanemask_lt();
	const uint64_t warp_id = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint64_t w = warp_id; w * 32 <= (uint64_t)a.S; w += nwarps) {
		const uint64_t s = w * 32 + lane;
		int cls = -1;
		uint64_t packed = 0;
		if (s < a.S) {
			const uint64_t len = checked_len(a.off, (uint32_t)s, a.n_cap, a.dev_status);
			if (len >= 2) {
				if (len <= a.max_warp) cls = 0;
				else if (len <= a.max_a) cls = 1;
				else if (len <= a.max_b) cls = 2;
				else {
					cls = 3;
					packed = (((len + a.large_tile - 1) / a.large_tile) << 32) | 1ull;
				}
			}
		}
		if (s <= a.S) a.tinfo[s] = packed;
#pragma unroll
		for (int c = 0; c < 4; ++c) {
			const uint32_t m = __ballot_sync(0xffffffffu, cls == c);
			if (m) {
				const int leader = __ffs(m) - 1;
				uint32_t base = 0;
				if ((int)lane == leader) base = atomicAdd(a.counts + c, (uint32_t)__popc(m));
				base = __shfl_sync(0xffffffffu, base, leader);
				if (cls == c) a.lists[(size_t)c * a.S + base + __popc(m & lt)] = (uint32_t)s;
			}
		}
	}
}

// --------------------------------------------------------- warp class
template <typename K>
__global__ void __launch_bounds__(256) seg_sort_warp(K *keys, const uint64_t *off,
	const uint32_t *list, const uint32_t *count, K mask) {
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
	const uint32_t cnt = *count;
	for (uint32_t i = gw; i < cnt; i += nw) {
		const uint32_t s = list[i];
		const uint64_t base = off[s];
		const uint32_t len = (uint32_t)(off[s + 1] - base);
		K v = lane < len ? keys[base + lane] : (K)~(K)0;
		K key = v & mask;
		uint32_t idx = lane;
		// Ascending bitonic network over (key, original lane): ties keep
		// their input order, so the result is the stable order.
#pragma unroll
		for (uint32_t size = 2; size <= 32; size <<= 1) {
#pragma unroll
			for (uint32_t j = size >> 1; j > 0; j >>= 1) {
				const K ov = shfl_xor_any(v, (int)j);
				const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, (int)j);
				const K okey = ov & mask;
				const bool up = (lane & size) == 0;
				const bool lower = (lane & j) == 0;
				const bool other_less = okey < key || (okey == key && oi < idx);
				if ((lower == up) == other_less) {
					v = ov;
					key = okey;
					idx = oi;
				}
			}
		}
		if (lane < len) keys[base + lane] = v;
	}
}

// ------------------------------------------------------ large segments
// Tile -> segment map and per-tile descriptors (segment start and end,
// tile index within the segment, large-segment rank: what a pass needs to
// start a tile, in one round trip), and clearing of what the passes
// accumulate into: the segment's digit histograms and the first pass's
// tile statuses.
__global__ void __launch_bounds__(256) seg_tiles(const uint64_t *off,
	const uint64_t *tstart, const uint32_t *list, const uint32_t *count,
	uint32_t *tile_seg, ulonglong2 *tile_span, uint2 *tile_x, uint32_t *seg_hist,
	int passes, uint32_t *status0, uint32_t tile) {
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
	const uint32_t cnt = *count;
	for (uint32_t i = gw; i < cnt; i += nw) {
		const uint32_t s = list[i];
		const uint64_t ts = tstart[s];
		const uint32_t first = (uint32_t)(ts >> 32), lr = (uint32_t)ts;
		const uint64_t len = off[s + 1] - off[s];
		const uint32_t ntiles = (uint32_t)((len + tile - 1) / tile);
		const ulonglong2 span = make_ulonglong2(off[s], off[s + 1]);
		for (uint32_t t = lane; t < ntiles; t += 32) {
			tile_seg[first + t] = s;
			tile_span[first + t] = span;
			tile_x[first + t] = make_uint2(t, lr);
		}
		uint4 *h = reinterpret_cast<uint4 *>(seg_hist + (size_t)lr * passes * kRadix);
		for (uint32_t q = lane; q < (uint32_t)passes * (kRadix / 4); q += 32)
			h[q] = make_uint4(0, 0, 0, 0);
		uint4 *st = reinterpret_cast<uint4 *>(status0 + (size_t)first * kRadix);
		for (uint32_t q = lane; q < ntiles * (kRadix / 4); q += 32)
			st[q] = make_uint4(0, 0, 0, 0);
	}
}

// Histograms of every digit position of every large segment: one CTA per
// tile at a time, shared-memory counts added to the segment's histograms.
constexpr int kSegUpLoads = 8;
template <typename K, int PASSES>
__global__ void __launch_bounds__(256) seg_upsweep(const K *keys, const uint64_t *off,
	const uint64_t *tstart, const uint32_t *tile_seg, uint32_t S,
	uint32_t *seg_hist, uint32_t tile) {
	__shared__ uint32_t h[PASSES * kRadix];
	__shared__ uint64_t s_a, s_e;
	__shared__ uint32_t s_lr;
	const uint32_t T = (uint32_t)(tstart[S] >> 32);
	for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
		for (int i = threadIdx.x; i < PASSES * kRadix; i += blockDim.x) h[i] = 0;
		if (threadIdx.x == 0) {
			const uint32_t s = tile_seg[t];
			const uint64_t ts = tstart[s];
			const uint64_t a = off[s] + (uint64_t)(t - (uint32_t)(ts >> 32)) * tile;
			const uint64_t e = off[s + 1];
			s_a = a;
			s_e = a + tile < e ? a + tile : e;
			s_lr = (uint32_t)ts;
		}
		__syncthreads();
		const uint64_t a = s_a, e = s_e;
		auto count = [&](K key) {
#pragma unroll
			for (int p = 0; p < PASSES; ++p)
				atomicAdd(&h[p * kRadix + digit_of(key, p * kRadixBits)], 1u);
		};
		// kSegUpLoads loads in flight per thread, then their counts.
		uint64_t i = a + threadIdx.x;
		for (; i + (uint64_t)(kSegUpLoads - 1) * blockDim.x < e; i += (uint64_t)kSegUpLoads * blockDim.x) {
			K kk[kSegUpLoads];
#pragma unroll
			for (int u = 0; u < kSegUpLoads; ++u) kk[u] = keys[i + (uint64_t)u * blockDim.x];
#pragma unroll
			for (int u = 0; u < kSegUpLoads; ++u) count(kk[u]);
		}
		for (; i < e; i += blockDim.x) count(keys[i]);
		__syncthreads();
		uint32_t *dst = seg_hist + (size_t)s_lr * PASSES * kRadix;
		for (int i = threadIdx.x; i < PASSES * kRadix; i += blockDim.x)
			if (h[i]) atomicAdd(dst + i, h[i]);
		__syncthreads();
	}
}

// Copies the large segments back from the alternate buffer (odd number of
// passes).
template <typename K>
__global__ void __launch_bounds__(256) seg_copy_large(K *dst, const K *src,
	const uint64_t *off, const uint64_t *tstart, const uint32_t *tile_seg, uint32_t S,
	uint32_t tile) {
	const uint32_t T = (uint32_t)(tstart[S] >> 32);
	for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
		const uint32_t s = tile_seg[t];
		const uint64_t a = off[s] + (uint64_t)(t - (uint32_t)(tstart[s] >> 32)) * tile;
		const uint64_t e = off[s + 1];
		const uint64_t end = a + tile < e ? a + tile : e;
		for (uint64_t i = a + threadIdx.x; i < end; i += blockDim.x) dst[i] = src[i];
	}
}

// Copies the segments sorted in place (warp and CTA classes) from `src`
// to `dst`, one warp per segment.
template <typename K>
__global__ void __launch_bounds__(256) seg_copy_short(K *dst, const K *src,
	const uint64_t *off, const uint32_t *lists, const uint32_t *counts, uint32_t S) {
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
	for (int c = 0; c < 3; ++c) {
		const uint32_t cnt = counts[c];
		for (uint32_t i = gw; i < cnt; i += nw) {
			const uint32_t s = lists[(size_t)c * S + i];
			for (uint64_t j = off[s] + lane; j < off[s + 1]; j += 32) dst[j] = src[j];
		}
	}
}

template <typename K>
void launch_seg_upsweep(int passes, uint32_t grid, cudaStream_t s, const K *keys,
	const uint64_t *off, const uint64_t *tstart, const uint32_t *tile_seg, uint32_t S,
	uint32_t *seg_hist, uint32_t tile) {
	switch (passes) {
	case 1: seg_upsweep<K, 1><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 2: seg_upsweep<K, 2><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 3: seg_upsweep<K, 3><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 4: seg_upsweep<K, 4><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 5: seg_upsweep<K, 5><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 6: seg_upsweep<K, 6><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	case 7: seg_upsweep<K, 7><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	default: seg_upsweep<K, 8><<<grid, 256, 0, s>>>(keys, off, tstart, tile_seg, S, seg_hist, tile); break;
	}
}

template <typename K>
cudaError_t seg_sort_typed(K *keys, uint64_t n_cap, const uint64_t *off, uint32_t S,
	int sort_bits, int variant, CCLContext *ctx, cudaStream_t s, GError **err,
	K *alt_ext, bool *in_alt) {
	const SegShape sh = seg_shape(variant);
	const uint32_t LTILE = long_tile<K>(sh.long_idx);
	const int passes = sort_bits / kRadixBits;
	if (in_alt) *in_alt = false;
	if (S == 0 || passes == 0 || n_cap < 2) return cudaSuccess;
	const uint32_t max_a = class_a_max<K>(sh);
	const uint32_t max_b = class_b_max<K>(sh);
	// Bounds the host can derive without reading the offsets.
	const uint64_t L_bound = std::min<uint64_t>(S, n_cap / (max_b + 1));
	const uint64_t T_bound = n_cap / LTILE + L_bound + 1;
	// Scratch: [counts 16][lists 4S][tinfo S+1][tstart S+1] then, with large
	// segments possible, [tile_seg T][tile_span T][tile_x T]
	// [seg_hist L*passes*256][status 2*T*256][alt keys n_cap].
	size_t off_cnt = 0;
	size_t off_lists = 64;
	size_t off_tinfo = (off_lists + 4 * (size_t)S * 4 + 15) / 16 * 16;
	size_t off_tstart = off_tinfo + ((size_t)S + 1) * 8;
	size_t off_tseg = (off_tstart + ((size_t)S + 1) * 8 + 255) / 256 * 256;
	size_t off_tspan = (off_tseg + T_bound * 4 + 255) / 256 * 256;
	size_t off_tx = off_tspan + T_bound * 16;
	size_t off_hist = (off_tx + T_bound * 8 + 255) / 256 * 256;
	size_t off_st0 = (off_hist + L_bound * passes * kRadix * 4 + 255) / 256 * 256;
	size_t off_st1 = off_st0 + T_bound * kRadix * 4;
	size_t off_alt = (off_st1 + T_bound * kRadix * 4 + 255) / 256 * 256;
	size_t total = L_bound ? off_alt + (alt_ext ? 0 : n_cap * sizeof(K)) : off_tseg;
	char *tmp = (char *)tmp_alloc(ctx, total, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	uint32_t *counts = (uint32_t *)(tmp + off_cnt);
	uint32_t *lists = (uint32_t *)(tmp + off_lists);
	uint64_t *tinfo = (uint64_t *)(tmp + off_tinfo);
	uint64_t *tstart = (uint64_t *)(tmp + off_tstart);
	uint32_t *tile_seg = (uint32_t *)(tmp + off_tseg);
	ulonglong2 *tile_span = (ulonglong2 *)(tmp + off_tspan);
	uint2 *tile_x = (uint2 *)(tmp + off_tx);
	uint32_t *seg_hist = (uint32_t *)(tmp + off_hist);
	uint32_t *st[2] = {(uint32_t *)(tmp + off_st0), (uint32_t *)(tmp + off_st1)};
	K *alt = alt_ext ? alt_ext : (K *)(tmp + off_alt);
	unsigned launches = 0;
	cudaError_t e = cudaMemsetAsync(counts, 0, 64, s);
	if (e == cudaSuccess) {
		ClassArgs ca;
		ca.off = off;
		ca.S = S;
		ca.n_cap = n_cap;
		ca.max_warp = 32;
		ca.max_a = max_a;
		ca.max_b = max_b;
		ca.large_tile = LTILE;
		ca.lists = lists;
		ca.counts = counts;
		ca.tinfo = tinfo;
		ca.dev_status = ctx->d_status;
		const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)S + 1 + 255) / 256,
			(uint64_t)ctx->sm_count * 8);
		seg_classify<<<grid, 256, 0, s>>>(ca);
		launches++;
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = scan_exclusive(tinfo, tstart, (size_t)S + 1, CLO_ULONG, 8, ctx, s, err);
	const K mask = sort_bits >= (int)(8 * sizeof(K)) ? (K)~(K)0
		: (K)(((K)1 << sort_bits) - 1);
	if (e == cudaSuccess) {
		const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)S + 7) / 8,
			(uint64_t)ctx->sm_count * 8);
		KernelTimer t("seg_sort_warp", s, 0.0);
		seg_sort_warp<K><<<grid, 256, 0, s>>>(keys, off, lists, counts, mask);
		t.stop();
		launches++;
		e = cudaGetLastError();
	}
	if (e == cudaSuccess)
		e = seg_launch_cta_classes<K>(sh, keys, off, lists, counts, S, sort_bits, n_cap, ctx, s);
	if (e == cudaSuccess && L_bound > 0) {
		const uint32_t *list3 = lists + 3 * (size_t)S;
		{
			const uint32_t grid = (uint32_t)std::min<uint64_t>((L_bound + 7) / 8,
				(uint64_t)ctx->sm_count * 8);
			seg_tiles<<<grid, 256, 0, s>>>(off, tstart, list3, counts + 3, tile_seg,
				tile_span, tile_x, seg_hist, passes, st[0], LTILE);
			launches++;
			e = cudaGetLastError();
		}
		if (e == cudaSuccess) {
			const uint32_t grid = (uint32_t)std::min<uint64_t>(T_bound,
				(uint64_t)ctx->sm_count * 8);
			KernelTimer t("seg_upsweep", s, 0.0);
			launch_seg_upsweep<K>(passes, grid, s, keys, off, tstart, tile_seg, S, seg_hist,
				LTILE);
			t.stop();
			launches++;
			e = cudaGetLastError();
		}
		K *src = keys, *dst = alt;
		for (int p = 0; p < passes && e == cudaSuccess; ++p) {
			SegPassArgs pa;
			pa.off = off;
			pa.tstart = tstart;
			pa.tile_seg = tile_seg;
			pa.tile_span = tile_span;
			pa.tile_x = tile_x;
			pa.seg_hist = seg_hist + (size_t)p * kRadix;
			pa.hist_stride = (uint32_t)(passes * kRadix);
			pa.status = st[p & 1];
			pa.status_next = st[(p + 1) & 1];
			pa.counter = counts + 8 + p;
			pa.dev_status = ctx->d_status;
			pa.S = S;
			pa.shift = p * kRadixBits;
			e = seg_launch_pass<K>(sh, src, dst, pa, T_bound, ctx, s);
			std::swap(src, dst);
		}
		if (e == cudaSuccess && (passes & 1) && alt_ext && in_alt) {
			// The caller takes the long segments from its alternate buffer;
			// the short ones, sorted in place, are copied there.
			const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)S + 7) / 8,
				(uint64_t)ctx->sm_count * 8);
			seg_copy_short<K><<<grid, 256, 0, s>>>(alt, keys, off, lists, counts, S);
			launches++;
			e = cudaGetLastError();
			*in_alt = true;
		} else if (e == cudaSuccess && (passes & 1)) {
			const uint32_t grid = (uint32_t)std::min<uint64_t>(T_bound,
				(uint64_t)ctx->sm_count * 8);
			seg_copy_large<K><<<grid, 256, 0, s>>>(keys, alt, off, tstart, tile_seg, S, LTILE);
			launches++;
			e = cudaGetLastError();
		}
	}
	count_launches(launches);
	tmp_free(tmp, s);
	if (e != cudaSuccess && (err == nullptr || *err == nullptr)) cuda_ok(e, err, "segmented sort");
	return e;
}

// ------------------------------------------------------------ segmented scan
// Head bitmap: bit i set when a segment starts at element i (and holds
// elements).
__global__ void __launch_bounds__(256) seg_heads(const uint64_t *off, uint32_t S,
	uint64_t n_cap, uint32_t *bits, int *dev_status) {
	const uint64_t end = off[S];
	for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < S;
		 s += (uint64_t)gridDim.x * blockDim.x) {
		const uint64_t len = checked_len(off, (uint32_t)s, n_cap, dev_status);
		const uint64_t a = off[s];
		if (len > 0 && a < end) atomicOr(bits + (a >> 5), 1u << (a & 31));
	}
}

// Segmented exclusive scan: out[i] = sum of in[j] for j from the start of
// i's segment to i - 1, for i in [off[0], off[S]); nothing else is written.
// The combine of (head seen, sum) pairs is the usual segmented one: a
// later head discards what came before it. Same tile layout and pipeline
// as the plain scan (csrc/scan_tile.cuh): persistent CTAs take 8192-element
// tiles in order; while warp 0 looks back, every warp prefetches the next
// tile and its 32 head words, finds its last head (max-reduction) and sums
// the elements from there on, so the next tile's (head seen, sum) is
// published before this tile's outputs -- as an inclusive prefix at once
// when it holds a head. A tile whose first element is a head needs no
// carry and does not look back.
template <typename InT, typename OutT>
__global__ void __launch_bounds__(scantile::kThreads, (scantile::scan_min_blocks<InT, OutT>()))
seg_scan_lookback(const InT *__restrict__ in, OutT *__restrict__ out, uint64_t n,
	const uint32_t *__restrict__ heads, const uint64_t *off, uint32_t S,
	lb::TileStatus ts, int *dev_status, bool vec_ok) {
	using namespace scantile;
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t, uint64_t>::type;
	constexpr int PT = lb::Slots<Acc>::kPerTile;
	constexpr int KW = lb::Slots<Acc>::kWords;
	extern __shared__ __align__(16) unsigned char s_dyn[];
	__shared__ Acc s_wsum[kWarps], s_nsum[kWarps];
	__shared__ uint32_t s_wflag[kWarps], s_nflag[kWarps];
	__shared__ Acc s_excl;
	__shared__ uint32_t s_tile, s_next;
	__shared__ uint64_t s_lo, s_hi;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t num_tiles = (uint32_t)((n + kTile - 1) / kTile);
	InT *s_in = reinterpret_cast<InT *>(s_dyn + (size_t)warp *
		(kBlocks * padded<InT>() * sizeof(InT) + padded<OutT>() * sizeof(OutT)));
	OutT *s_out = reinterpret_cast<OutT *>(s_in + kBlocks * padded<InT>());
	auto full_tile = [&](uint32_t t) { return vec_ok && (uint64_t)(t + 1) * kTile <= n; };
	if (tid == 0) {
		s_tile = atomicAdd(ts.counter, 1u);
		s_lo = off[0];
		s_hi = off[S];
	}
	__syncthreads();
	uint32_t tile = s_tile;
	const uint64_t lo = s_lo, hi = s_hi;
	if (tile >= num_tiles) return;
	{
		const uint64_t wseg = (uint64_t)tile * kTile + (uint64_t)warp * kWarpElems;
		if (full_tile(tile)) {
			BlockRegs<InT> r;
			issue_loads<InT>(r, in, wseg, lane);
			store_loads<InT>(r, s_in, lane);
		} else {
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
				load_block_scalar<InT>(in, n, wseg + (uint64_t)b * kBlock, s_in + b * padded<InT>(), lane);
		}
	}
	__syncwarp();
	bool published = false;  // the current tile's status is already out

	for (;;) {
		if (tid == 0) s_next = atomicAdd(ts.counter, 1u);
		const uint64_t wseg = (uint64_t)tile * kTile + (uint64_t)warp * kWarpElems;

		// ---- per block: head bits, lane runs, warp segmented scan -------
		uint32_t hb[kBlocks], fex[kBlocks], bf[kBlocks];
		Acc ex[kBlocks], bs[kBlocks];
#pragma unroll
		for (int b = 0; b < kBlocks; ++b) {
			const InT *sin = s_in + b * padded<InT>();
			// 16 elements starting at a multiple of 16: one half of one word.
			const uint64_t e0 = wseg + (uint64_t)b * kBlock + (uint64_t)lane * kItems;
			hb[b] = e0 < n ? (heads[e0 >> 5] >> (uint32_t)(e0 & 31)) & 0xffffu : 0u;
			Acc run = 0;
#pragma unroll
			for (int j = 0; j < kItems; ++j) {
				const Acc v = (Acc)(OutT)sin[pidx<InT>(lane * kItems + j)];
				if ((hb[b] >> j) & 1u) run = 0;
				run += v;
			}
			Acc inc = run;
			uint32_t finc = hb[b] != 0;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const Acc t = __shfl_up_sync(0xffffffffu, inc, d);
				const uint32_t tf = __shfl_up_sync(0xffffffffu, finc, d);
				if (lane >= d) {
					if (!finc) inc += t;
					finc |= tf;
				}
			}
			ex[b] = __shfl_up_sync(0xffffffffu, inc, 1);
			fex[b] = __shfl_up_sync(0xffffffffu, finc, 1);
			if (lane == 0) {
				ex[b] = 0;
				fex[b] = 0;
			}
			bs[b] = __shfl_sync(0xffffffffu, inc, 31);
			bf[b] = __shfl_sync(0xffffffffu, finc, 31);
		}
		if (lane == 0) {
			Acc ws = 0;
			uint32_t wf = 0;
#pragma unroll
			for (int b = 0; b < kBlocks; ++b) {
				ws = bf[b] ? bs[b] : ws + bs[b];
				wf |= bf[b];
			}
			s_wsum[warp] = ws;
			s_wflag[warp] = wf;
		}
		__syncthreads();
		const uint32_t next = s_next;
		const bool have_next = next < num_tiles;
		const bool next_full = have_next && full_tile(next);
		const uint64_t nseg = (uint64_t)next * kTile + (uint64_t)warp * kWarpElems;

		// ---- prefetch of the next tile and its head words ----------------
		BlockRegs<InT> r;
		uint32_t nhw = 0;
		if (next_full) {
			issue_loads<InT>(r, in, nseg, lane);
			nhw = heads[(nseg >> 5) + lane];
		}

		// ---- tile status, lookback (warp 0) ------------------------------
		if (warp == 0) {
			const Acc wt = lane < kWarps ? s_wsum[lane] : (Acc)0;
			const uint32_t wf = lane < kWarps ? s_wflag[lane] : 0u;
			Acc winc = wt;
			uint32_t wfinc = wf;
#pragma unroll
			for (int d = 1; d < kWarps; d <<= 1) {
				const Acc t = __shfl_up_sync(0xffffffffu, winc, d);
				const uint32_t tf = __shfl_up_sync(0xffffffffu, wfinc, d);
				if (lane >= d) {
					if (!wfinc) winc += t;
					wfinc |= tf;
				}
			}
			const Acc agg = __shfl_sync(0xffffffffu, winc, kWarps - 1);
			const uint32_t agg_f = __shfl_sync(0xffffffffu, wfinc, kWarps - 1);
			Acc wex = __shfl_up_sync(0xffffffffu, winc, 1);
			uint32_t wfex = __shfl_up_sync(0xffffffffu, wfinc, 1);
			if (lane == 0) {
				wex = 0;
				wfex = 0;
			}
			uint64_t *tw = ts.words + (size_t)tile * PT;
			// A tile holding a head knows its inclusive prefix at once.
			if (lane == 0 && !published) {
				if (agg_f || tile == 0) lb::publish<Acc>(tw + KW, agg);
				else lb::publish<Acc>(tw, agg);
			}
			// The carry from earlier tiles matters only when the tile's
			// first element is not a head.
			const uint32_t first_head = __shfl_sync(0xffffffffu, hb[0], 0) & 1u;
			Acc excl = 0;
			if (tile > 0 && !first_head) excl = lb::lookback_warp<Acc>(ts.words, tile, dev_status);
			if (lane == 0 && !agg_f && tile > 0) lb::publish<Acc>(tw + KW, excl + agg);
			if (lane < kWarps) {
				s_wsum[lane] = wex;
				s_wflag[lane] = wfex;
			}
			if (lane == 0) s_excl = excl;
		}
		// ---- the next tile's (head seen, sum since its last head) --------
		if (next_full) {
			// Last head in the warp's 1024 elements, +1 (0: none).
			const uint32_t mine = nhw ? (uint32_t)lane * 32u + 32u - (uint32_t)__clz(nhw) : 0u;
			const uint32_t last1 = __reduce_max_sync(0xffffffffu, mine);
			constexpr int EPC = BlockRegs<InT>::kEpc;
			Acc part = 0;
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
#pragma unroll
				for (int k = 0; k < BlockRegs<InT>::kPerLane; ++k) {
					const InT *e = reinterpret_cast<const InT *>(&r.v[b][k]);
					const uint32_t i0 = (uint32_t)(b * kBlock + (lane + 32 * k) * EPC);
#pragma unroll
					for (int q = 0; q < EPC; ++q)
						if (i0 + q + 1 >= last1) part += (Acc)(OutT)e[q];
				}
			part = lb::warp_sum<Acc>(part);
			if (lane == 0) {
				s_nsum[warp] = part;
				s_nflag[warp] = last1 != 0;
			}
		}
		__syncthreads();
		if (next_full && tid == 0) {
			Acc ns = 0;
			uint32_t nf = 0;
#pragma unroll
			for (int w = 0; w < kWarps; ++w) {
				ns = s_nflag[w] ? s_nsum[w] : ns + s_nsum[w];
				nf |= s_nflag[w];
			}
			uint64_t *nw = ts.words + (size_t)next * PT;
			if (nf) lb::publish<Acc>(nw + KW, ns);
			else lb::publish<Acc>(nw, ns);
		}

		// ---- outputs per block: second read, staged, coalesced stores ----
		Acc carry = s_wsum[warp] + (s_wflag[warp] ? (Acc)0 : s_excl);
#pragma unroll
		for (int b = 0; b < kBlocks; ++b) {
			const InT *sin = s_in + b * padded<InT>();
			Acc run = ex[b] + (fex[b] ? (Acc)0 : carry);
#pragma unroll
			for (int j = 0; j < kItems; ++j) {
				const int q = lane * kItems + j;
				const Acc v = (Acc)(OutT)sin[pidx<InT>(q)];
				if ((hb[b] >> j) & 1u) run = 0;
				s_out[pidx<OutT>(q)] = (OutT)run;
				run += v;
			}
			carry = bf[b] ? bs[b] : bs[b] + carry;
			__syncwarp();
			const uint64_t seg = wseg + (uint64_t)b * kBlock;
			if (vec_ok && seg >= lo && seg + kBlock <= hi && seg + kBlock <= n) {
				constexpr int EPC = 16 / sizeof(OutT);
				constexpr int CHUNKS = kBlock / EPC;
				uint4 *dst = reinterpret_cast<uint4 *>(out + seg);
#pragma unroll
				for (int c = lane; c < CHUNKS; c += 32) {
					uint4 v;
					OutT *e = reinterpret_cast<OutT *>(&v);
#pragma unroll
					for (int k = 0; k < EPC; ++k) e[k] = s_out[pidx<OutT>(c * EPC + k)];
					dev::st_stream_v4(dst + c, v);
				}
			} else {
				for (int i = lane; i < kBlock; i += 32) {
					const uint64_t g = seg + i;
					if (g < n && g >= lo && g < hi) out[g] = s_out[pidx<OutT>(i)];
				}
			}
			__syncwarp();
		}
		if (!have_next) break;

		// ---- the next tile into shared memory ----------------------------
		if (next_full) {
			store_loads<InT>(r, s_in, lane);
		} else {
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
				load_block_scalar<InT>(in, n, nseg + (uint64_t)b * kBlock, s_in + b * padded<InT>(), lane);
		}
		__syncwarp();
		published = next_full;
		tile = next;
	}
}

// Per device and type pair, once: the kernel's dynamic shared memory and
// its resident CTAs per SM (later calls, possibly during a graph capture,
// only read the cache).
template <typename InT, typename OutT>
cudaError_t seg_scan_prepare(int *per_sm) {
	static std::atomic<int> cached[64];
	static std::mutex mu;
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
	int v = cached[dev].load(std::memory_order_acquire);
	if (v == 0) {
		std::lock_guard<std::mutex> lk(mu);
		v = cached[dev].load(std::memory_order_relaxed);
		if (v == 0) {
			constexpr size_t smem = scantile::scan_smem<InT, OutT>();
			e = cudaFuncSetAttribute(seg_scan_lookback<InT, OutT>,
				cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
			if (e == cudaSuccess)
				e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, seg_scan_lookback<InT, OutT>,
					scantile::kThreads, smem);
			if (e != cudaSuccess) return e;
			if (v < 1) v = 1;
			cached[dev].store(v, std::memory_order_release);
		}
	}
	*per_sm = v;
	return cudaSuccess;
}

template <typename InT, typename OutT>
cudaError_t launch_seg_scan(const void *in, void *out, uint64_t n_cap,
	const uint64_t *off, uint32_t S, CCLContext *ctx, cudaStream_t s, GError **err) {
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t, uint64_t>::type;
	const uint64_t tiles = (n_cap + scantile::kTile - 1) / scantile::kTile;
	if (tiles >= (1ull << 31)) {
		set_error(err, CLO_ERROR_ARGS, "Segmented scan buffer of %llu elements is too large",
			(unsigned long long)n_cap);
		return cudaErrorInvalidValue;
	}
	// One bitmap word per 32 elements, plus one word of slack.
	const size_t words = (size_t)((n_cap + 31) / 32) + 1;
	const size_t bm_bytes = (words * 4 + 15) / 16 * 16;
	const size_t st_bytes = (size_t)tiles * lb::Slots<Acc>::kPerTile * 8;
	const size_t total = bm_bytes + st_bytes + 16;
	int per_sm = 1;
	cudaError_t e = seg_scan_prepare<InT, OutT>(&per_sm);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "segmented scan");
		return e;
	}
	char *tmp = (char *)tmp_alloc(ctx, total, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	uint32_t *bits = (uint32_t *)tmp;
	lb::TileStatus ts;
	ts.words = (uint64_t *)(tmp + bm_bytes);
	ts.counter = (uint32_t *)(tmp + bm_bytes + st_bytes);
	e = cudaMemsetAsync(tmp, 0, total, s);
	if (e == cudaSuccess) {
		const uint32_t grid = (uint32_t)std::min<uint64_t>(((uint64_t)S + 255) / 256,
			(uint64_t)ctx->sm_count * 8);
		seg_heads<<<std::max<uint32_t>(grid, 1), 256, 0, s>>>(off, S, n_cap, bits,
			ctx->d_status);
		e = cudaGetLastError();
	}
	const bool vec_ok = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
	if (e == cudaSuccess) {
		const unsigned grid = (unsigned)std::max<uint64_t>(1,
			std::min<uint64_t>(tiles, (uint64_t)per_sm * ctx->sm_count));
		KernelTimer t("seg_scan_lookback", s, (double)n_cap * (sizeof(InT) + sizeof(OutT)));
		seg_scan_lookback<InT, OutT><<<grid, scantile::kThreads, scantile::scan_smem<InT, OutT>(), s>>>(
			(const InT *)in, (OutT *)out, n_cap, bits, off, S, ts, ctx->d_status, vec_ok);
		t.stop();
		e = cudaGetLastError();
	}
	count_launches(2);
	tmp_free(tmp, s);
	if (e != cudaSuccess) cuda_ok(e, err, "segmented scan");
	return e;
}

template <typename InT>
cudaError_t seg_scan_out(const void *in, void *out, uint64_t n_cap, const uint64_t *off,
	uint32_t S, int out_bytes, CCLContext *ctx, cudaStream_t s, GError **err) {
	switch (out_bytes) {
	case 1: return launch_seg_scan<InT, uint8_t>(in, out, n_cap, off, S, ctx, s, err);
	case 2: return launch_seg_scan<InT, uint16_t>(in, out, n_cap, off, S, ctx, s, err);
	case 4: return launch_seg_scan<InT, uint32_t>(in, out, n_cap, off, S, ctx, s, err);
	case 8: return launch_seg_scan<InT, uint64_t>(in, out, n_cap, off, S, ctx, s, err);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported sum width %d", out_bytes);
	return cudaErrorInvalidValue;
}

// ------------------------------------------------ gather / scatter
// Each warp moves 512 consecutive elements of the contiguous buffer, lane l
// taking elements l, l + 32, ... (coalesced on both sides within a run):
// one binary search for the segment of the lane's first element, then
// forward.
constexpr int kGatherRun = 16;  // elements per lane per warp chunk

__device__ __forceinline__ uint32_t segment_of(const uint64_t *off, uint32_t k, uint64_t g) {
	// Largest i with off[i] <= g (off[0] = 0 <= g < off[k]).
	uint32_t lo = 0, hi = k;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (off[mid] <= g) lo = mid;
		else hi = mid;
	}
	return lo;
}

template <typename T, bool GATHER>
__global__ void __launch_bounds__(256) seg_move(T *flat, T *const *ptrs, const uint64_t *off,
	uint32_t k, uint64_t total) {
	constexpr uint64_t kChunk = 32 * kGatherRun;
	const uint32_t lane = threadIdx.x & 31u;
	const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
		 c * kChunk < total; c += warps) {
		const uint64_t g0 = c * kChunk + lane;
		if (g0 >= total) continue;
		uint32_t i = segment_of(off, k, g0);
		uint64_t start = off[i], next = off[i + 1];
		T *base = ptrs[i];
#pragma unroll 4
		for (int e = 0; e < kGatherRun; ++e) {
			const uint64_t g = g0 + (uint64_t)e * 32;
			if (g >= total) break;
			if (next <= g) {
				do {
					++i;
					next = off[i + 1];
				} while (next <= g);
				start = off[i];
				base = ptrs[i];
			}
			T *p = base + (g - start);
			if (GATHER) flat[g] = *p;
			else *p = flat[g];
		}
	}
}

template <bool GATHER>
cudaError_t seg_move_launch(void *flat, void *const *ptrs, const uint64_t *off, uint32_t k,
	uint64_t total, int eb, int sm_count, cudaStream_t s) {
	if (total == 0 || k == 0) return cudaSuccess;
	const uint64_t warps = (total + 32 * kGatherRun - 1) / (32 * kGatherRun);
	const unsigned grid = (unsigned)std::max<uint64_t>(1,
		std::min<uint64_t>((warps + 7) / 8, (uint64_t)sm_count * 16));
	switch (eb) {
	case 1: seg_move<uint8_t, GATHER><<<grid, 256, 0, s>>>((uint8_t *)flat, (uint8_t *const *)ptrs, off, k, total); break;
	case 2: seg_move<uint16_t, GATHER><<<grid, 256, 0, s>>>((uint16_t *)flat, (uint16_t *const *)ptrs, off, k, total); break;
	case 4: seg_move<uint32_t, GATHER><<<grid, 256, 0, s>>>((uint32_t *)flat, (uint32_t *const *)ptrs, off, k, total); break;
	case 8: seg_move<uint64_t, GATHER><<<grid, 256, 0, s>>>((uint64_t *)flat, (uint64_t *const *)ptrs, off, k, total); break;
	default: return cudaErrorInvalidValue;
	}
	count_launches(1);
	return cudaGetLastError();
}

}  // namespace

int seg_sort_num_variants() { return kSegVariants; }

cudaError_t seg_sort(void *keys, uint64_t n_cap, const uint64_t *off, size_t S,
	int key_bytes, int sort_bits, int variant, CCLContext *ctx, cudaStream_t s,
	GError **err, void *alt, bool *in_alt) {
	if (S >= (1ull << 31)) {
		set_error(err, CLO_ERROR_ARGS, "Too many segments (%zu)", S);
		return cudaErrorInvalidValue;
	}
	const uint32_t s32 = (uint32_t)S;
	switch (key_bytes) {
	case 1: return seg_sort_typed<uint8_t>((uint8_t *)keys, n_cap, off, s32, sort_bits, variant, ctx, s, err, (uint8_t *)alt, in_alt);
	case 2: return seg_sort_typed<uint16_t>((uint16_t *)keys, n_cap, off, s32, sort_bits, variant, ctx, s, err, (uint16_t *)alt, in_alt);
	case 4: return seg_sort_typed<uint32_t>((uint32_t *)keys, n_cap, off, s32, sort_bits, variant, ctx, s, err, (uint32_t *)alt, in_alt);
	case 8: return seg_sort_typed<uint64_t>((uint64_t *)keys, n_cap, off, s32, sort_bits, variant, ctx, s, err, (uint64_t *)alt, in_alt);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported key width %d", key_bytes);
	return cudaErrorInvalidValue;
}

cudaError_t seg_scan(const void *in, void *out, uint64_t n_cap, const uint64_t *off,
	size_t S, CloType in_type, int out_bytes, CCLContext *ctx, cudaStream_t s,
	GError **err) {
	if (S == 0 || n_cap == 0) return cudaSuccess;
	if (S >= (1ull << 31)) {
		set_error(err, CLO_ERROR_ARGS, "Too many segments (%zu)", S);
		return cudaErrorInvalidValue;
	}
	const uint32_t s32 = (uint32_t)S;
	switch (in_type) {
	case CLO_CHAR: return seg_scan_out<int8_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_UCHAR: return seg_scan_out<uint8_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_SHORT: return seg_scan_out<int16_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_USHORT: return seg_scan_out<uint16_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_INT: return seg_scan_out<int32_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_UINT: return seg_scan_out<uint32_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_LONG: return seg_scan_out<int64_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	case CLO_ULONG: return seg_scan_out<uint64_t>(in, out, n_cap, off, s32, out_bytes, ctx, s, err);
	default: break;
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported scan element type %d", (int)in_type);
	return cudaErrorInvalidValue;
}


cudaError_t seg_gather(void *dst, const void *const *srcs, const uint64_t *off, uint32_t k,
	uint64_t total, int elem_bytes, int sm_count, cudaStream_t s) {
	return seg_move_launch<true>(dst, const_cast<void *const *>(srcs), off, k, total,
		elem_bytes, sm_count, s);
}

cudaError_t seg_scatter(void *const *dsts, const void *src, const uint64_t *off, uint32_t k,
	uint64_t total, int elem_bytes, int sm_count, cudaStream_t s) {
	return seg_move_launch<false>(const_cast<void *>(src), dsts, off, k, total, elem_bytes,
		sm_count, s);
}

}  // namespace clo
