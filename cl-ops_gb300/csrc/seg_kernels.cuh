// Kernels of the segmented sort that depend on the key width: the CTA
// classes' shared-memory radix sorts and the long-segment onesweep pass,
// with the launchers seg_common.cuh declares. Included once per key width
// (seg_sort_k{1,2,4,8}.cu), each of which instantiates the launchers for
// its width.
#pragma once

#include <algorithm>
#include <type_traits>

#include "dev_common.cuh"
#include "seg_common.cuh"
#include "timing.h"

namespace clo {
namespace seg {
namespace {

template <typename K, int THREADS, int KPT, int RB>
struct CtaCfg {
	static constexpr int kR = 1 << RB;  // digits per local pass
	static constexpr int kWarps = THREADS / 32;
	static constexpr int kTile = THREADS * KPT;
	static constexpr int kDigitsPerThread = THREADS >= kR ? 1 : kR / THREADS;
	static constexpr int kDigitThreads = kR / kDigitsPerThread;
	static constexpr int kScanWarps = (kDigitThreads + 31) / 32;
	static size_t smem() {
		return (2 * (size_t)kWarps * kR + 64) * sizeof(uint32_t) +
			(size_t)kTile * sizeof(K);
	}
};

// One CTA per segment of the list: keys stay in registers (warp-striped,
// so index order is (warp, round, lane)); per RB-bit digit, per-warp counts,
// a block scan of the digit totals, stable ranks through shared-memory OR
// peer masks, and a pass through shared memory back to index order.
// Elements past the segment end are all-ones keys: they rank last in every
// digit, so they stay behind the segment and are never written. Warps whose
// keys all lie past the end take no part in the passes (their counts stay
// zero), so a segment pays only for the warps it fills.
template <typename K, int THREADS, int KPT, int RB>
__global__ void __launch_bounds__(THREADS) seg_sort_cta(K *keys, const uint64_t *off,
	const uint32_t *list, const uint32_t *count, int passes) {
	using Cfg = CtaCfg<K, THREADS, KPT, RB>;
	constexpr int R = Cfg::kR;
	constexpr int W = Cfg::kWarps;
	constexpr int TILE = Cfg::kTile;
	constexpr int DPT = Cfg::kDigitsPerThread;
	constexpr int DT = Cfg::kDigitThreads;
	extern __shared__ __align__(16) unsigned char smem[];
	uint32_t *s_hist = reinterpret_cast<uint32_t *>(smem);  // [W][R]
	uint32_t *s_match = s_hist + W * R;                     // [W][R]
	uint32_t *s_misc = s_match + W * R;                     // [64]
	K *sk = reinterpret_cast<K *>(s_misc + 64);             // [TILE]

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	uint32_t *my_hist = s_hist + warp * R;
	uint32_t *my_match = s_match + warp * R;
	const uint32_t lt = dev::lanemask_lt();
	for (int i = lane; i < R; i += 32) my_match[i] = 0;
	auto dig = [](K key, int shift) { return (uint32_t)(key >> shift) & (uint32_t)(R - 1); };
	const uint32_t cnt = *count;
	const uint32_t wb = (uint32_t)warp * (KPT * 32);

	for (uint32_t li = blockIdx.x; li < cnt; li += gridDim.x) {
		const uint32_t s = list[li];
		const uint64_t base = off[s];
		const uint32_t len = (uint32_t)(off[s + 1] - base);
		// Warps holding part of the segment, and the keys they hold.
		const bool active = wb < len;
		const uint32_t held = std::min<uint32_t>(TILE, (len + KPT * 32 - 1) / (KPT * 32) * (KPT * 32));
		K k[KPT];
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			const uint32_t idx = wb + j * 32 + lane;
			k[j] = idx < len ? keys[base + idx] : (K)~(K)0;
		}
		for (int p = 0; p < passes; ++p) {
			const int shift = p * RB;
			for (int i = lane; i < R; i += 32) my_hist[i] = 0;
			__syncwarp();
			if (active) {
#pragma unroll
				for (int j = 0; j < KPT; ++j) atomicAdd(my_hist + dig(k[j], shift), 1u);
			}
			__syncthreads();
			// Digit totals (DPT consecutive digits per thread), the scan of
			// the threads' sums within each warp, and whether one digit holds
			// every key (then this digit leaves the order unchanged).
			uint32_t tot[DPT];
			uint32_t tsum = 0, tinc = 0;
			bool triv = false;
			if (warp < Cfg::kScanWarps) {  // whole warps; lanes past DT hold zeros
				if (tid < DT) {
#pragma unroll
					for (int q = 0; q < DPT; ++q) {
						const int d = tid * DPT + q;
						uint32_t c = 0;
#pragma unroll
						for (int w = 0; w < W; ++w) c += s_hist[w * R + d];
						tot[q] = c;
						tsum += c;
						triv = triv || c == (d == R - 1 ? held : len);
					}
				}
				tinc = tsum;
#pragma unroll
				for (int d = 1; d < 32; d <<= 1) {
					const uint32_t t = __shfl_up_sync(0xffffffffu, tinc, d);
					if (lane >= d) tinc += t;
				}
				if (lane == 31) s_misc[warp] = tinc;
			}
			if (__syncthreads_or(triv)) continue;
			if (tid < DT) {
				uint32_t run = tinc - tsum;
				for (int w = 0; w < warp; ++w) run += s_misc[w];
#pragma unroll
				for (int q = 0; q < DPT; ++q) {
					const int d = tid * DPT + q;
					uint32_t r = run;
#pragma unroll
					for (int w = 0; w < W; ++w) {
						const uint32_t c = s_hist[w * R + d];
						s_hist[w * R + d] = r;
						r += c;
					}
					run += tot[q];
				}
			}
			__syncthreads();
			if (active) {
#pragma unroll
				for (int j = 0; j < KPT; ++j) {
					sk[dev::warp_rank_digit(my_match, my_hist, dig(k[j], shift), lane, lt)] = k[j];
				}
			}
			__syncthreads();
			if (active) {
#pragma unroll
				for (int j = 0; j < KPT; ++j) k[j] = sk[wb + j * 32 + lane];
			}
		}
#pragma unroll
		for (int j = 0; j < KPT; ++j) {
			const uint32_t idx = wb + j * 32 + lane;
			if (idx < len) keys[base + idx] = k[j];
		}
		__syncthreads();
	}
}

// ------------------------------------------------------ large segments
// Reads tiles base, base-1, ... (W of them, one round trip) for one digit
// and adds them to `excl` up to the first inclusive prefix.
template <int W>
__device__ __forceinline__ bool seg_lookback_window(const uint32_t *status, int digit,
	long long &base, uint32_t &excl) {
	uint32_t sv[W];
#pragma unroll
	for (int i = 0; i < W; ++i) {
		const long long j = base - i;
		sv[i] = j >= 0 ? dev::ld_relaxed_u32(status + (size_t)j * kRadix + digit) : kStPrefix;
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

// Ranking rows (one per half-warp unit) and count rows: 256 digits each,
// 264 words apart, odd rows 8 words later, so the two units of a warp hold
// a digit 16 banks apart.
constexpr int kSegRowWords = kRadix + 8;
__device__ __forceinline__ int seg_row(int r) { return r * kSegRowWords + (r & 1) * 8; }
constexpr int kLUnits = 2 * kLWarps;  // 16 half-warp units per tile
constexpr int kSegLookWindow = 8;     // predecessor statuses per round trip

// One pass over all tiles of all large segments, by persistent CTAs that
// take tiles in order from a counter (the next tile and its descriptor are
// claimed during the write-out). Per tile as the plain sort's pass: keys
// loaded in half-warp units (a unit's (round, lane) order is index order),
// unit counts in 16-bit halves of 8 count rows (units u and u + 8 share
// row u), the tile's counts published before it is ranked (a segment's
// first tile publishes an inclusive prefix at once, so lookbacks stop at
// the segment's start), ranking with dev::unit_rank_digit (the unit's word
// per digit holds its next tile position in the upper 16 bits and the
// round's peer mask in the lower 16), staging, then a lookback in windows
// of kSegLookWindow and a write-out with one base per digit.
template <typename K, int KPT>
__global__ void __launch_bounds__(kLThreads, 2)
seg_pass(const K *__restrict__ kin, K *__restrict__ kout, SegPassArgs a) {
	constexpr int TILE = kLThreads * KPT;
	constexpr int UKEYS = 16 * KPT;          // a unit's keys in one tile
	constexpr int HALF = kLUnits / 2;        // 8 count rows
	static_assert(TILE <= 0xFFFF, "16-bit unit and tile counts");
	extern __shared__ __align__(16) unsigned char smem[];
	uint32_t *s_rank = reinterpret_cast<uint32_t *>(smem);     // [16] rows
	uint32_t *s_cnt = s_rank + kLUnits * kSegRowWords;         // [8] rows
	uint32_t *s_tile_off = s_cnt + HALF * kSegRowWords;        // [256]
	uint32_t *s_part = s_tile_off + kRadix;                    // [256]
	uint32_t *s_misc = s_part + kRadix;                        // [64]
	uint64_t *s_seg = reinterpret_cast<uint64_t *>(s_misc + 64);  // [2]
	unsigned char *s_stage = reinterpret_cast<unsigned char *>(s_seg + 2);

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int unit = 2 * warp + (lane >> 4);
	const uint32_t l16 = lane & 15;
	const uint32_t lt16 = (1u << l16) - 1u;
	uint32_t *my_rank = s_rank + seg_row(unit);
	uint32_t *my_cnt = s_cnt + seg_row(unit % HALF);
	const uint32_t cnt_inc = 1u << ((unit / HALF) * 16);
	const int pd = tid;        // the digit this thread scans
	const int dw = tid >> 5;   // the warp that owns digit pd
	const int shift = a.shift;
#pragma unroll
	for (int i = 0; i < HALF; ++i) s_cnt[seg_row(i) + pd] = 0;
	const uint32_t T = (uint32_t)(a.tstart[a.S] >> 32);
	// Thread 0 takes the next tile and its descriptor (one round trip after
	// the claim); after the first tile this overlaps the write-out.
	auto claim = [&]() {
		const uint32_t t = atomicAdd(a.counter, 1u);
		s_misc[0] = t;
		if (t < T) {
			const ulonglong2 span = a.tile_span[t];
			const uint2 x = a.tile_x[t];
			s_misc[1] = x.x;   // tile index within the segment
			s_misc[2] = x.y;   // large-segment rank
			s_seg[0] = span.x;
			s_seg[1] = span.y;
		}
	};
	if (tid == 0) claim();
	__syncthreads();

	for (;;) {
		const uint32_t tile = s_misc[0];
		if (tile >= T) break;
		const uint32_t ti = s_misc[1];
		const uint32_t lr = s_misc[2];
		const uint64_t seg_a = s_seg[0], seg_e = s_seg[1];
		// One copy of the tile's steps for full tiles and one for a
		// segment's partial last tile.
		auto do_tile = [&](auto partial_tag) {
			constexpr bool PARTIAL = decltype(partial_tag)::value;
			const uint64_t ubase = seg_a + (uint64_t)ti * TILE + (uint64_t)unit * UKEYS;

			// A segment's last tile is partial: its keys past the segment's end
			// are neither counted nor ranked, and rounds wholly past the end
			// are skipped by the whole warp (the upper unit of a warp never
			// holds a key below the lower unit's). Full tiles take none of
			// these tests.
			uint32_t nvalid = UKEYS, wvalid = UKEYS;
			if constexpr (PARTIAL) {
				const int64_t left = (int64_t)(seg_e - ubase);
				nvalid = left <= 0 ? 0u : left >= UKEYS ? (uint32_t)UKEYS : (uint32_t)left;
				wvalid = __shfl_sync(0xffffffffu, nvalid, 0);
			}
			K k[KPT];
#pragma unroll
			for (int j = 0; j < KPT; ++j) {
				const uint64_t idx = ubase + (uint64_t)j * 16 + l16;
				if constexpr (PARTIAL) k[j] = idx < seg_e ? kin[idx] : (K)~(K)0;
				else k[j] = kin[idx];
			}
			// Digit base within the segment: exclusive scan of its histogram.
			const uint32_t hv = a.seg_hist[(size_t)lr * a.hist_stride + pd];
			uint32_t hinc = hv;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				const uint32_t t = __shfl_up_sync(0xffffffffu, hinc, d);
				if (lane >= d) hinc += t;
			}
			if (lane == 31) s_misc[16 + dw] = hinc;
#pragma unroll
			for (int j = 0; j < KPT; ++j)
				if (!PARTIAL || (uint32_t)j * 16 + l16 < nvalid)
					atomicAdd(my_cnt + digit_of(k[j], shift), cnt_inc);
			__syncthreads();
			uint32_t gbase = hinc - hv;
#pragma unroll
			for (int w = 0; w < 8; ++w)
				if (w < dw) gbase += s_misc[16 + w];
			// Unit prefixes of digit pd in unit order (low halves: units
			// 0..7, high halves: units 8..15); rows cleared as they are read.
			uint32_t c2[HALF];
#pragma unroll
			for (int i = 0; i < HALF; ++i) {
				c2[i] = s_cnt[seg_row(i) + pd];
				s_cnt[seg_row(i) + pd] = 0;
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
			uint32_t *st = a.status + (size_t)tile * kRadix + pd;
			dev::st_relaxed_u32(st, (ti == 0 ? kStPrefix : kStAgg) | sum);
			a.status_next[(size_t)tile * kRadix + pd] = 0;
			{
				uint32_t inc = sum;
#pragma unroll
				for (int d = 1; d < 32; d <<= 1) {
					const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
					if (lane >= d) inc += t;
				}
				if (lane == 31) s_misc[8 + dw] = inc;
				s_part[pd] = inc - sum;
			}
			__syncthreads();
			uint32_t to = s_part[pd];
#pragma unroll
			for (int w = 0; w < 8; ++w)
				if (w < dw) to += s_misc[8 + w];
#pragma unroll
			for (int i = 0; i < HALF; ++i) {
				s_rank[seg_row(i) + pd] = (to + (c2[i] & 0xFFFFu)) << 16;
				s_rank[seg_row(i + HALF) + pd] = (to + (c2[i] >> 16)) << 16;
			}
			__syncthreads();
			K *sk = reinterpret_cast<K *>(s_stage);
#pragma unroll
			for (int j = 0; j < KPT; ++j) {
				if (!PARTIAL || (uint32_t)j * 16 < wvalid) {
					const uint32_t pos = dev::unit_rank_digit(my_rank + digit_of(k[j], shift), l16,
						lt16);
					if (pos < (uint32_t)TILE) sk[pos] = k[j];
				}
			}
			// Lookback over the segment's preceding tiles (bounded waits).
			uint32_t excl = 0;
			if (ti > 0) {
				long long base = (long long)tile - 1;
				uint32_t iter = 0;
				bool done = seg_lookback_window<kSegLookWindow>(a.status, pd, base, excl);
				while (!done && base >= 0) {
					uint32_t sv = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
					while ((sv & ~kStValue) == 0) {
						if (++iter >= dev::kSpinLimit) break;
						dev::backoff(iter);
						sv = dev::ld_relaxed_u32(a.status + (size_t)base * kRadix + pd);
					}
					if ((sv & ~kStValue) == 0) {
						dev::report_timeout(a.dev_status, DEV_ERR_LOOKBACK_TIMEOUT, (int)tile);
						break;
					}
					done = seg_lookback_window<kSegLookWindow>(a.status, pd, base, excl);
				}
				dev::st_relaxed_u32(st, kStPrefix | (excl + sum));
			}
			// Output offset (within the segment) of staged position q of digit
			// d is q + G[d] (modulo 2^32).
			s_tile_off[pd] = gbase + excl - to;
			__syncthreads();
			if (tid == 0) claim();
			const uint32_t tile_keys = PARTIAL ? (uint32_t)(seg_e - (seg_a + (uint64_t)ti * TILE))
				: (uint32_t)TILE;
#pragma unroll
			for (int i = 0; i < KPT; ++i) {
				const int q = i * kLThreads + tid;
				if (PARTIAL && (uint32_t)q >= tile_keys) continue;
				const K key = sk[q];
				const uint64_t o = seg_a + (uint32_t)(s_tile_off[digit_of(key, shift)] + (uint32_t)q);
				if (o < seg_e) kout[o] = key;
			}
		};
		if (seg_e - (seg_a + (uint64_t)ti * TILE) >= (uint64_t)TILE) do_tile(std::false_type{});
		else do_tile(std::true_type{});
		__syncthreads();
	}
}

template <typename K, int KPT>
size_t seg_pass_smem() {
	return ((size_t)(kLUnits + kLUnits / 2) * kSegRowWords + 3 * kRadix + 64) * sizeof(uint32_t) +
		2 * sizeof(uint64_t) + (size_t)kLThreads * KPT * sizeof(K);
}


template <typename K, int THREADS, int KPT, int RB>
cudaError_t launch_cta_class(K *keys, const uint64_t *off, const uint32_t *list,
	const uint32_t *count, int sort_bits, uint32_t max_blocks, CCLContext *ctx,
	cudaStream_t s) {
	using Cfg = CtaCfg<K, THREADS, KPT, RB>;
	const size_t smem = Cfg::smem();
	auto kern = seg_sort_cta<K, THREADS, KPT, RB>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	if (e != cudaSuccess) return e;
	int occ = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, smem);
	if (e != cudaSuccess) return e;
	uint32_t grid = (uint32_t)std::max(1, occ) * (uint32_t)ctx->sm_count;
	if (grid > max_blocks) grid = std::max<uint32_t>(max_blocks, 1);
	KernelTimer t("seg_sort_cta", s, 0.0);
	kern<<<grid, THREADS, smem, s>>>(keys, off, list, count, sort_bits / RB);
	t.stop();
	count_launches(1);
	return cudaGetLastError();
}

template <typename K, int THREADS, int KPT>
cudaError_t launch_cta_rb(int rb, K *keys, const uint64_t *off, const uint32_t *list,
	const uint32_t *count, int sort_bits, uint32_t max_blocks, CCLContext *ctx,
	cudaStream_t s) {
	return rb == 4
		? launch_cta_class<K, THREADS, KPT, 4>(keys, off, list, count, sort_bits, max_blocks, ctx, s)
		: launch_cta_class<K, THREADS, KPT, 8>(keys, off, list, count, sort_bits, max_blocks, ctx, s);
}

template <typename K, int KPT>
cudaError_t launch_pass_kpt(const K *src, K *dst, const SegPassArgs &pa, uint64_t t_bound,
	CCLContext *ctx, cudaStream_t s) {
	const size_t smem = seg_pass_smem<K, KPT>();
	auto kern = seg_pass<K, KPT>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
		(int)smem);
	int occ = 0;
	if (e == cudaSuccess)
		e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kLThreads, smem);
	if (e != cudaSuccess) return e;
	const uint32_t grid = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(t_bound, 1),
		(uint64_t)std::max(occ, 1) * ctx->sm_count);
	KernelTimer t("seg_pass", s, 0.0);
	kern<<<grid, kLThreads, smem, s>>>(src, dst, pa);
	t.stop();
	count_launches(1);
	return cudaGetLastError();
}

}  // namespace

template <typename K>
cudaError_t seg_launch_cta_classes(const SegShape &sh, K *keys, const uint64_t *off,
	const uint32_t *lists, const uint32_t *counts, uint32_t S, int sort_bits,
	uint64_t n_cap, CCLContext *ctx, cudaStream_t s) {
	constexpr int DIV = sizeof(K) > 4 ? 2 : 1;
	// Blocks beyond the number of segments that can exist would only exit.
	auto cap = [&](uint64_t shorter) {
		return (uint32_t)std::min<uint64_t>(S, n_cap / (shorter + 1) + 1);
	};
	const uint32_t *la = lists + (size_t)S, *lb = lists + 2 * (size_t)S;
	const uint32_t max_a = class_a_max<K>(sh);
	cudaError_t e;
	if (sh.a_threads == 256)
		e = launch_cta_rb<K, 256, 8 / DIV>(sh.rb, keys, off, la, counts + 1, sort_bits, cap(32),
			ctx, s);
	else
		e = launch_cta_rb<K, 128, 8 / DIV>(sh.rb, keys, off, la, counts + 1, sort_bits, cap(32),
			ctx, s);
	if (e != cudaSuccess) return e;
	switch (sh.b_threads) {
	case 256:
		return launch_cta_rb<K, 256, 16 / DIV>(sh.rb, keys, off, lb, counts + 2, sort_bits,
			cap(max_a), ctx, s);
	case 1024:
		return launch_cta_rb<K, 1024, 16 / DIV>(sh.rb, keys, off, lb, counts + 2, sort_bits,
			cap(max_a), ctx, s);
	default:
		return launch_cta_rb<K, 512, 16 / DIV>(sh.rb, keys, off, lb, counts + 2, sort_bits,
			cap(max_a), ctx, s);
	}
}

template <typename K>
cudaError_t seg_launch_pass(const SegShape &sh, const K *src, K *dst, const SegPassArgs &pa,
	uint64_t t_bound, CCLContext *ctx, cudaStream_t s) {
	switch (sh.long_idx) {
	case 1: return launch_pass_kpt<K, long_kpt<K>(1)>(src, dst, pa, t_bound, ctx, s);
	case 2: return launch_pass_kpt<K, long_kpt<K>(2)>(src, dst, pa, t_bound, ctx, s);
	default: return launch_pass_kpt<K, long_kpt<K>(0)>(src, dst, pa, t_bound, ctx, s);
	}
}

}  // namespace seg
}  // namespace clo
