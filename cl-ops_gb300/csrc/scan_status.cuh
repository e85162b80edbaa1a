// Tile status words of the decoupled-lookback scans (plain and segmented).
//
// No fences are needed: every value is published once into its own slot of
// 64-bit words, each word carrying a ready bit (bit 0) and 32 payload bits
// (bits 32..63). A word is either still zero or final, so a reader that
// sees every word of a slot ready has the whole value. Per tile:
// [aggregate slot][inclusive-prefix slot].
#pragma once

#include <stdint.h>

#include "clo_internal.h"
#include "dev_common.cuh"

namespace clo {
namespace lb {

template <typename Acc>
struct Slots {
	static constexpr int kWords = sizeof(Acc) / 4;
	static constexpr int kPerTile = 2 * kWords;
};

template <typename Acc>
__device__ __forceinline__ void publish(uint64_t *w, Acc v) {
#pragma unroll
	for (int i = 0; i < Slots<Acc>::kWords; ++i)
		dev::st_relaxed_u64(w + i, ((uint64_t)(uint32_t)((uint64_t)v >> (32 * i)) << 32) | 1ull);
}

// 0 = nothing published, 1 = aggregate, 2 = inclusive prefix.
template <typename Acc>
__device__ __forceinline__ uint32_t read_status(const uint64_t *tile_words, Acc &v) {
	constexpr int W = Slots<Acc>::kWords;
	uint64_t a[W], p[W];
#pragma unroll
	for (int i = 0; i < W; ++i) {
		a[i] = dev::ld_relaxed_u64(tile_words + i);
		p[i] = dev::ld_relaxed_u64(tile_words + W + i);
	}
	bool pr = true, ar = true;
	uint64_t pv = 0, av = 0;
#pragma unroll
	for (int i = 0; i < W; ++i) {
		pr = pr && (p[i] & 1ull);
		ar = ar && (a[i] & 1ull);
		pv |= (p[i] >> 32) << (32 * i);
		av |= (a[i] >> 32) << (32 * i);
	}
	if (pr) {
		v = (Acc)pv;
		return 2;
	}
	if (ar) {
		v = (Acc)av;
		return 1;
	}
	return 0;
}

struct TileStatus {
	uint64_t *words;     // tiles * Slots<Acc>::kPerTile
	uint32_t *counter;   // dynamic tile ids
};

template <typename Acc>
__device__ __forceinline__ Acc warp_sum(Acc v) {
#pragma unroll
	for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
	return v;
}

// Exclusive prefix of the tile `tile` from its predecessors' statuses,
// computed by one full warp: a window of 64 predecessors per round trip
// (lane l covers tiles pred - l and pred - 32 - l), summing aggregates up
// to and including the nearest inclusive prefix. Waits are bounded: a
// predecessor that never publishes is recorded in dev_status and counted
// as a zero prefix so the kernel ends. Every lane returns the sum.
template <typename Acc>
__device__ __forceinline__ Acc lookback_warp(const uint64_t *words, uint32_t tile,
	int *dev_status) {
	constexpr int PT = Slots<Acc>::kPerTile;
	const int lane = threadIdx.x & 31;
	Acc excl = 0;
	long long pred = (long long)tile - 1;
	for (;;) {
		const long long t0 = pred - lane, t1 = pred - 32 - lane;
		Acc v0 = 0, v1 = 0;
		uint32_t s0 = t0 >= 0 ? read_status<Acc>(words + (size_t)t0 * PT, v0) : 2u;
		uint32_t s1 = t1 >= 0 ? read_status<Acc>(words + (size_t)t1 * PT, v1) : 2u;
		uint32_t iter = 0;
		while (__any_sync(0xffffffffu, s0 == 0 || s1 == 0)) {
			if (iter >= dev::kSpinLimit) {
				if (s0 == 0 || s1 == 0)
					dev::report_timeout(dev_status, DEV_ERR_LOOKBACK_TIMEOUT, (int)tile);
				if (s0 == 0) { s0 = 2; v0 = 0; }
				if (s1 == 0) { s1 = 2; v1 = 0; }
				continue;
			}
			dev::backoff(iter);
			if (s0 == 0) s0 = read_status<Acc>(words + (size_t)t0 * PT, v0);
			if (s1 == 0) s1 = read_status<Acc>(words + (size_t)t1 * PT, v1);
			++iter;
		}
		uint32_t pm = __ballot_sync(0xffffffffu, s0 == 2);
		if (pm) {
			const int first = __ffs(pm) - 1;
			excl += warp_sum<Acc>(lane <= first ? v0 : (Acc)0);
			break;
		}
		excl += warp_sum<Acc>(v0);
		pm = __ballot_sync(0xffffffffu, s1 == 2);
		if (pm) {
			const int first = __ffs(pm) - 1;
			excl += warp_sum<Acc>(lane <= first ? v1 : (Acc)0);
			break;
		}
		excl += warp_sum<Acc>(v1);
		pred -= 64;
	}
	return excl;
}

}  // namespace lb
}  // namespace clo
