// Tile layout of the decoupled-lookback scans (plain and segmented):
// 8192-element tiles, 256 threads; each warp owns 1024 consecutive
// elements as two blocks of 512, lane l holding elements 16 l .. 16 l + 15
// of each block. A block moves between global and shared memory with
// coalesced 16-byte vector accesses through a padded transpose, and the
// next tile's blocks can be prefetched into registers (BlockRegs) while the
// current tile waits on its lookback.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include "dev_common.cuh"

namespace clo {
namespace scantile {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;                       // a lane's run in one block
constexpr int kBlock = 32 * kItems;              // 512 elements
constexpr int kBlocks = 2;                       // blocks per warp
constexpr int kWarpElems = kBlocks * kBlock;     // 1024
constexpr int kTile = kWarps * kWarpElems;       // 8192
// A block in shared memory is padded by one element per 128 bytes
// (per 32 elements of 4 bytes or fewer, per 16 of 8 bytes), so both the
// lanes' 16-element runs and the 16-byte vector columns are conflict-free.
template <typename T>
__host__ __device__ constexpr int pad_shift() { return sizeof(T) == 8 ? 4 : 5; }
template <typename T>
__host__ __device__ constexpr int padded() { return kBlock + (kBlock >> pad_shift<T>()); }
template <typename T>
__device__ __forceinline__ int pidx(int i) { return i + (i >> pad_shift<T>()); }

// Shared memory of one CTA: per warp, its two input blocks and one output
// staging block.
template <typename InT, typename OutT>
constexpr size_t scan_smem() {
	return (size_t)kWarps * (kBlocks * padded<InT>() * sizeof(InT) + padded<OutT>() * sizeof(OutT));
}

// Resident CTAs per SM (228 KB per SM, 1 KB reserved per CTA), at most 4,
// and at most 2 for 8-byte inputs (their prefetch takes 64 registers).
template <typename InT, typename OutT>
constexpr int scan_min_blocks() {
	constexpr int by_smem = (int)((228 * 1024) / (scan_smem<InT, OutT>() + 1024 + 128));
	constexpr int cap = sizeof(InT) == 8 ? 2 : 4;
	return by_smem < cap ? by_smem : cap;
}

// One warp's block b of a tile, global -> padded shared memory.
template <typename InT>
__device__ __forceinline__ void load_block_scalar(const InT *__restrict__ in, size_t n,
	size_t seg, InT *sin, int lane) {
	for (int i = lane; i < kBlock; i += 32)
		sin[pidx<InT>(i)] = (seg + i < n) ? in[seg + i] : (InT)0;
}

template <typename InT>
struct BlockRegs {
	static constexpr int kEpc = 16 / sizeof(InT);          // elements per 16 B
	static constexpr int kPerLane = kBlock / kEpc / 32;    // 16-byte loads per lane
	uint4 v[kBlocks][kPerLane];
};

// Issues the 16-byte loads of a warp's full blocks (prefetch).
template <typename InT>
__device__ __forceinline__ void issue_loads(BlockRegs<InT> &r, const InT *__restrict__ in,
	size_t wseg, int lane) {
#pragma unroll
	for (int b = 0; b < kBlocks; ++b) {
		const uint4 *src = reinterpret_cast<const uint4 *>(in + wseg + (size_t)b * kBlock);
#pragma unroll
		for (int k = 0; k < BlockRegs<InT>::kPerLane; ++k)
			r.v[b][k] = dev::ld_stream_v4(src + lane + 32 * k);
	}
}

// Transposes prefetched loads into the warp's padded blocks.
template <typename InT>
__device__ __forceinline__ void store_loads(const BlockRegs<InT> &r, InT *s_in, int lane) {
	constexpr int EPC = BlockRegs<InT>::kEpc;
#pragma unroll
	for (int b = 0; b < kBlocks; ++b) {
		InT *sin = s_in + b * padded<InT>();
#pragma unroll
		for (int k = 0; k < BlockRegs<InT>::kPerLane; ++k) {
			const int c = lane + 32 * k;
			const InT *e = reinterpret_cast<const InT *>(&r.v[b][k]);
#pragma unroll
			for (int q = 0; q < EPC; ++q) sin[pidx<InT>(c * EPC + q)] = e[q];
		}
	}
}

}  // namespace scantile
}  // namespace clo
