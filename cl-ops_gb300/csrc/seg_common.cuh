// Declarations shared by the segmented sort's driver (segmented.cu) and its
// per-key-width kernel units (seg_sort_k{1,2,4,8}.cu, built from
// seg_kernels.cuh so that the widths compile in parallel).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "clo_internal.h"

namespace clo {
namespace seg {

constexpr int kRadix = 256;
constexpr int kRadixBits = 8;
constexpr uint32_t kMaxSegLen = (1u << 30) - 1u;

// Large-segment pass: 256 threads (one per digit in the per-tile scans),
// 2 CTAs per SM, keys per thread from the shape below.
constexpr int kLThreads = 256;
constexpr int kLWarps = kLThreads / 32;

// Tile status word of the large-segment pass: 2-bit flag | 30-bit count.
constexpr uint32_t kStAgg = 1u << 30;
constexpr uint32_t kStPrefix = 2u << 30;
constexpr uint32_t kStValue = (1u << 30) - 1u;

template <typename K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift) {
	return (uint32_t)(k >> shift) & (kRadix - 1);
}

// ------------------------------------------------------------ shapes
// The segmented sort's tunable shape, four choices the autotuner searches
// (each list's first entry is the default):
//   class A CTA layout    (threads, keys per thread): 128 x 8, 256 x 8
//   class B CTA layout    512 x 16, 256 x 16, 1024 x 16
//   long-segment pass     keys per thread of 256-thread tiles: 56, 48, 40
//                         (8-byte keys: 32, 28, 24)
//   CTA classes' digits   8 or 4 bits per local LSD pass
// Keys of 8 bytes halve the CTA classes' keys per thread. The class
// boundaries follow from the layouts: a segment goes to the warp class up
// to 32 keys, to class A up to A's tile, to class B up to B's tile, and to
// the long-segment passes beyond.
struct SegShape {
	int a_threads, a_kpt, b_threads, b_kpt;
	int long_idx;  // index into the long-pass keys-per-thread lists
	int rb;        // digit bits of the CTA classes
};
constexpr int kSegA = 2, kSegB = 3, kSegL = 3, kSegRB = 2;
constexpr int kSegVariants = kSegA * kSegB * kSegL * kSegRB;

// variant = ((a * kSegB + b) * kSegL + l) * kSegRB + d
inline SegShape seg_shape(int v) {
	static const int A[kSegA][2] = {{128, 8}, {256, 8}};
	static const int B[kSegB][2] = {{512, 16}, {256, 16}, {1024, 16}};
	static const int RB[kSegRB] = {8, 4};
	if (v < 0 || v >= kSegVariants) v = 0;
	const int d = v % kSegRB;
	v /= kSegRB;
	const int l = v % kSegL;
	v /= kSegL;
	const int b = v % kSegB;
	const int a = v / kSegB;
	return SegShape{A[a][0], A[a][1], B[b][0], B[b][1], l, RB[d]};
}

// Keys per thread and tile of the long-segment pass.
template <typename K>
constexpr int long_kpt(int idx) {
	return sizeof(K) <= 4 ? (idx == 0 ? 56 : idx == 1 ? 48 : 40)
						  : (idx == 0 ? 32 : idx == 1 ? 28 : 24);
}
template <typename K>
constexpr uint32_t long_tile(int idx) {
	return (uint32_t)(kLThreads * long_kpt<K>(idx));
}

// Largest segment of class A / class B for key type K under a shape.
template <typename K>
uint32_t class_a_max(const SegShape &sh) {
	return (uint32_t)(sh.a_threads * (sh.a_kpt / (sizeof(K) > 4 ? 2 : 1)));
}
template <typename K>
uint32_t class_b_max(const SegShape &sh) {
	return (uint32_t)(sh.b_threads * (sh.b_kpt / (sizeof(K) > 4 ? 2 : 1)));
}

struct SegPassArgs {
	const uint64_t *off;
	const uint64_t *tstart;
	const uint32_t *tile_seg;
	const ulonglong2 *tile_span;  // segment [start, end) of each tile
	const uint2 *tile_x;          // (tile index within the segment, rank)
	const uint32_t *seg_hist;  // + pass * 256; stride passes * 256 per segment
	uint32_t hist_stride;
	uint32_t *status;
	uint32_t *status_next;
	uint32_t *counter;
	int *dev_status;
	uint32_t S;
	int shift;
};

// The CTA-class sorts of classes A and B (lists[S], lists[2S] with
// counts[1], counts[2]) under a shape. Defined per key width in
// seg_sort_k{1,2,4,8}.cu.
template <typename K>
cudaError_t seg_launch_cta_classes(const SegShape &sh, K *keys, const uint64_t *off,
	const uint32_t *lists, const uint32_t *counts, uint32_t S, int sort_bits,
	uint64_t n_cap, CCLContext *ctx, cudaStream_t s);

// One long-segment pass (persistent CTAs over every tile of every long
// segment) with the shape's tile size; grid at most t_bound CTAs.
template <typename K>
cudaError_t seg_launch_pass(const SegShape &sh, const K *src, K *dst, const SegPassArgs &pa,
	uint64_t t_bound, CCLContext *ctx, cudaStream_t s);

}  // namespace seg
}  // namespace clo
