// Exclusive prefix sum ("blelloch" scanner) as one single-pass kernel with
// decoupled lookback.
//
// Semantics follow src/cl_ops/scan/clo_scan_blelloch.cl:49-211: out[0] = 0
// and out[i] = sum_{j<i} (SUM_TYPE) in[j], with the element converted to
// the sum type by C rules and the sum wrapping modulo 2^(8*sizeof(SUM)).
// Integer addition is associative, so the result is bit-identical to the
// reference's work-group Blelloch trees whatever the summation order.
//
// Layout: tiles of 8192 elements, 256 threads. Each warp owns 1024
// consecutive elements as two blocks of 512, lane l holding elements
// 16 l .. 16 l + 15 of each block. A block moves between global memory and
// shared memory with coalesced 16-byte vector accesses through a padded
// transpose (conflict-free per-lane runs). Inputs stay in shared memory:
// the thread and warp sums are taken before the lookback and the outputs
// are formed by a second read after it, so no per-element state is held
// in registers across the wait. Tiles take ids from an atomic counter (so
// a tile only ever waits on tiles already running), publish their
// aggregate, then warp 0 looks back over a 64-tile window per round trip
// until it meets an inclusive prefix. Status words carry their own ready
// bits, so neither side needs a memory fence. Every wait is bounded.
//
// The lookback bounds the rate of tiles, not of bytes: a window of 64
// tiles per L2 round trip, so the tile is made large enough (8192
// elements, 96 KB of uint -> ulong traffic) that the tile rate HBM needs
// stays well inside it.
//
// HBM roofline: sizeof(in) + sizeof(out) bytes per element (12 B for
// uint -> ulong), plus 32 B of tile status per 8192 elements.
#include <atomic>
#include <mutex>
#include <type_traits>

#include "clo_internal.h"
#include "dev_common.cuh"
#include "scan_status.cuh"
#include "scan_tile.cuh"
#include "timing.h"

namespace clo {
namespace {

using namespace scantile;

using lb::Slots;
using lb::TileStatus;
using lb::publish;
using lb::read_status;
using lb::warp_sum;

template <typename Acc>
__device__ __forceinline__ Acc shfl_up(Acc v, int d) {
	return __shfl_up_sync(0xffffffffu, v, d);
}

// Persistent CTAs (one per resident slot) take tiles in order from an
// atomic counter. Per tile: the sums of the tile already in shared memory
// and publication of its aggregate; then, while warp 0 looks back, every
// warp issues the loads of the CTA's next tile (claimed at the top of the
// iteration) into registers and sums them, so the next tile's aggregate is
// published as soon as the lookback ends -- before this tile's outputs are
// written -- and no later tile waits on it longer than on a freshly
// launched one; after the outputs the prefetched data is transposed into
// shared memory. Every wait is on a lower tile id (down to tile 0, which
// publishes its prefix at once), so the waits cannot form a cycle.
template <typename InT, typename OutT>
__global__ void __launch_bounds__(kThreads, (scan_min_blocks<InT, OutT>()))
scan_lookback(const InT *__restrict__ in, OutT *__restrict__ out, size_t n,
	TileStatus ts,
	int *dev_status, bool vec_ok, long long debug_skip_tile,
	const void *carry_in, void *carry_out) {
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t,
		uint64_t>::type;
	extern __shared__ __align__(16) unsigned char s_dyn[];
	__shared__ Acc s_warp_tot[kWarps];
	__shared__ Acc s_next_tot[kWarps];
	__shared__ Acc s_excl;
	__shared__ uint32_t s_tile, s_next;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t num_tiles = (uint32_t)((n + kTile - 1) / kTile);
	InT *s_in = reinterpret_cast<InT *>(s_dyn + (size_t)warp *
		(kBlocks * padded<InT>() * sizeof(InT) + padded<OutT>() * sizeof(OutT)));
	OutT *s_out = reinterpret_cast<OutT *>(s_in + kBlocks * padded<InT>());
	auto full_tile = [&](uint32_t t) {
		return vec_ok && (size_t)(t + 1) * kTile <= n;
	};
	if (tid == 0) s_tile = atomicAdd(ts.counter, 1u);
	__syncthreads();
	uint32_t tile = s_tile;
	if (tile >= num_tiles) return;
	{
		const size_t wseg = (size_t)tile * kTile + (size_t)warp * kWarpElems;
		if (full_tile(tile)) {
			BlockRegs<InT> r;
			issue_loads<InT>(r, in, wseg, lane);
			store_loads<InT>(r, s_in, lane);
		} else {
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
				load_block_scalar<InT>(in, n, wseg + (size_t)b * kBlock, s_in + b * padded<InT>(), lane);
		}
	}
	__syncwarp();
	bool agg_published = false;  // the current tile's aggregate is out

	for (;;) {
		if (tid == 0) s_next = atomicAdd(ts.counter, 1u);
		const size_t wseg = (size_t)tile * kTile + (size_t)warp * kWarpElems;

		// ---- lane run sums and their warp scans, per block --------------
		Acc lane_excl[kBlocks], block_tot[kBlocks];
#pragma unroll
		for (int b = 0; b < kBlocks; ++b) {
			const InT *sin = s_in + b * padded<InT>();
			Acc run = 0;
#pragma unroll
			for (int j = 0; j < kItems; ++j) run += (Acc)(OutT)sin[pidx<InT>(lane * kItems + j)];
			Acc inc = run;
#pragma unroll
			for (int d = 1; d < 32; d <<= 1) {
				Acc t = shfl_up(inc, d);
				if (lane >= d) inc += t;
			}
			lane_excl[b] = inc - run;
			block_tot[b] = __shfl_sync(0xffffffffu, inc, 31);
		}
		if (lane == 0) {
			Acc wsum = 0;
#pragma unroll
			for (int b = 0; b < kBlocks; ++b) wsum += block_tot[b];
			s_warp_tot[warp] = wsum;
		}
		__syncthreads();
		const uint32_t next = s_next;
		const bool have_next = next < num_tiles;
		const bool next_full = have_next && full_tile(next);
		const size_t nseg = (size_t)next * kTile + (size_t)warp * kWarpElems;

		// ---- prefetch of the next tile (all warps) ----------------------
		BlockRegs<InT> r;
		if (next_full) issue_loads<InT>(r, in, nseg, lane);
		const bool next_publish = next_full && (long long)next != debug_skip_tile;

		// ---- tile aggregate, publication and lookback (warp 0) ----------
		if (warp == 0) {
			Acc wt = lane < kWarps ? s_warp_tot[lane] : (Acc)0;
			Acc winc = wt;
#pragma unroll
			for (int d = 1; d < kWarps; d <<= 1) {
				Acc t = shfl_up(winc, d);
				if (lane >= d) winc += t;
			}
			const Acc aggregate = __shfl_sync(0xffffffffu, winc, kWarps - 1);
			if (lane < kWarps) s_warp_tot[lane] = winc - wt;  // warp exclusive
			const bool do_publish = (long long)tile != debug_skip_tile;
			constexpr int PT = Slots<Acc>::kPerTile;
			Acc excl = 0;
			if (tile == 0) {
				// A scan continuing an earlier one starts from its carry.
				if (carry_in) excl = *reinterpret_cast<const Acc *>(carry_in);
				if (lane == 0 && do_publish)
					publish<Acc>(ts.words + Slots<Acc>::kWords, excl + aggregate);
			} else {
				if (lane == 0 && do_publish && !agg_published)
					publish<Acc>(ts.words + (size_t)tile * PT, aggregate);
				excl = lb::lookback_warp<Acc>(ts.words, tile, dev_status);
				if (lane == 0 && do_publish)
					publish<Acc>(ts.words + (size_t)tile * PT + Slots<Acc>::kWords,
						excl + aggregate);
			}
			if (lane == 0) {
				s_excl = excl;
				if (carry_out && (size_t)(tile + 1) * kTile >= n)
					*reinterpret_cast<Acc *>(carry_out) = excl + aggregate;
			}
		}
		// The next tile's sum from the prefetched registers.
		if (next_full) {
			constexpr int EPC = BlockRegs<InT>::kEpc;
			Acc part = 0;
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
#pragma unroll
				for (int k = 0; k < BlockRegs<InT>::kPerLane; ++k) {
					const InT *e = reinterpret_cast<const InT *>(&r.v[b][k]);
#pragma unroll
					for (int q = 0; q < EPC; ++q) part += (Acc)(OutT)e[q];
				}
			part = warp_sum<Acc>(part);
			if (lane == 0) s_next_tot[warp] = part;
		}
		__syncthreads();
		if (next_publish && tid == 0) {
			Acc agg = 0;
#pragma unroll
			for (int w = 0; w < kWarps; ++w) agg += s_next_tot[w];
			publish<Acc>(ts.words + (size_t)next * Slots<Acc>::kPerTile, agg);
		}

		// ---- outputs per block: second read, staged, coalesced stores ----
		Acc base = s_excl + s_warp_tot[warp];
#pragma unroll
		for (int b = 0; b < kBlocks; ++b) {
			const InT *sin = s_in + b * padded<InT>();
			Acc run = base + lane_excl[b];
#pragma unroll
			for (int j = 0; j < kItems; ++j) {
				const int q = lane * kItems + j;
				const Acc v = (Acc)(OutT)sin[pidx<InT>(q)];
				s_out[pidx<OutT>(q)] = (OutT)run;
				run += v;
			}
			base += block_tot[b];
			__syncwarp();
			const size_t seg = wseg + (size_t)b * kBlock;
			if (seg + kBlock <= n && vec_ok) {
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
				for (int i = lane; i < kBlock; i += 32)
					if (seg + i < n) out[seg + i] = s_out[pidx<OutT>(i)];
			}
			__syncwarp();
		}
		if (!have_next) break;

		// ---- the next tile into shared memory ---------------------------
		if (next_full) {
			store_loads<InT>(r, s_in, lane);
		} else {
#pragma unroll
			for (int b = 0; b < kBlocks; ++b)
				load_block_scalar<InT>(in, n, nseg + (size_t)b * kBlock, s_in + b * padded<InT>(), lane);
		}
		__syncwarp();
		agg_published = next_full;
		tile = next;
	}
}

// Per device and type pair, once: opts the kernel into its dynamic shared
// memory (more than 48 KB for most pairs) and records its resident CTAs
// per SM. Later calls (possibly while a graph is being captured) only read
// the cached count.
template <typename InT, typename OutT>
cudaError_t scan_prepare(int *per_sm) {
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
			e = cudaFuncSetAttribute(scan_lookback<InT, OutT>,
				cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scan_smem<InT, OutT>());
			if (e == cudaSuccess)
				e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, scan_lookback<InT, OutT>,
					kThreads, scan_smem<InT, OutT>());
			if (e != cudaSuccess) return e;
			if (v < 1) v = 1;
			cached[dev].store(v, std::memory_order_release);
		}
	}
	*per_sm = v;
	return cudaSuccess;
}

// Persistent grid: one CTA per resident slot, at most one per tile.
inline unsigned scan_grid(size_t tiles, int per_sm, int sm_count) {
	const size_t g = std::min<size_t>(tiles, (size_t)per_sm * (size_t)sm_count);
	return (unsigned)std::max<size_t>(g, 1);
}

template <typename InT, typename OutT>
cudaError_t launch_scan(const void *in, void *out, size_t n, CCLContext *ctx,
	cudaStream_t s, GError **err, long long debug_skip_tile,
	const void *carry_in = nullptr, void *carry_out = nullptr) {
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t,
		uint64_t>::type;
	const size_t tiles = (n + kTile - 1) / kTile;
	if (tiles >= (1ull << 31)) {
		set_error(err, CLO_ERROR_ARGS, "Scan of %zu elements is too large", n);
		return cudaErrorInvalidValue;
	}
	const size_t status_bytes = tiles * Slots<Acc>::kPerTile * sizeof(uint64_t);
	const size_t bytes = status_bytes + 16;
	char *tmp = (char *)tmp_alloc(ctx, bytes, s, err);
	if (!tmp) return cudaErrorMemoryAllocation;
	TileStatus ts;
	ts.words = (uint64_t *)tmp;
	ts.counter = (uint32_t *)(tmp + status_bytes);
	cudaError_t e = cudaMemsetAsync(tmp, 0, bytes, s);
	bool vec_ok = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
	int per_sm = 1;
	if (e == cudaSuccess) e = scan_prepare<InT, OutT>(&per_sm);
	if (e == cudaSuccess) {
		KernelTimer t("scan_lookback", s, (double)n * (sizeof(InT) + sizeof(OutT)));
		scan_lookback<InT, OutT><<<scan_grid(tiles, per_sm, ctx->sm_count), kThreads,
			scan_smem<InT, OutT>(), s>>>(
			(const InT *)in, (OutT *)out, n, ts, ctx->d_status, vec_ok,
			debug_skip_tile, carry_in, carry_out);
		t.stop();
		count_launches(1);
		e = cudaGetLastError();
	}
	tmp_free(tmp, s);
	if (e != cudaSuccess) cuda_ok(e, err, "scan_lookback");
	return e;
}

template <typename InT>
cudaError_t dispatch_out(const void *in, void *out, size_t n, int out_bytes,
	CCLContext *ctx, cudaStream_t s, GError **err, long long dbg,
	const void *ci = nullptr, void *co = nullptr) {
	switch (out_bytes) {
	case 1: return launch_scan<InT, uint8_t>(in, out, n, ctx, s, err, dbg, ci, co);
	case 2: return launch_scan<InT, uint16_t>(in, out, n, ctx, s, err, dbg, ci, co);
	case 4: return launch_scan<InT, uint32_t>(in, out, n, ctx, s, err, dbg, ci, co);
	case 8: return launch_scan<InT, uint64_t>(in, out, n, ctx, s, err, dbg, ci, co);
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported sum width %d", out_bytes);
	return cudaErrorInvalidValue;
}

}  // namespace

// Tile whose publication is withheld (-1: none). Only the watchdog test
// sets it, through clo_gb300_debug_scan_withhold().
static long long g_debug_skip_tile = -1;

cudaError_t scan_exclusive(const void *in, void *out, size_t n,
	CloType in_type, int out_bytes, CCLContext *ctx, cudaStream_t s,
	GError **err) {
	return scan_exclusive_carry(in, out, n, in_type, out_bytes, nullptr, nullptr, ctx, s, err);
}

cudaError_t scan_exclusive_carry(const void *in, void *out, size_t n,
	CloType in_type, int out_bytes, const void *ci, void *co, CCLContext *ctx,
	cudaStream_t s, GError **err) {
	if (n == 0) return cudaSuccess;
	long long dbg = g_debug_skip_tile;
	switch (in_type) {
	case CLO_CHAR: return dispatch_out<int8_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_UCHAR: return dispatch_out<uint8_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_SHORT: return dispatch_out<int16_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_USHORT: return dispatch_out<uint16_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_INT: return dispatch_out<int32_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_UINT: return dispatch_out<uint32_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_LONG: return dispatch_out<int64_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	case CLO_ULONG: return dispatch_out<uint64_t>(in, out, n, out_bytes, ctx, s, err, dbg, ci, co);
	default: break;
	}
	set_error(err, CLO_ERROR_ARGS, "Unsupported scan element type %d", (int)in_type);
	return cudaErrorInvalidValue;
}

}  // namespace clo

// Test hook for the lookback watchdog: the given tile of the next scans
// never publishes its status, so its successor's bounded wait runs out
// and reports through the context status word. -1 restores normal
// operation.
extern "C" void clo_gb300_debug_scan_withhold(long long tile) {
	clo::g_debug_skip_tile = tile;
}

// ---------------------------------------------------------------------
// Scan that allocates nothing (clo_scan_blelloch_noalloc).
//
// Same kernel as above; its tile statuses and tile counter live in the
// file-scope device array below instead of a pool temporary. The array is
// part of the library's device image: every GPU that loads the library
// holds it (1 MiB + 16 B) until the process exits. Host code cannot use
// the array's name as a device address (on the host it names a stand-in),
// so the device address is looked up once per device with
// cudaGetSymbolAddress and cached.
// ---------------------------------------------------------------------

// Largest no-allocation scan: 2^15 tiles of 8192 elements = 2^28 elements.
#define CLO_NOALLOC_MAX_TILES (1u << 15)
// Four status words per tile (64-bit sums) and one word for the counter.
#define CLO_NOALLOC_WORDS (CLO_NOALLOC_MAX_TILES * 4u + 2u)

static __device__ __align__(256) uint64_t g_scan_noalloc_scratch[CLO_NOALLOC_WORDS];

namespace clo {
namespace {

constexpr size_t kNoAllocMaxElems = (size_t)CLO_NOALLOC_MAX_TILES * kTile;
static_assert(kNoAllocMaxElems == ((size_t)1 << 28), "no-allocation scan limit");

std::mutex g_noalloc_mu;
uint64_t *g_noalloc_addr[64] = {};

// Makes `ordinal` the calling thread's current device for the guard's
// lifetime and restores the previous one afterwards.
struct CurrentDevice {
	int prev = -1;
	cudaError_t status;
	explicit CurrentDevice(int ordinal) {
		if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
		status = cudaSetDevice(ordinal);
	}
	~CurrentDevice() {
		if (prev >= 0) cudaSetDevice(prev);
	}
};

// Opts every (element, sum) instantiation of the scan kernel into its
// shared memory and caches its occupancy, so that no later call does any
// set-up work, whatever its type pair.
template <typename InT>
cudaError_t noalloc_prepare_in() {
	int v = 0;
	cudaError_t e = scan_prepare<InT, uint8_t>(&v);
	if (e == cudaSuccess) e = scan_prepare<InT, uint16_t>(&v);
	if (e == cudaSuccess) e = scan_prepare<InT, uint32_t>(&v);
	if (e == cudaSuccess) e = scan_prepare<InT, uint64_t>(&v);
	return e;
}

cudaError_t noalloc_prepare_all() {
	cudaError_t e = noalloc_prepare_in<int8_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<uint8_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<int16_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<uint16_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<int32_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<uint32_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<int64_t>();
	if (e == cudaSuccess) e = noalloc_prepare_in<uint64_t>();
	return e;
}

// Device address of the scratch array on device `ordinal` (which must be
// current), looked up on the first call for that device, together with
// the set-up of every scan instantiation.
uint64_t *noalloc_scratch(int ordinal, GError **err) {
	std::lock_guard<std::mutex> lk(g_noalloc_mu);
	if (g_noalloc_addr[ordinal] == nullptr) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_scan_noalloc_scratch);
		if (e != cudaSuccess || p == nullptr) {
			cudaGetLastError();
			set_error(err, CLO_ERROR_LIBRARY,
				"cudaGetSymbolAddress of the no-allocation scan scratch failed on "
				"device %d: %s", ordinal, cudaGetErrorString(e));
			return nullptr;
		}
		e = noalloc_prepare_all();
		if (e != cudaSuccess) {
			cudaGetLastError();
			set_error(err, CLO_ERROR_LIBRARY,
				"No-allocation scan set-up failed on device %d: %s", ordinal,
				cudaGetErrorString(e));
			return nullptr;
		}
		g_noalloc_addr[ordinal] = (uint64_t *)p;
	}
	return g_noalloc_addr[ordinal];
}

template <typename InT, typename OutT>
cudaError_t launch_scan_noalloc(const void *in, void *out, size_t n,
	uint64_t *scratch, int *dev_status, int sm_count, cudaStream_t s) {
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t,
		uint64_t>::type;
	const size_t tiles = (n + kTile - 1) / kTile;
	TileStatus ts;
	ts.words = scratch;
	ts.counter = (uint32_t *)(scratch + (size_t)CLO_NOALLOC_MAX_TILES * 4);
	// The array keeps the previous call's statuses: clear the words this
	// call reads before writing (its tiles' slots and the tile counter).
	cudaError_t e = cudaMemsetAsync(ts.words, 0,
		tiles * Slots<Acc>::kPerTile * sizeof(uint64_t), s);
	if (e == cudaSuccess) e = cudaMemsetAsync(ts.counter, 0, sizeof(uint64_t), s);
	if (e != cudaSuccess) return e;
	bool vec_ok = ((uintptr_t)in % 16 == 0) && ((uintptr_t)out % 16 == 0);
	int per_sm = 1;
	e = scan_prepare<InT, OutT>(&per_sm);
	if (e != cudaSuccess) return e;
	scan_lookback<InT, OutT><<<scan_grid(tiles, per_sm, sm_count), kThreads,
		scan_smem<InT, OutT>(), s>>>(
		(const InT *)in, (OutT *)out, n, ts, dev_status, vec_ok, -1, nullptr, nullptr);
	count_launches(1);
	return cudaGetLastError();
}

template <typename InT>
cudaError_t noalloc_out(const void *in, void *out, size_t n, int out_bytes,
	uint64_t *scratch, int *st, int sms, cudaStream_t s) {
	switch (out_bytes) {
	case 1: return launch_scan_noalloc<InT, uint8_t>(in, out, n, scratch, st, sms, s);
	case 2: return launch_scan_noalloc<InT, uint16_t>(in, out, n, scratch, st, sms, s);
	case 4: return launch_scan_noalloc<InT, uint32_t>(in, out, n, scratch, st, sms, s);
	default: return launch_scan_noalloc<InT, uint64_t>(in, out, n, scratch, st, sms, s);
	}
}

}  // namespace
}  // namespace clo

extern "C" cl_bool clo_scan_blelloch_noalloc(CCLQueue *cq, CloType elem_type,
	CloType sum_type, const void *d_in, void *d_out, size_t numel,
	GError **err) {
	using namespace clo;
	if (err && *err) return CL_FALSE;
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return CL_FALSE;
	}
	if (!type_is_integer(elem_type) || !type_is_integer(sum_type)) {
		set_error(err, CLO_ERROR_ARGS,
			"No-allocation scan: integer element and sum types only");
		return CL_FALSE;
	}
	if (numel > kNoAllocMaxElems) {
		set_error(err, CLO_ERROR_ARGS,
			"No-allocation scan of %zu elements exceeds its limit of %zu elements "
			"(the size of its static device scratch); use clo_scan_with_device_data",
			numel, kNoAllocMaxElems);
		return CL_FALSE;
	}
	if (numel == 0) return CL_TRUE;
	if (!d_in || !d_out) {
		set_error(err, CLO_ERROR_ARGS, "NULL input or output pointer");
		return CL_FALSE;
	}
	const int ordinal = cq->ctx->ordinal;
	if (ordinal < 0 || ordinal >= 64) {
		set_error(err, CLO_ERROR_ARGS, "Device ordinal %d out of range", ordinal);
		return CL_FALSE;
	}
	CurrentDevice dev(ordinal);
	if (!cuda_ok(dev.status, err, "clo_scan_blelloch_noalloc: cudaSetDevice")) return CL_FALSE;
	uint64_t *scratch = noalloc_scratch(ordinal, err);
	if (!scratch) return CL_FALSE;
	const int ob = (int)clo_type_sizeof(sum_type);
	int *st = cq->ctx->d_status;
	const int sms = cq->ctx->sm_count;
	cudaStream_t s = cq->stream;
	cudaError_t e;
	switch (elem_type) {
	case CLO_CHAR: e = noalloc_out<int8_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_UCHAR: e = noalloc_out<uint8_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_SHORT: e = noalloc_out<int16_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_USHORT: e = noalloc_out<uint16_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_INT: e = noalloc_out<int32_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_UINT: e = noalloc_out<uint32_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	case CLO_LONG: e = noalloc_out<int64_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	default: e = noalloc_out<uint64_t>(d_in, d_out, numel, ob, scratch, st, sms, s); break;
	}
	return cuda_ok(e, err, "clo_scan_blelloch_noalloc") ? CL_TRUE : CL_FALSE;
}
