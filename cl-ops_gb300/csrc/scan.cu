// Exclusive prefix sum ("blelloch" scanner) as one single-pass kernel with
// decoupled lookback.
//
// Semantics follow src/cl_ops/scan/clo_scan_blelloch.cl:49-211: out[0] = 0
// and out[i] = sum_{j<i} (SUM_TYPE) in[j], with the element converted to
// the sum type by C rules and the sum wrapping modulo 2^(8*sizeof(SUM)).
// Integer addition is associative, so the result is bit-identical to the
// reference's work-group Blelloch trees whatever the summation order.
//
// Layout: tiles of 4096 elements, 256 threads, 16 consecutive elements per
// thread. Each warp moves its 512-element segment between global memory
// and registers through a padded shared-memory transpose, so every global
// access is a coalesced 16-byte vector access. Tiles take ids from an
// atomic counter (so a tile only ever waits on tiles already running),
// publish their aggregate, then warp 0 looks back over a 64-tile window
// per round trip until it meets an inclusive prefix. Status words carry
// their own ready bits, so neither side needs a memory fence. Every wait
// is bounded.
//
// HBM roofline: sizeof(in) + sizeof(out) bytes per element (12 B for
// uint -> ulong), plus 32 B of tile status per 4096 elements.
#include <mutex>
#include <type_traits>

#include "clo_internal.h"
#include "dev_common.cuh"
#include "scan_status.cuh"
#include "timing.h"

namespace clo {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kWarpElems = 32 * kItems;
constexpr int kTile = kWarps * kWarpElems;
constexpr int kPadded = kWarpElems + kWarpElems / 32;

__device__ __forceinline__ int pidx(int i) { return i + (i >> 5); }

using lb::Slots;
using lb::TileStatus;
using lb::publish;
using lb::read_status;
using lb::warp_sum;

template <typename Acc>
__device__ __forceinline__ Acc shfl_up(Acc v, int d) {
	return __shfl_up_sync(0xffffffffu, v, d);
}

template <typename InT, typename OutT>
__global__ void __launch_bounds__(kThreads, 5)
scan_lookback(const InT *__restrict__ in, OutT *__restrict__ out, size_t n,
	TileStatus ts,
	int *dev_status, bool vec_ok, long long debug_skip_tile,
	const void *carry_in, void *carry_out) {
	using Acc = typename std::conditional<(sizeof(OutT) <= 4), uint32_t,
		uint64_t>::type;
	constexpr int ESZ = sizeof(InT) > sizeof(OutT) ? sizeof(InT) : sizeof(OutT);
	__shared__ __align__(16) unsigned char s_buf[kWarps][kPadded * ESZ];
	__shared__ Acc s_warp_tot[kWarps];
	__shared__ Acc s_excl;
	__shared__ uint32_t s_tile;

	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const uint32_t num_tiles = (uint32_t)((n + kTile - 1) / kTile);
	(void)num_tiles;
	if (tid == 0) s_tile = atomicAdd(ts.counter, 1u);
	__syncthreads();
	const uint32_t tile = s_tile;
	const size_t seg = (size_t)tile * kTile + (size_t)warp * kWarpElems;
	const bool full = seg + kWarpElems <= n;

	// ---- load the warp's segment (coalesced) into padded smem -----------
	InT *sin = reinterpret_cast<InT *>(s_buf[warp]);
	if (full && vec_ok) {
		constexpr int EPC = 16 / sizeof(InT);
		constexpr int CHUNKS = kWarpElems / EPC;
		const uint4 *src = reinterpret_cast<const uint4 *>(in + seg);
#pragma unroll
		for (int c = lane; c < CHUNKS; c += 32) {
			uint4 v = dev::ld_stream_v4(src + c);
			const InT *e = reinterpret_cast<const InT *>(&v);
#pragma unroll
			for (int k = 0; k < EPC; ++k) sin[pidx(c * EPC + k)] = e[k];
		}
	} else {
		for (int i = lane; i < kWarpElems; i += 32)
			sin[pidx(i)] = (seg + i < n) ? in[seg + i] : (InT)0;
	}
	__syncwarp();

	// ---- per-thread sequential scan of 16 consecutive elements ----------
	Acc x[kItems];
	Acc run = 0;
#pragma unroll
	for (int j = 0; j < kItems; ++j) {
		Acc v = (Acc)(OutT)sin[pidx(lane * kItems + j)];
		x[j] = run;  // exclusive within the thread
		run += v;
	}
	// Warp inclusive scan of thread totals.
	Acc inc = run;
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		Acc t = shfl_up(inc, d);
		if (lane >= d) inc += t;
	}
	const Acc lane_excl = inc - run;
	if (lane == 31) s_warp_tot[warp] = inc;
	__syncthreads();

	// ---- tile aggregate, publication and lookback (warp 0) --------------
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
			if (lane == 0 && do_publish) publish<Acc>(ts.words + (size_t)tile * PT, aggregate);
			excl = lb::lookback_warp<Acc>(ts.words, tile, dev_status);
			if (lane == 0 && do_publish)
				publish<Acc>(ts.words + (size_t)tile * PT + Slots<Acc>::kWords, excl + aggregate);
		}
		if (lane == 0) {
			s_excl = excl;
			if (carry_out && (size_t)(tile + 1) * kTile >= n)
				*reinterpret_cast<Acc *>(carry_out) = excl + aggregate;
		}
	}
	__syncthreads();

	// ---- outputs through padded smem, coalesced stores -------------------
	const Acc base = s_excl + s_warp_tot[warp] + lane_excl;
	OutT *sout = reinterpret_cast<OutT *>(s_buf[warp]);
#pragma unroll
	for (int j = 0; j < kItems; ++j) sout[pidx(lane * kItems + j)] = (OutT)(base + x[j]);
	__syncwarp();
	if (full && vec_ok) {
		constexpr int EPC = 16 / sizeof(OutT);
		constexpr int CHUNKS = kWarpElems / EPC;
		uint4 *dst = reinterpret_cast<uint4 *>(out + seg);
#pragma unroll
		for (int c = lane; c < CHUNKS; c += 32) {
			uint4 v;
			OutT *e = reinterpret_cast<OutT *>(&v);
#pragma unroll
			for (int k = 0; k < EPC; ++k) e[k] = sout[pidx(c * EPC + k)];
			dev::st_stream_v4(dst + c, v);
		}
	} else {
		for (int i = lane; i < kWarpElems; i += 32)
			if (seg + i < n) out[seg + i] = sout[pidx(i)];
	}
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
	if (e == cudaSuccess) {
		KernelTimer t("scan_lookback", s, (double)n * (sizeof(InT) + sizeof(OutT)));
		scan_lookback<InT, OutT><<<(unsigned)tiles, kThreads, 0, s>>>(
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
// holds it (2 MiB + 16 B) until the process exits. Host code cannot use
// the array's name as a device address (on the host it names a stand-in),
// so the device address is looked up once per device with
// cudaGetSymbolAddress and cached.
// ---------------------------------------------------------------------

// Largest no-allocation scan: 2^16 tiles of 4096 elements = 2^28 elements.
#define CLO_NOALLOC_MAX_TILES (1u << 16)
// Four status words per tile (64-bit sums) and one word for the counter.
#define CLO_NOALLOC_WORDS (CLO_NOALLOC_MAX_TILES * 4u + 2u)

static __device__ __align__(256) uint64_t g_scan_noalloc_scratch[CLO_NOALLOC_WORDS];

namespace clo {
namespace {

constexpr size_t kNoAllocMaxElems = (size_t)CLO_NOALLOC_MAX_TILES * kTile;

std::mutex g_noalloc_mu;
uint64_t *g_noalloc_addr[64] = {};

// Device address of the scratch array on device `ordinal`, looked up on
// the first call for that device with the device current.
uint64_t *noalloc_scratch(int ordinal, GError **err) {
	if (ordinal < 0 || ordinal >= 64) {
		set_error(err, CLO_ERROR_ARGS, "Device ordinal %d out of range", ordinal);
		return nullptr;
	}
	std::lock_guard<std::mutex> lk(g_noalloc_mu);
	if (g_noalloc_addr[ordinal] == nullptr) {
		cudaError_t e = cudaSetDevice(ordinal);
		void *p = nullptr;
		if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_scan_noalloc_scratch);
		if (e != cudaSuccess || p == nullptr) {
			cudaGetLastError();
			set_error(err, CLO_ERROR_LIBRARY,
				"cudaGetSymbolAddress of the no-allocation scan scratch failed on "
				"device %d: %s", ordinal, cudaGetErrorString(e));
			return nullptr;
		}
		g_noalloc_addr[ordinal] = (uint64_t *)p;
	}
	return g_noalloc_addr[ordinal];
}

template <typename InT, typename OutT>
cudaError_t launch_scan_noalloc(const void *in, void *out, size_t n,
	uint64_t *scratch, int *dev_status, cudaStream_t s) {
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
	scan_lookback<InT, OutT><<<(unsigned)tiles, kThreads, 0, s>>>(
		(const InT *)in, (OutT *)out, n, ts, dev_status, vec_ok, -1, nullptr, nullptr);
	count_launches(1);
	return cudaGetLastError();
}

template <typename InT>
cudaError_t noalloc_out(const void *in, void *out, size_t n, int out_bytes,
	uint64_t *scratch, int *st, cudaStream_t s) {
	switch (out_bytes) {
	case 1: return launch_scan_noalloc<InT, uint8_t>(in, out, n, scratch, st, s);
	case 2: return launch_scan_noalloc<InT, uint16_t>(in, out, n, scratch, st, s);
	case 4: return launch_scan_noalloc<InT, uint32_t>(in, out, n, scratch, st, s);
	default: return launch_scan_noalloc<InT, uint64_t>(in, out, n, scratch, st, s);
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
	uint64_t *scratch = noalloc_scratch(cq->ctx->ordinal, err);
	if (!scratch) return CL_FALSE;
	cudaSetDevice(cq->ctx->ordinal);
	const int ob = (int)clo_type_sizeof(sum_type);
	int *st = cq->ctx->d_status;
	cudaStream_t s = cq->stream;
	cudaError_t e;
	switch (elem_type) {
	case CLO_CHAR: e = noalloc_out<int8_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_UCHAR: e = noalloc_out<uint8_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_SHORT: e = noalloc_out<int16_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_USHORT: e = noalloc_out<uint16_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_INT: e = noalloc_out<int32_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_UINT: e = noalloc_out<uint32_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	case CLO_LONG: e = noalloc_out<int64_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	default: e = noalloc_out<uint64_t>(d_in, d_out, numel, ob, scratch, st, s); break;
	}
	return cuda_ok(e, err, "clo_scan_blelloch_noalloc") ? CL_TRUE : CL_FALSE;
}
