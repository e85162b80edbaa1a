// Internal definitions shared by the host layer (*.cpp) and the kernel
// launchers (*.cu). Not installed; the public API is in include/*.h.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

#include "cl_ops.h"

// ---------------------------------------------------------------------
// Wrapper objects (see include/ccl_shim.h for the mapping to cf4ocl2).
// ---------------------------------------------------------------------
struct ccl_device {
	int ordinal;
};

struct ccl_context {
	std::atomic<int> refcount;
	int ordinal;
	ccl_device device;
	int sm_count;
	size_t smem_optin;
	// Device-resident status words written by bounded spin-waits:
	// [0] = error code (clo::DevError), [1] = detail (tile index).
	int *d_status;
	// Pinned mirror of d_status for cheap polling.
	int *h_status;
};

struct ccl_event {
	cudaEvent_t start;
	cudaEvent_t end;
	bool timing;
	bool started;
	std::string name;
	struct ccl_queue *queue;
};

struct ccl_queue {
	CCLContext *ctx;
	cudaStream_t stream;
	bool owned;
	bool profiling;
	std::vector<ccl_event *> events;
	std::vector<ccl_event *> free_events;
};

struct ccl_buffer {
	std::atomic<int> refcount;
	CCLContext *ctx;
	void *ptr;
	size_t size;
	bool owned;
};

struct ccl_program {
	std::string src;
	std::string opts;
};

struct ccl_ewl_impl {
	std::vector<ccl_event *> evts;
};

struct clo_graph {
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	CCLContext *ctx;
	size_t nodes;
};

namespace clo {

// Device-side error codes reported through ccl_context::d_status.
enum DevError : int {
	DEV_OK = 0,
	DEV_ERR_LOOKBACK_TIMEOUT = 1,  // decoupled-lookback wait hit its cap
	DEV_ERR_BAD_SEGMENTS = 2,      // segment offsets decrease or pass the buffer
	DEV_ERR_COPY_TIMEOUT = 3,      // a bulk copy's completion wait hit its cap
};

// Error helpers (GError semantics: *err must be NULL on entry; err may be
// NULL to ignore errors).
void set_error(GError **err, int code, const char *fmt, ...);
void propagate_error(GError **dest, GError *src);
bool cuda_ok(cudaError_t e, GError **err, const char *what);

// Object counters for ccl_wrapper_memcheck.
void wrapper_created();
void wrapper_destroyed();

// Launch accounting (clo_gb300_launch_count).
void count_launches(unsigned n);

// Stream-ordered temporaries from the device's memory pool.
void *tmp_alloc(CCLContext *ctx, size_t bytes, cudaStream_t s, GError **err);
void tmp_free(void *p, cudaStream_t s);

// Event plumbing used by the object API.
ccl_event *event_begin(CCLQueue *q, const char *name);
void event_end(ccl_event *e);
bool wait_ewl(CCLQueue *q, CCLEventWaitList *ewl, GError **err);
// Checks (and clears) the device status word after a synchronisation.
bool check_device_status(CCLContext *ctx, GError **err);

// True when the stream is being captured into a CUDA graph.
bool stream_capturing(cudaStream_t s);

// Scalar type helpers.
bool type_is_integer(CloType t);
bool type_is_signed(CloType t);

// ---------------------------------------------------------------------
// Kernel launchers (implemented in *.cu).
// ---------------------------------------------------------------------

// Stable LSD radix sort (onesweep) of n keys of key_bytes in {1,2,4,8},
// ascending by bits [0, sort_bits) of the unsigned key pattern, carrying
// optional values of val_bytes in {0,4,8}. In place on keys/vals.
// `allow_skip` lets the launcher read back the digit histograms and skip
// passes whose digit is constant (not allowed during graph capture).
cudaError_t radix_sort(void *keys, void *vals, size_t n, int key_bytes,
	int val_bytes, int sort_bits, CCLContext *ctx, cudaStream_t s,
	bool allow_skip, GError **err);

// Stable partition of n keys (key_bytes 2, 4 or 8) by the top 8 bits of
// their low sort_bits bits, into keys_out; counts (host, 256 entries)
// receives the size of each group. Synchronises the stream once.
cudaError_t radix_msd_partition(const void *keys_in, void *keys_out, size_t n, int key_bytes,
	int sort_bits, uint32_t *counts, CCLContext *ctx, cudaStream_t s, GError **err);

// Exclusive scan: out[i] = sum_{j<i} (sum type) in[j] modulo
// 2^(8*out_bytes). in_type is an integer CloType, out_bytes in {1,2,4,8}.
cudaError_t scan_exclusive(const void *in, void *out, size_t n,
	CloType in_type, int out_bytes, CCLContext *ctx, cudaStream_t s,
	GError **err);

// The same scan continuing an earlier one: the sums start from the value
// at carry_in (device, the sum type; null = 0), and the total (carry plus
// this part's sum) is written to carry_out (device; null = not written).
cudaError_t scan_exclusive_carry(const void *in, void *out, size_t n,
	CloType in_type, int out_bytes, const void *carry_in, void *carry_out,
	CCLContext *ctx, cudaStream_t s, GError **err);

// Bitonic network sort of n elements (default compare "a > b" on the
// element's own type), reproducing the reference network exactly:
// pairs, directions and the strict-compare-xor-direction swap rule.
// Non-power-of-two n is padded (in a temporary) with the type's maximum.
cudaError_t bitonic_sort(void *data, size_t n, CloType type,
	CCLContext *ctx, cudaStream_t s, GError **err);

// Rank-by-counting sort (stable, out of place): out[rank(i)] = in[i].
// Optional values (val_bytes 0/4/8) follow their keys.
cudaError_t gselect_sort(const void *in, void *out, size_t n, CloType type,
	const void *vals_in, void *vals_out, int val_bytes, CCLContext *ctx,
	cudaStream_t s, GError **err);

// Segmented sort ("satradix" order within each segment [off[i], off[i+1])
// of keys; off is a device array of S + 1 non-decreasing offsets within
// n_cap elements), in a fixed launch sequence with no host readback.
// variant selects the CTA class layout (0 .. seg_sort_num_variants()-1).
// With `alt` (n_cap elements) and `in_alt`, the multi-CTA passes use `alt`
// as their second buffer and, after an odd number of passes, leave every
// segment's result there (*in_alt = true) instead of copying it back.
int seg_sort_num_variants();
cudaError_t seg_sort(void *keys, uint64_t n_cap, const uint64_t *off, size_t S,
	int key_bytes, int sort_bits, int variant, CCLContext *ctx, cudaStream_t s,
	GError **err, void *alt = nullptr, bool *in_alt = nullptr);

// Segmented exclusive scan: within each segment, out as the scan of that
// segment alone; elements outside [off[0], off[S]) are not written.
cudaError_t seg_scan(const void *in, void *out, uint64_t n_cap, const uint64_t *off,
	size_t S, CloType in_type, int out_bytes, CCLContext *ctx, cudaStream_t s,
	GError **err);

// Host check of segment offsets (non-decreasing, within numel, segments
// shorter than 2^30): CLO_ERROR_ARGS otherwise.
// Copies k device segments into one buffer and back: segment i holds
// off[i + 1] - off[i] elements of elem_bytes bytes at srcs[i] (gather) or
// dsts[i] (scatter), and at element off[i] of the contiguous buffer. srcs,
// dsts and off are device arrays.
cudaError_t seg_gather(void *dst, const void *const *srcs, const uint64_t *off, uint32_t k,
	uint64_t total, int elem_bytes, int sm_count, cudaStream_t s);
cudaError_t seg_scatter(void *const *dsts, const void *src, const uint64_t *off, uint32_t k,
	uint64_t total, int elem_bytes, int sm_count, cudaStream_t s);

bool check_offsets(const uint64_t *off, size_t S, size_t numel, GError **err);

// Generator ids (index into clo_rng_infos).
enum RngGen : int {
	RNG_LCG = 0, RNG_XS64 = 1, RNG_XS128 = 2, RNG_MWC64X = 3,
	RNG_PARKMILLER = 4, RNG_TAUSLCG = 5
};

// A compiled DEV_GID seed hash: a small stack program over the 64-bit
// seed variable x (see rng.cpp for the grammar).
struct HashProgram {
	enum { MAX_OPS = 96 };
	int n_ops;
	uint8_t op[MAX_OPS];
	uint64_t imm[MAX_OPS];
};

cudaError_t rng_init_gid(void *states, size_t count, int gen,
	uint64_t main_seed, const HashProgram &hp, cudaStream_t s);

cudaError_t rng_fill(void *states, size_t count, int gen, uint32_t *out,
	size_t draws, unsigned bits, unsigned maxint, cudaStream_t s);

}  // namespace clo
