/*
 * cl_ops on GB300 -- entry points that extend the reference API.
 *
 * None of these has a counterpart in the reference. Each exists because
 * the reference cannot express the operation:
 *  - key-value sorting: the reference sorts one CloType per element and
 *    has no 12-byte type for a (uint64 key, uint32 value) pair;
 *  - clo_rng_fill: the reference draws random numbers from client kernels
 *    only (its benchmark kernel src/benchmarks/clo_rng_bench.cl:23-37 is
 *    what this entry point packages, with the whole draw loop on device);
 *  - pinned host buffers for full-speed host<->device copies.
 */
#ifndef CLO_GB300_H
#define CLO_GB300_H

#include "clo_common.h"
#include "ccl_shim.h"
#include "clo_sort_abstract.h"
#include "clo_scan_abstract.h"
#include "clo_rng.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Stable sort of `keys` (the sorter's element type, ascending by the
 * key's unsigned bit pattern, as "satradix" sorts) carrying `values`
 * (value_type, any 4- or 8-byte type) along. In place on both buffers.
 * Only "satradix" and "gselect" (both stable) accept it; other sorters set
 * CLO_ERROR_ARGS. Asynchronous; returns the last event. */
CCLEvent *clo_sort_kv_with_device_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLBuffer *keys, CCLBuffer *values, CloType value_type, size_t numel,
	GError **err);

/* Blocking host-memory form of clo_sort_kv_with_device_data. */
cl_bool clo_sort_kv_with_host_data(CloSort *sorter, CCLQueue *cq_exec,
	void *keys, void *values, CloType value_type, size_t numel,
	GError **err);

/* Draws `draws` numbers from every state of `rng` into `out`, draw-major:
 * out[r * n_states + i] = next(state i) >> (32 - bits) when maxint == 0,
 * else next(state i) % maxint (the two modes of clo_rng_bench.cl). The
 * states advance, so consecutive calls continue the streams. `out` must
 * hold draws * n_states uint32 values. bits in [1, 32]. */
CCLEvent *clo_rng_fill(CloRng *rng, CCLQueue *cq, CCLBuffer *out,
	size_t draws, cl_uint bits, cl_uint maxint, GError **err);

/* Page-locked host memory for full-bandwidth copies (cudaMallocHost). */
void *clo_host_alloc(size_t size, GError **err);
void clo_host_free(void *ptr);

/* Number of kernel launches this library issued so far in this process
 * (all devices). */
cl_ulong clo_gb300_launch_count(void);

/* Per-kernel device time: when enabled, every kernel launch of this
 * library is bracketed by CUDA events on its stream, and
 * clo_gb300_timing_get returns (after waiting for them) the summed time,
 * the summed algorithmic HBM bytes and the launch count of the named
 * kernel ("satradix_onesweep", "satradix_upsweep", "scan_lookback",
 * "abitonic_tile_sort", "abitonic_global_steps", "abitonic_tile_finish",
 * "rng_fill"); it returns 0 when the kernel has not run. */
void clo_gb300_timing_enable(int on);
void clo_gb300_timing_reset(void);
int clo_gb300_timing_get(const char *kernel, double *total_ms,
	double *total_bytes, cl_ulong *launches);

/* Exclusive scan ("blelloch" semantics, integer types as clo_scan_new)
 * that allocates no memory. It has no counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc or any other allocator
 * when they scan: code that runs while another thread captures a CUDA
 * graph in global mode (where allocation calls are errors), processes
 * whose device memory is all reserved up front by another allocator or a
 * fixed budget (so a new allocation fails), and loops that cannot afford
 * an allocation that may synchronise the device. The caller passes the
 * device input and output pointers; the scan's own scratch (its tile
 * statuses) is a file-scope device array of this library, sized for at
 * most 2^28 elements (1 MiB, held on every GPU that loads the library
 * until the process exits). Larger numel is rejected with CLO_ERROR_ARGS.
 *
 * The first call on a device does all of the entry point's set-up for
 * that device: it looks the array's device address up
 * (cudaGetSymbolAddress, with that device current) and prepares the scan
 * kernel for every element and sum type, so later calls with any type
 * pair do no set-up work. Make that first call before any stream
 * capture. Each call makes the queue's device current for its duration
 * and restores the caller's current device before it returns. Every call
 * clears the part of the array it
 * uses, on cq's stream, before the scan; all calls share the one array,
 * so calls whose work overlaps on the GPU (different streams, no ordering
 * between them) race and give wrong results. Asynchronous on cq: no event
 * is created; a bounded-wait failure is reported by the next
 * ccl_queue_finish on cq. */
cl_bool clo_scan_blelloch_noalloc(CCLQueue *cq, CloType elem_type,
	CloType sum_type, const void *d_in, void *d_out, size_t numel,
	GError **err);

/* ---------------------------------------------------------------------
 * Segmented operations: many independent segments of one buffer in one
 * call. `offsets` holds num_segments + 1 cl_ulong values, non-decreasing;
 * segment i is elements [offsets[i], offsets[i+1]). Every segment comes
 * out exactly as a separate clo_sort_with_device_data /
 * clo_scan_with_device_data call on that segment alone would leave it;
 * elements outside [offsets[0], offsets[num_segments]) are not written.
 * Segments must be shorter than 2^30 elements. The device-data forms
 * issue a fixed sequence of launches that depends only on the buffer sizes
 * and num_segments (no host readback of the offsets), so they can be
 * captured into a CUDA graph (clo_queue_begin_capture); invalid offsets
 * are detected on the device and reported (CLO_ERROR_ARGS) by the next
 * synchronising call on the queue. The host-data forms check the offsets
 * first and block.
 * --------------------------------------------------------------------- */

/* Sorts every segment of `data` (in place) in "satradix" order: stable,
 * ascending by the unsigned bit pattern of the sorter's key. Only
 * "satradix" sorters accept it; others set CLO_ERROR_ARGS. The buffer
 * capacity (its size / element size) bounds the offsets. Segments go by
 * length to a warp (<= 32 elements), a CTA (two classes of shared-memory
 * radix sort) or the multi-CTA onesweep passes. The shape -- the two CTA
 * classes' layouts (threads x keys per thread, which also set the class
 * boundaries), the CTA classes' digit width (8 or 4 bits) and the keys
 * per thread of the long-segment passes' tiles -- is the sorter's
 * "segvariant=<n>" option or the autotuner's choice; variant 0 is the
 * default shape. */
CCLEvent *clo_sort_segmented_with_device_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLBuffer *data, CCLBuffer *offsets, size_t num_segments, GError **err);
cl_bool clo_sort_segmented_with_host_data(CloSort *sorter, CCLQueue *cq_exec,
	void *data, size_t numel, const cl_ulong *offsets, size_t num_segments,
	GError **err);

/* Number of segmented-sort shapes: class A layout (128 x 8, 256 x 8) x
 * class B layout (512 x 16, 256 x 16, 1024 x 16) x long-pass keys per
 * thread (56, 48, 40; 32, 28, 24 for 8-byte keys) x CTA-class digit bits
 * (8, 4); variant = ((a * 3 + b) * 3 + l) * 2 + d. */
#define CLO_SEG_SORT_VARIANTS 36

/* Autotuner: times every shape on a copy of `data` with these offsets
 * (best of two runs each), stores the fastest in the sorter for its later
 * segmented sorts and returns its index (-1 on error). The caller's data
 * is not modified. times_ms, when not NULL, receives CLO_SEG_SORT_VARIANTS
 * times in milliseconds. Blocking. */
cl_int clo_sort_segmented_tune(CloSort *sorter, CCLQueue *cq_exec,
	CCLBuffer *data, CCLBuffer *offsets, size_t num_segments, double *times_ms,
	GError **err);
/* The class layout the sorter's segmented sorts use (-1: not satradix). */
cl_int clo_sort_segmented_get_variant(CloSort *sorter);

/* Per-segment exclusive scan of data_in into data_out (the scanner's
 * element and sum types): within each segment, the scan of that segment
 * alone. One launch over the buffer, whatever the number of segments. The
 * capacity is the smaller of the two buffers' element counts. */
CCLEvent *clo_scan_segmented_with_device_data(CloScan *scanner, CCLQueue *cq_exec,
	CCLBuffer *data_in, CCLBuffer *data_out, CCLBuffer *offsets,
	size_t num_segments, GError **err);
cl_bool clo_scan_segmented_with_host_data(CloScan *scanner, CCLQueue *cq_exec,
	const void *data_in, void *data_out, size_t numel, const cl_ulong *offsets,
	size_t num_segments, GError **err);

/* ---------------------------------------------------------------------
 * CUDA graphs of queue work: everything enqueued on cq between
 * clo_queue_begin_capture and clo_queue_end_capture (by this thread) is
 * recorded instead of run, and replayed by clo_graph_launch. Device-data
 * calls of this library are capturable (satradix then runs every pass: it
 * skips no constant digit, which needs a host readback); host-data calls
 * and anything that waits are not. Temporaries become graph memory nodes.
 * --------------------------------------------------------------------- */
typedef struct clo_graph CloGraph;
cl_bool clo_queue_begin_capture(CCLQueue *cq, GError **err);
CloGraph *clo_queue_end_capture(CCLQueue *cq, GError **err);
cl_bool clo_graph_launch(CloGraph *graph, CCLQueue *cq, GError **err);
size_t clo_graph_get_num_nodes(CloGraph *graph);
void clo_graph_destroy(CloGraph *graph);

/* Test hook for the bounded lookback waits: tile `tile` of subsequent
 * scans withholds its status, so the next tile's wait runs out, the
 * kernel ends and the next synchronising call reports CLO_ERROR_LIBRARY.
 * -1 restores normal operation. */
void clo_gb300_debug_scan_withhold(long long tile);

#ifdef __cplusplus
}
#endif

#endif /* CLO_GB300_H */
