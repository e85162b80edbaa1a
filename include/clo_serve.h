/*
 * cl_ops on GB300 -- serving layer (no counterpart in the reference).
 *
 * A server owns one GPU context and runs sort, scan and random-fill
 * requests whose data live either in host memory (page-locked memory from
 * clo_host_alloc keeps the copies asynchronous) or in device memory of the
 * server's GPU (device-resident buffers: no host copies; small requests of
 * a batch are gathered into one buffer and scattered back by kernels).
 * Requests are admitted in
 * arrival order while their device footprint fits in the server's byte
 * budget; small requests of the same kind (sort or scan, same types) that
 * wait together are batched into one segmented call, which gives each of
 * them exactly the result it would get alone. Batches run on several CUDA
 * streams, so copies of one batch overlap the kernels of another. Every
 * request's latency (submission to completion of its result copy) is
 * recorded.
 */
#ifndef CLO_SERVE_H
#define CLO_SERVE_H

#include "clo_common.h"
#include "ccl_shim.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum clo_serve_op {
	CLO_SERVE_SORT = 0,     /* "satradix" sort of n elements of `type` */
	CLO_SERVE_SCAN = 1,     /* "blelloch" exclusive scan, `type` -> `sum_type` */
	CLO_SERVE_RNG_FILL = 2  /* clo_rng_fill of n states, `draws` each, 32 bits */
} CloServeOp;

typedef struct clo_serve_request {
	CloServeOp op;
	CloType type;      /* SORT / SCAN: element type (integer types) */
	CloType sum_type;  /* SCAN: sum type */
	size_t n;          /* SORT / SCAN: elements; RNG_FILL: generator states */
	size_t draws;      /* RNG_FILL: draws per state */
	int rng;           /* RNG_FILL: generator, index into clo_rng_infos */
	const void *in;    /* input: the elements, or the states' raw bytes */
	void *out;         /* output: n elements / n sums / draws * n uint32
	                    * (draw-major, as clo_rng_fill) */
	cl_bool device_data;  /* CL_TRUE: in and out are device pointers on the
	                       * server's GPU (device-resident buffers; `in` is
	                       * only read); CL_FALSE: host memory */
} CloServeRequest;

typedef struct clo_serve_stats {
	cl_ulong submitted, admitted, completed, failed, rejected;
	cl_ulong batches;       /* admitted groups, one device call sequence each */
	cl_ulong max_queued;    /* most requests waiting for admission at once */
	size_t budget_bytes;
	size_t peak_bytes;      /* most budget bytes held by admitted requests */
	double p50_ms, p99_ms, max_ms, mean_ms;  /* latency of completed requests */
	double elements;        /* elements (draws for RNG_FILL) completed */
	double span_s;          /* first submission to last completion */
	/* Device overlap, from each batch's [start, end] on the device (events
	 * recorded on its stream before its first and after its last
	 * operation): the most batches in flight at one time, the time at
	 * least one was in flight, and the batches' summed device time over
	 * that time (1.0 = no overlap). */
	cl_ulong max_concurrent_batches;
	double device_busy_s;
	double mean_concurrent_batches;
} CloServeStats;

typedef struct clo_server CloServer;

/* Budget: device bytes that admitted requests may hold at once (inputs,
 * outputs and scratch, as clo_serve_footprint estimates them). streams:
 * concurrent batches (1..16). */
CloServer *clo_serve_new(CCLContext *ctx, size_t budget_bytes, int streams,
	GError **err);

/* Queues a request (the descriptor is copied; the host buffers must stay
 * valid until it completes). Returns its ticket (> 0), or 0 with
 * CLO_ERROR_ARGS for a malformed request or one whose footprint exceeds the
 * budget. */
cl_ulong clo_serve_submit(CloServer *srv, const CloServeRequest *req, GError **err);

/* Blocks until the ticket's request completes; its latency in ms. A failed
 * request sets CLO_ERROR_LIBRARY. */
cl_bool clo_serve_wait(CloServer *srv, cl_ulong ticket, double *latency_ms,
	GError **err);

/* Blocks until every submitted request has completed; reports device
 * errors (bounded-wait timeouts, invalid offsets) seen meanwhile. */
cl_bool clo_serve_drain(CloServer *srv, GError **err);

/* Open-loop driver: submits reqs[i] at arrival_s[i] seconds (non-
 * decreasing) after the call starts, whatever the server's progress, and
 * returns when all are submitted (tickets[i] receives each ticket, 0 for
 * a rejected request). */
cl_bool clo_serve_replay(CloServer *srv, const CloServeRequest *reqs,
	const double *arrival_s, size_t count, cl_ulong *tickets, GError **err);

/* Batching policy: requests of at most small_n elements are batched, a
 * batch holds at most batch_elems elements and max_batch (1..4096)
 * requests. The defaults are 2^20, 2^26 and 4096; max_batch 1 turns
 * batching off (every request runs alone through the plain kernels).
 * Takes effect for batches formed after the call. */
cl_bool clo_serve_configure(CloServer *srv, size_t small_n, size_t batch_elems,
	size_t max_batch, GError **err);

void clo_serve_get_stats(CloServer *srv, CloServeStats *stats);
void clo_serve_reset_stats(CloServer *srv);

/* Drains, then frees the server. */
void clo_serve_destroy(CloServer *srv);

/* The admission and batching policy, as pure host functions.
 * clo_serve_footprint: device bytes a request holds while it runs (0 for a
 * malformed request). clo_serve_select: given the waiting requests in
 * arrival order and the free budget, writes the indices of the next batch
 * to `chosen` (at most max_batch) and returns how many: none when the
 * oldest does not fit; else the oldest, plus -- when it is a small sort or
 * scan (n <= small_n) -- later waiting requests of the same op and types
 * that are small too (and whose data live in the same kind of memory),
 * while their elements total at most batch_elems and their footprints
 * fit. */
size_t clo_serve_footprint(const CloServeRequest *req);
size_t clo_serve_select(const CloServeRequest *pending, size_t npending,
	size_t free_bytes, size_t small_n, size_t batch_elems, size_t max_batch,
	size_t *chosen);

#ifdef __cplusplus
}
#endif

#endif /* CLO_SERVE_H */
