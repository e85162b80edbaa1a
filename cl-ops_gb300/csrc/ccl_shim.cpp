// CUDA-backed implementations of the cf4ocl2 wrapper calls the reference
// API is written against (see include/ccl_shim.h for the mapping).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "clo_internal.h"

namespace clo {
long live_wrappers();
}

using clo::cuda_ok;
using clo::set_error;

namespace {

std::once_flag g_pool_once[64];

// Library temporaries come from the device's default stream-ordered pool.
// Keeping freed blocks cached (release threshold = max) turns per-call
// temporaries into pool hits instead of driver allocations; this is a
// property of this process's pool only.
void configure_pool(int ordinal) {
	if (ordinal < 0 || ordinal >= 64) return;
	std::call_once(g_pool_once[ordinal], [ordinal]() {
		cudaMemPool_t pool;
		if (cudaDeviceGetDefaultMemPool(&pool, ordinal) == cudaSuccess) {
			uint64_t thr = UINT64_MAX;
			cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold,
				&thr);
		}
	});
}

CCLContext *context_new(int ordinal, GError **err) {
	int ndev = 0;
	if (!cuda_ok(cudaGetDeviceCount(&ndev), err, "cudaGetDeviceCount"))
		return nullptr;
	if (ndev == 0) {
		set_error(err, CLO_ERROR_LIBRARY, "No CUDA device available");
		return nullptr;
	}
	if (ordinal < 0) ordinal = 0;
	if (ordinal >= ndev) {
		set_error(err, CLO_ERROR_ARGS, "Device index %d out of range (%d)",
			ordinal, ndev);
		return nullptr;
	}
	if (!cuda_ok(cudaSetDevice(ordinal), err, "cudaSetDevice")) return nullptr;
	CCLContext *ctx = new ccl_context();
	ctx->refcount = 1;
	ctx->ordinal = ordinal;
	ctx->device.ordinal = ordinal;
	cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
		ordinal);
	int optin = 0;
	cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
		ordinal);
	ctx->smem_optin = (size_t)optin;
	ctx->d_status = nullptr;
	ctx->h_status = nullptr;
	if (!cuda_ok(cudaMalloc(&ctx->d_status, 4 * sizeof(int)), err,
			"cudaMalloc(status)") ||
		!cuda_ok(cudaMemset(ctx->d_status, 0, 4 * sizeof(int)), err,
			"cudaMemset(status)") ||
		!cuda_ok(cudaMallocHost(&ctx->h_status, 4 * sizeof(int)), err,
			"cudaMallocHost(status)")) {
		if (ctx->d_status) cudaFree(ctx->d_status);
		delete ctx;
		return nullptr;
	}
	configure_pool(ordinal);
	clo::wrapper_created();
	return ctx;
}

void event_release(ccl_event *e) {
	if (e->start) cudaEventDestroy(e->start);
	if (e->end) cudaEventDestroy(e->end);
	delete e;
	clo::wrapper_destroyed();
}

}  // namespace

namespace clo {

void *tmp_alloc(CCLContext *ctx, size_t bytes, cudaStream_t s, GError **err) {
	void *p = nullptr;
	if (bytes == 0) bytes = 16;
	cudaSetDevice(ctx->ordinal);
	cudaError_t e = cudaMallocAsync(&p, bytes, s);
	if (e != cudaSuccess) {
		cudaGetLastError();
		set_error(err, CLO_ERROR_LIBRARY,
			"Unable to allocate %zu bytes of device scratch: %s", bytes,
			cudaGetErrorString(e));
		return nullptr;
	}
	return p;
}

void tmp_free(void *p, cudaStream_t s) {
	if (p) cudaFreeAsync(p, s);
}

bool stream_capturing(cudaStream_t s) {
	cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return st != cudaStreamCaptureStatusNone;
}

ccl_event *event_begin(CCLQueue *q, const char *name) {
	ccl_event *e = nullptr;
	if (!q->free_events.empty()) {
		e = q->free_events.back();
		q->free_events.pop_back();
	} else {
		e = new ccl_event();
		e->timing = q->profiling;
		unsigned flags = q->profiling ? cudaEventDefault
									  : cudaEventDisableTiming;
		cudaEventCreateWithFlags(&e->start, flags);
		cudaEventCreateWithFlags(&e->end, flags);
		e->queue = q;
		wrapper_created();
	}
	e->name = name ? name : "";
	e->started = false;
	if (e->timing && !stream_capturing(q->stream)) {
		cudaEventRecord(e->start, q->stream);
		e->started = true;
	}
	q->events.push_back(e);
	return e;
}

void event_end(ccl_event *e) {
	if (!stream_capturing(e->queue->stream))
		cudaEventRecord(e->end, e->queue->stream);
}

bool wait_ewl(CCLQueue *q, CCLEventWaitList *ewl, GError **err) {
	if (ewl == nullptr || *ewl == nullptr) return true;
	for (ccl_event *e : (*ewl)->evts) {
		if (e && e->queue != q) {
			if (!cuda_ok(cudaStreamWaitEvent(q->stream, e->end, 0), err,
					"cudaStreamWaitEvent"))
				return false;
		}
	}
	ccl_event_wait_list_clear(ewl);
	return true;
}

bool check_device_status(CCLContext *ctx, GError **err) {
	int st[2] = {0, 0};
	if (!cuda_ok(cudaMemcpy(st, ctx->d_status, 2 * sizeof(int),
			cudaMemcpyDeviceToHost), err, "status readback"))
		return false;
	if (st[0] == DEV_ERR_BAD_SEGMENTS) {
		cudaMemset(ctx->d_status, 0, 2 * sizeof(int));
		set_error(err, CLO_ERROR_ARGS,
			"Segment offsets are invalid (segment %d: offsets must not decrease "
			"and must stay within the buffer, segments shorter than 2^30); "
			"results of the operation are invalid", st[1]);
		return false;
	}
	if (st[0] != DEV_OK) {
		cudaMemset(ctx->d_status, 0, 2 * sizeof(int));
		set_error(err, CLO_ERROR_LIBRARY,
			"Device watchdog: a bounded spin-wait gave up (code %d, tile %d);"
			" results of the operation are invalid", st[0], st[1]);
		return false;
	}
	return true;
}

}  // namespace clo

extern "C" {

// ---------------------------------------------------------------- context
CCLContext *ccl_context_new_any(GError **err) { return context_new(0, err); }
CCLContext *ccl_context_new_gpu(GError **err) { return context_new(0, err); }

CCLContext *ccl_context_new_from_menu_full(void *data, GError **err) {
	int ordinal = data ? *(int *)data : 0;
	return context_new(ordinal < 0 ? 0 : ordinal, err);
}

CCLContext *ccl_context_new_from_device_index(int ordinal, GError **err) {
	return context_new(ordinal, err);
}

void ccl_context_ref(CCLContext *ctx) {
	if (ctx) ctx->refcount.fetch_add(1);
}

void ccl_context_unref(CCLContext *ctx) {
	if (!ctx) return;
	if (ctx->refcount.fetch_sub(1) == 1) {
		cudaSetDevice(ctx->ordinal);
		cudaFree(ctx->d_status);
		cudaFreeHost(ctx->h_status);
		delete ctx;
		clo::wrapper_destroyed();
	}
}

void ccl_context_destroy(CCLContext *ctx) { ccl_context_unref(ctx); }

cl_uint ccl_context_get_num_devices(CCLContext *ctx, GError **err) {
	(void)err;
	return ctx ? 1u : 0u;
}

CCLDevice *ccl_context_get_device(CCLContext *ctx, cl_uint index,
	GError **err) {
	if (!ctx || index != 0) {
		set_error(err, CLO_ERROR_ARGS, "Context has no device %u", index);
		return nullptr;
	}
	return &ctx->device;
}

int ccl_device_get_ordinal(CCLDevice *dev) { return dev ? dev->ordinal : -1; }

// ------------------------------------------------------------------ queue
static CCLQueue *queue_make(CCLContext *ctx, cudaStream_t s, bool owned,
	cl_command_queue_properties props) {
	CCLQueue *q = new ccl_queue();
	q->ctx = ctx;
	ccl_context_ref(ctx);
	q->stream = s;
	q->owned = owned;
	q->profiling = (props & CL_QUEUE_PROFILING_ENABLE) != 0;
	clo::wrapper_created();
	return q;
}

CCLQueue *ccl_queue_new(CCLContext *ctx, CCLDevice *dev,
	cl_command_queue_properties properties, GError **err) {
	if (!ctx) {
		set_error(err, CLO_ERROR_ARGS, "NULL context");
		return nullptr;
	}
	(void)dev;
	cudaSetDevice(ctx->ordinal);
	cudaStream_t s;
	if (!cuda_ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), err,
			"cudaStreamCreate"))
		return nullptr;
	return queue_make(ctx, s, true, properties);
}

CCLQueue *ccl_queue_new_wrap(CCLContext *ctx, void *cuda_stream,
	cl_command_queue_properties properties, GError **err) {
	if (!ctx) {
		set_error(err, CLO_ERROR_ARGS, "NULL context");
		return nullptr;
	}
	return queue_make(ctx, (cudaStream_t)cuda_stream, false, properties);
}

void ccl_queue_gc(CCLQueue *cq) {
	if (!cq) return;
	for (ccl_event *e : cq->events) cq->free_events.push_back(e);
	cq->events.clear();
}

void ccl_queue_destroy(CCLQueue *cq) {
	if (!cq) return;
	cudaSetDevice(cq->ctx->ordinal);
	cudaStreamSynchronize(cq->stream);
	for (ccl_event *e : cq->events) event_release(e);
	for (ccl_event *e : cq->free_events) event_release(e);
	if (cq->owned) cudaStreamDestroy(cq->stream);
	ccl_context_unref(cq->ctx);
	delete cq;
	clo::wrapper_destroyed();
}

cl_bool ccl_queue_finish(CCLQueue *cq, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return CL_FALSE;
	}
	if (!cuda_ok(cudaStreamSynchronize(cq->stream), err, "ccl_queue_finish"))
		return CL_FALSE;
	return clo::check_device_status(cq->ctx, err) ? CL_TRUE : CL_FALSE;
}

CCLDevice *ccl_queue_get_device(CCLQueue *cq, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	return &cq->ctx->device;
}

CCLContext *ccl_queue_get_context(CCLQueue *cq, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	return cq->ctx;
}

void *ccl_queue_unwrap(CCLQueue *cq) { return cq ? (void *)cq->stream : nullptr; }

// ---------------------------------------------------------------- buffers
CCLBuffer *ccl_buffer_new(CCLContext *ctx, cl_mem_flags flags, size_t size,
	void *host_ptr, GError **err) {
	if (!ctx) {
		set_error(err, CLO_ERROR_ARGS, "NULL context");
		return nullptr;
	}
	cudaSetDevice(ctx->ordinal);
	void *p = nullptr;
	if (!cuda_ok(cudaMalloc(&p, size ? size : 16), err, "ccl_buffer_new"))
		return nullptr;
	if ((flags & CL_MEM_COPY_HOST_PTR) && host_ptr && size) {
		if (!cuda_ok(cudaMemcpy(p, host_ptr, size, cudaMemcpyHostToDevice),
				err, "ccl_buffer_new(copy)")) {
			cudaFree(p);
			return nullptr;
		}
	}
	CCLBuffer *b = new ccl_buffer();
	b->refcount = 1;
	b->ctx = ctx;
	ccl_context_ref(ctx);
	b->ptr = p;
	b->size = size;
	b->owned = true;
	clo::wrapper_created();
	return b;
}

CCLBuffer *ccl_buffer_new_wrap(CCLContext *ctx, void *dev_ptr, size_t size,
	GError **err) {
	if (!ctx) {
		set_error(err, CLO_ERROR_ARGS, "NULL context");
		return nullptr;
	}
	CCLBuffer *b = new ccl_buffer();
	b->refcount = 1;
	b->ctx = ctx;
	ccl_context_ref(ctx);
	b->ptr = dev_ptr;
	b->size = size;
	b->owned = false;
	clo::wrapper_created();
	return b;
}

void ccl_buffer_ref(CCLBuffer *buf) {
	if (buf) buf->refcount.fetch_add(1);
}

void ccl_buffer_destroy(CCLBuffer *buf) {
	if (!buf) return;
	if (buf->refcount.fetch_sub(1) == 1) {
		if (buf->owned) {
			cudaSetDevice(buf->ctx->ordinal);
			cudaFree(buf->ptr);
		}
		ccl_context_unref(buf->ctx);
		delete buf;
		clo::wrapper_destroyed();
	}
}

void *ccl_buffer_unwrap(CCLBuffer *buf) { return buf ? buf->ptr : nullptr; }
size_t ccl_buffer_get_size(CCLBuffer *buf) { return buf ? buf->size : 0; }

static bool range_ok(CCLBuffer *b, size_t off, size_t size, GError **err) {
	if (!b || off > b->size || size > b->size - off) {
		set_error(err, CLO_ERROR_ARGS,
			"Transfer of %zu bytes at offset %zu exceeds buffer of %zu bytes",
			size, off, b ? b->size : (size_t)0);
		return false;
	}
	return true;
}

CCLEvent *ccl_buffer_enqueue_read(CCLBuffer *buf, CCLQueue *cq,
	cl_bool blocking_read, size_t offset, size_t size, void *ptr,
	CCLEventWaitList *evt_wait_lst, GError **err) {
	if (!cq || !range_ok(buf, offset, size, err)) {
		if (!cq) set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	if (!clo::wait_ewl(cq, evt_wait_lst, err)) return nullptr;
	ccl_event *e = clo::event_begin(cq, "read");
	if (!cuda_ok(cudaMemcpyAsync(ptr, (char *)buf->ptr + offset, size,
			cudaMemcpyDeviceToHost, cq->stream), err, "enqueue_read"))
		return nullptr;
	clo::event_end(e);
	if (blocking_read &&
		!cuda_ok(cudaEventSynchronize(e->end), err, "enqueue_read(wait)"))
		return nullptr;
	return e;
}

CCLEvent *ccl_buffer_enqueue_write(CCLBuffer *buf, CCLQueue *cq,
	cl_bool blocking_write, size_t offset, size_t size, const void *ptr,
	CCLEventWaitList *evt_wait_lst, GError **err) {
	if (!cq || !range_ok(buf, offset, size, err)) {
		if (!cq) set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	if (!clo::wait_ewl(cq, evt_wait_lst, err)) return nullptr;
	ccl_event *e = clo::event_begin(cq, "write");
	if (!cuda_ok(cudaMemcpyAsync((char *)buf->ptr + offset, ptr, size,
			cudaMemcpyHostToDevice, cq->stream), err, "enqueue_write"))
		return nullptr;
	clo::event_end(e);
	if (blocking_write &&
		!cuda_ok(cudaEventSynchronize(e->end), err, "enqueue_write(wait)"))
		return nullptr;
	return e;
}

CCLEvent *ccl_buffer_enqueue_copy(CCLBuffer *src_buf, CCLBuffer *dst_buf,
	CCLQueue *cq, size_t src_offset, size_t dst_offset, size_t size,
	CCLEventWaitList *evt_wait_lst, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	if (!range_ok(src_buf, src_offset, size, err) ||
		!range_ok(dst_buf, dst_offset, size, err))
		return nullptr;
	if (!clo::wait_ewl(cq, evt_wait_lst, err)) return nullptr;
	ccl_event *e = clo::event_begin(cq, "copy");
	if (!cuda_ok(cudaMemcpyAsync((char *)dst_buf->ptr + dst_offset,
			(char *)src_buf->ptr + src_offset, size, cudaMemcpyDeviceToDevice,
			cq->stream), err, "enqueue_copy"))
		return nullptr;
	clo::event_end(e);
	return e;
}

// ----------------------------------------------------------------- events
static void ewl_append(CCLEventWaitList *ewl, va_list ap) {
	if (!ewl) return;
	for (;;) {
		CCLEvent *e = va_arg(ap, CCLEvent *);
		if (!e) break;
		if (!*ewl) *ewl = new ccl_ewl_impl();
		(*ewl)->evts.push_back(e);
	}
}

CCLEventWaitList *ccl_ewl(CCLEventWaitList *evt_wait_lst, ...) {
	va_list ap;
	va_start(ap, evt_wait_lst);
	ewl_append(evt_wait_lst, ap);
	va_end(ap);
	return evt_wait_lst;
}

void ccl_event_wait_list_add(CCLEventWaitList *evt_wait_lst, ...) {
	va_list ap;
	va_start(ap, evt_wait_lst);
	ewl_append(evt_wait_lst, ap);
	va_end(ap);
}

void ccl_event_wait_list_clear(CCLEventWaitList *evt_wait_lst) {
	if (evt_wait_lst && *evt_wait_lst) {
		delete *evt_wait_lst;
		*evt_wait_lst = nullptr;
	}
}

cl_bool ccl_event_wait(CCLEventWaitList *evt_wait_lst, GError **err) {
	if (!evt_wait_lst || !*evt_wait_lst) return CL_TRUE;
	bool ok = true;
	CCLContext *ctx = nullptr;
	for (ccl_event *e : (*evt_wait_lst)->evts) {
		if (!e) continue;
		if (!cuda_ok(cudaEventSynchronize(e->end), err, "ccl_event_wait")) {
			ok = false;
			break;
		}
		ctx = e->queue->ctx;
	}
	ccl_event_wait_list_clear(evt_wait_lst);
	if (ok && ctx) ok = clo::check_device_status(ctx, err);
	return ok ? CL_TRUE : CL_FALSE;
}

void ccl_event_set_name(CCLEvent *evt, const char *name) {
	if (evt) evt->name = name ? name : "";
}

const char *ccl_event_get_name(CCLEvent *evt) {
	return evt ? evt->name.c_str() : nullptr;
}

cl_ulong ccl_event_get_duration(CCLEvent *evt, GError **err) {
	if (!evt || !evt->timing || !evt->started) {
		set_error(err, CLO_ERROR_ARGS,
			"Event has no timing (queue without CL_QUEUE_PROFILING_ENABLE)");
		return 0;
	}
	if (!cuda_ok(cudaEventSynchronize(evt->end), err, "event sync"))
		return 0;
	float ms = 0.f;
	if (!cuda_ok(cudaEventElapsedTime(&ms, evt->start, evt->end), err,
			"cudaEventElapsedTime"))
		return 0;
	return (cl_ulong)((double)ms * 1.0e6);
}

CCLEvent *ccl_enqueue_marker(CCLQueue *cq, CCLEventWaitList *evt_wait_lst,
	GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	if (!clo::wait_ewl(cq, evt_wait_lst, err)) return nullptr;
	ccl_event *e = clo::event_begin(cq, "marker");
	clo::event_end(e);
	return e;
}

cl_ulong ccl_event_elapsed_ns(CCLEvent *from, CCLEvent *to, GError **err) {
	if (!from || !to || !from->timing || !to->timing) {
		set_error(err, CLO_ERROR_ARGS,
			"Events have no timing (queue without CL_QUEUE_PROFILING_ENABLE)");
		return 0;
	}
	if (!cuda_ok(cudaEventSynchronize(to->end), err, "event sync")) return 0;
	float ms = 0.f;
	if (!cuda_ok(cudaEventElapsedTime(&ms, from->end, to->end), err,
			"cudaEventElapsedTime"))
		return 0;
	return (cl_ulong)((double)ms * 1.0e6);
}

const char *ccl_program_get_source(CCLProgram *prg) {
	return prg ? prg->src.c_str() : nullptr;
}

const char *ccl_program_get_build_options(CCLProgram *prg) {
	return prg ? prg->opts.c_str() : nullptr;
}

cl_bool ccl_wrapper_memcheck(void) {
	return clo::live_wrappers() == 0 ? CL_TRUE : CL_FALSE;
}

// ----------------------------------------------------------------- extras
void *clo_host_alloc(size_t size, GError **err) {
	void *p = nullptr;
	if (!cuda_ok(cudaMallocHost(&p, size ? size : 16), err, "cudaMallocHost"))
		return nullptr;
	return p;
}

void clo_host_free(void *ptr) {
	if (ptr) cudaFreeHost(ptr);
}

// ------------------------------------------------------------ CUDA graphs
cl_bool clo_queue_begin_capture(CCLQueue *cq, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return CL_FALSE;
	}
	cudaSetDevice(cq->ctx->ordinal);
	return cuda_ok(cudaStreamBeginCapture(cq->stream, cudaStreamCaptureModeThreadLocal),
		err, "cudaStreamBeginCapture") ? CL_TRUE : CL_FALSE;
}

CloGraph *clo_queue_end_capture(CCLQueue *cq, GError **err) {
	if (!cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL queue");
		return nullptr;
	}
	cudaSetDevice(cq->ctx->ordinal);
	cudaGraph_t g = nullptr;
	if (!cuda_ok(cudaStreamEndCapture(cq->stream, &g), err, "cudaStreamEndCapture"))
		return nullptr;
	cudaGraphExec_t x = nullptr;
	if (!cuda_ok(cudaGraphInstantiate(&x, g, 0), err, "cudaGraphInstantiate")) {
		cudaGraphDestroy(g);
		return nullptr;
	}
	CloGraph *r = new CloGraph();
	r->graph = g;
	r->exec = x;
	r->ctx = cq->ctx;
	ccl_context_ref(cq->ctx);
	size_t nodes = 0;
	cudaGraphGetNodes(g, nullptr, &nodes);
	r->nodes = nodes;
	clo::wrapper_created();
	return r;
}

cl_bool clo_graph_launch(CloGraph *g, CCLQueue *cq, GError **err) {
	if (!g || !cq) {
		set_error(err, CLO_ERROR_ARGS, "NULL graph or queue");
		return CL_FALSE;
	}
	cudaSetDevice(cq->ctx->ordinal);
	return cuda_ok(cudaGraphLaunch(g->exec, cq->stream), err, "cudaGraphLaunch")
		? CL_TRUE : CL_FALSE;
}

size_t clo_graph_get_num_nodes(CloGraph *g) { return g ? g->nodes : 0; }

void clo_graph_destroy(CloGraph *g) {
	if (!g) return;
	cudaSetDevice(g->ctx->ordinal);
	cudaGraphExecDestroy(g->exec);
	cudaGraphDestroy(g->graph);
	ccl_context_unref(g->ctx);
	delete g;
	clo::wrapper_destroyed();
}

}  // extern "C"
