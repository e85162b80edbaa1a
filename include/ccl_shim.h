/*
 * cl_ops on GB300 -- CUDA-backed stand-ins for the cf4ocl2 wrapper
 * handles the reference API is written against.
 *
 * The reference passes cf4ocl2 objects (CCLContext, CCLDevice, CCLQueue,
 * CCLBuffer, CCLEvent, CCLProgram) through every entry point
 * (src/cl_ops/sort/clo_sort_abstract.in.h:116-170,
 * src/cl_ops/scan/clo_scan_abstract.in.h:109-162,
 * src/cl_ops/rng/clo_rng.in.h:97-111). cf4ocl2 itself is a third-party
 * OpenCL wrapper and is not part of this library; what is declared here is
 * the subset of its API that the reference's library code, tests
 * (src/tests/test_rng.c) and benchmarks (src/benchmarks/clo_*_bench.c) call, with the
 * same names and argument meanings, mapped onto CUDA:
 *
 *   CCLContext  one CUDA device (primary context) + a stream-ordered
 *               memory pool for library temporaries + a device status
 *               word that bounded spin-waits report into.
 *   CCLDevice   a device ordinal.
 *   CCLQueue    a cudaStream_t (created, or wrapped with ccl_queue_new_wrap).
 *   CCLBuffer   a device allocation {pointer, size, reference count}.
 *   CCLEvent    a pair of cudaEvents bracketing one enqueued operation;
 *               owned by the queue it was enqueued on.
 *   CCLProgram  a descriptor of the compiled-in kernels a sorter/scanner
 *               uses, or a program built by NVRTC from a caller's CUDA
 *               source (ccl_program_new_from_source).
 *   CCLKernel   a kernel of such a program (owned by the program).
 *
 * Functions marked [addition] have no cf4ocl2 counterpart with the same
 * signature; they exist because a CUDA pointer or stream carries no
 * size or context information of its own.
 */
#ifndef CCL_SHIM_H
#define CCL_SHIM_H

#include "clo_common.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ccl_context CCLContext;
typedef struct ccl_device CCLDevice;
typedef struct ccl_queue CCLQueue;
typedef struct ccl_buffer CCLBuffer;
typedef struct ccl_event CCLEvent;
typedef struct ccl_program CCLProgram;
typedef struct ccl_kernel CCLKernel;
typedef struct ccl_arg CCLArg;
typedef struct ccl_ewl_impl *CCLEventWaitList;

/* Memory flags accepted by ccl_buffer_new (OpenCL values). Only
 * CL_MEM_COPY_HOST_PTR changes behaviour: the buffer is initialised from
 * host_ptr. */
#ifndef CL_MEM_READ_WRITE
#define CL_MEM_READ_WRITE (1 << 0)
#define CL_MEM_WRITE_ONLY (1 << 1)
#define CL_MEM_READ_ONLY (1 << 2)
#define CL_MEM_USE_HOST_PTR (1 << 3)
#define CL_MEM_ALLOC_HOST_PTR (1 << 4)
#define CL_MEM_COPY_HOST_PTR (1 << 5)
#endif
#ifndef CL_QUEUE_PROFILING_ENABLE
#define CL_QUEUE_OUT_OF_ORDER_EXEC_MODE_ENABLE (1 << 0)
#define CL_QUEUE_PROFILING_ENABLE (1 << 1)
#endif
typedef cl_ulong cl_mem_flags;
typedef cl_ulong cl_command_queue_properties;

/* ---- context ---------------------------------------------------------- */
CCLContext *ccl_context_new_any(GError **err);
CCLContext *ccl_context_new_gpu(GError **err);
/* cf4ocl2 shows a device menu; here *data (int*, may be NULL) selects the
 * CUDA device ordinal, -1 or NULL meaning device 0. */
CCLContext *ccl_context_new_from_menu_full(void *data, GError **err);
/* [addition] context on CUDA device `ordinal`. */
CCLContext *ccl_context_new_from_device_index(int ordinal, GError **err);
void ccl_context_destroy(CCLContext *ctx);
void ccl_context_ref(CCLContext *ctx);
void ccl_context_unref(CCLContext *ctx);
cl_uint ccl_context_get_num_devices(CCLContext *ctx, GError **err);
CCLDevice *ccl_context_get_device(CCLContext *ctx, cl_uint index,
	GError **err);
/* [addition] CUDA ordinal of a device handle. */
int ccl_device_get_ordinal(CCLDevice *dev);

/* ---- queue ------------------------------------------------------------ */
CCLQueue *ccl_queue_new(CCLContext *ctx, CCLDevice *dev,
	cl_command_queue_properties properties, GError **err);
/* [addition] wrap an existing cudaStream_t (0 = legacy default stream);
 * the stream is not destroyed by ccl_queue_destroy. */
CCLQueue *ccl_queue_new_wrap(CCLContext *ctx, void *cuda_stream,
	cl_command_queue_properties properties, GError **err);
void ccl_queue_destroy(CCLQueue *cq);
cl_bool ccl_queue_finish(CCLQueue *cq, GError **err);
CCLDevice *ccl_queue_get_device(CCLQueue *cq, GError **err);
CCLContext *ccl_queue_get_context(CCLQueue *cq, GError **err);
/* [addition] the underlying cudaStream_t. */
void *ccl_queue_unwrap(CCLQueue *cq);
/* Releases the events the queue owns (cf4ocl2 ccl_queue_gc). */
void ccl_queue_gc(CCLQueue *cq);

/* ---- buffers ---------------------------------------------------------- */
CCLBuffer *ccl_buffer_new(CCLContext *ctx, cl_mem_flags flags, size_t size,
	void *host_ptr, GError **err);
/* [addition] wrap caller-owned device memory (not freed on destroy). */
CCLBuffer *ccl_buffer_new_wrap(CCLContext *ctx, void *dev_ptr, size_t size,
	GError **err);
void ccl_buffer_destroy(CCLBuffer *buf);
void ccl_buffer_ref(CCLBuffer *buf);
/* [addition] device pointer and size of a buffer. */
void *ccl_buffer_unwrap(CCLBuffer *buf);
size_t ccl_buffer_get_size(CCLBuffer *buf);

CCLEvent *ccl_buffer_enqueue_read(CCLBuffer *buf, CCLQueue *cq,
	cl_bool blocking_read, size_t offset, size_t size, void *ptr,
	CCLEventWaitList *evt_wait_lst, GError **err);
CCLEvent *ccl_buffer_enqueue_write(CCLBuffer *buf, CCLQueue *cq,
	cl_bool blocking_write, size_t offset, size_t size, const void *ptr,
	CCLEventWaitList *evt_wait_lst, GError **err);
CCLEvent *ccl_buffer_enqueue_copy(CCLBuffer *src_buf, CCLBuffer *dst_buf,
	CCLQueue *cq, size_t src_offset, size_t dst_offset, size_t size,
	CCLEventWaitList *evt_wait_lst, GError **err);

/* ---- events ----------------------------------------------------------- */
/* Appends the NULL-terminated list of events to *evt_wait_lst and
 * returns evt_wait_lst (cf4ocl2 ccl_ewl). */
CCLEventWaitList *ccl_ewl(CCLEventWaitList *evt_wait_lst, ...);
void ccl_event_wait_list_add(CCLEventWaitList *evt_wait_lst, ...);
void ccl_event_wait_list_clear(CCLEventWaitList *evt_wait_lst);
/* Blocks until every event in the list completed; clears the list.
 * Returns CL_FALSE and sets err when a device-side watchdog fired. */
cl_bool ccl_event_wait(CCLEventWaitList *evt_wait_lst, GError **err);
void ccl_event_set_name(CCLEvent *evt, const char *name);
const char *ccl_event_get_name(CCLEvent *evt);
/* [addition] elapsed device time of the operation in nanoseconds (the
 * queue must have CL_QUEUE_PROFILING_ENABLE); waits for completion. */
cl_ulong ccl_event_get_duration(CCLEvent *evt, GError **err);

/* Enqueues a marker: an event that completes when everything enqueued
 * before it on cq has completed (cf4ocl2 ccl_enqueue_marker). */
CCLEvent *ccl_enqueue_marker(CCLQueue *cq, CCLEventWaitList *evt_wait_lst,
	GError **err);
/* [addition] device time in nanoseconds from the completion of `from` to
 * the completion of `to` (both on profiling queues); waits for `to`. */
cl_ulong ccl_event_elapsed_ns(CCLEvent *from, CCLEvent *to, GError **err);

/* ---- programs --------------------------------------------------------- */
const char *ccl_program_get_source(CCLProgram *prg);
const char *ccl_program_get_build_options(CCLProgram *prg);

/* Client programs, as src/tests/test_rng.c:79-115 builds one around the
 * text of clo_rng_get_source(). The source is CUDA; kernels that
 * ccl_program_get_kernel looks up are declared extern "C" __global__.
 * ccl_program_build compiles it with NVRTC for the context's device
 * (options are passed to NVRTC); a compile error is CLO_ERROR_LIBRARY
 * with NVRTC's log, which ccl_program_get_build_log also returns.
 * The program refs its context; ccl_program_destroy releases it and its
 * kernels (it ignores a sorter's or scanner's program, which its owner
 * releases). */
CCLProgram *ccl_program_new_from_source(CCLContext *ctx, const char *string,
	GError **err);
CCLProgram *ccl_program_new_from_sources(CCLContext *ctx, cl_uint count,
	const char **strings, const size_t *lengths, GError **err);
cl_bool ccl_program_build(CCLProgram *prg, const char *options, GError **err);
const char *ccl_program_get_build_log(CCLProgram *prg, GError **err);
CCLKernel *ccl_program_get_kernel(CCLProgram *prg, const char *kernel_name,
	GError **err);
void ccl_program_destroy(CCLProgram *prg);

/* Kernel arguments (cf4ocl2 ccl_arg_*): a value's bytes, or (value NULL)
 * a local-memory size, which adds to the launch's dynamic shared memory
 * (reached in the kernel through extern __shared__) and takes no
 * parameter slot. Arguments passed to an enqueue are released by it. */
CCLArg *ccl_arg_new(void *value, size_t size);
void ccl_arg_destroy(CCLArg *arg);
#define ccl_arg_priv(value, type) ccl_arg_new(&(value), sizeof(type))
#define ccl_arg_local(count, type) ccl_arg_new(NULL, (count) * sizeof(type))
#define ccl_arg_full(value, size) ccl_arg_new((value), (size))

/* One dimension only. Without a global size the suggestion is the largest
 * work-group of at most 256 that divides the real size; with one, 256 (or
 * the real size if smaller) and the global size rounded up to it. */
cl_bool ccl_kernel_suggest_worksizes(CCLKernel *krnl, CCLDevice *dev, cl_uint dims,
	const size_t *real_worksize, size_t *gws, size_t *lws, GError **err);
/* Launches global_work_size[0] / local_work_size[0] blocks of
 * local_work_size[0] threads (the global size must be a multiple of the
 * local one; a NULL local size takes the suggestion above) on cq after the
 * events of evt_wait_lst. The variadic arguments, NULL-terminated, are
 * the kernel's parameters in order: a CCLBuffer* passes its device
 * pointer, a CCLArg* its value. Returns the launch's event. */
CCLEvent *ccl_kernel_set_args_and_enqueue_ndrange(CCLKernel *krnl, CCLQueue *cq,
	cl_uint work_dim, const size_t *global_work_offset, const size_t *global_work_size,
	const size_t *local_work_size, CCLEventWaitList *evt_wait_lst, GError **err, ...);

/* True when every wrapper object created so far has been released
 * (cf4ocl2 ccl_wrapper_memcheck). */
cl_bool ccl_wrapper_memcheck(void);

#ifdef __cplusplus
}
#endif

#endif /* CCL_SHIM_H */
