/*
 * cl_ops on GB300 -- sorter object API and implementation registry.
 *
 * Same plugin interface and entry points as the reference's
 * src/cl_ops/sort/clo_sort_abstract.in.h:43-170. Registered
 * implementations (clo_sort_abstract.c:111-117): "sbitonic", "abitonic",
 * "gselect", "satradix". Each is backed by hand-written sm_103a kernels;
 * `init` returns a short descriptor string instead of OpenCL source
 * (NULL on error, as in the reference).
 */
#ifndef CLO_SORT_ABSTRACT_H
#define CLO_SORT_ABSTRACT_H

#include "clo_common.h"
#include "ccl_shim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CLO_SORT_IMPLS "sbitonic, abitonic, gselect, satradix"

/* clo_sort_abstract.in.h:43-110 */
typedef struct clo_sort_impl_def {
	const char *name;
	cl_bool in_place;
	const char *(*init)(CloSort *sorter, const char *options, GError **err);
	void (*finalize)(CloSort *sorter);
	CCLEvent *(*sort_with_device_data)(CloSort *sorter, CCLQueue *cq_exec,
		CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out,
		size_t numel, size_t lws_max, GError **err);
	cl_uint (*get_num_kernels)(CloSort *sorter, GError **err);
	const char *(*get_kernel_name)(CloSort *sorter, cl_uint i, GError **err);
	size_t (*get_localmem_usage)(CloSort *sorter, cl_uint i, size_t lws_max,
		size_t numel, GError **err);
} CloSortImplDef;

extern const CloSortImplDef clo_sort_sbitonic_def;
extern const CloSortImplDef clo_sort_abitonic_def;
extern const CloSortImplDef clo_sort_gselect_def;
extern const CloSortImplDef clo_sort_satradix_def;

/* clo_sort_abstract.c:91 -- `compare` and `get_key` are the reference's
 * macro bodies. NULL selects the defaults "((a) > (b))" and "(x)". The
 * compiled-in kernels implement the defaults; "satradix" ignores
 * `compare` exactly as the reference does (it always sorts ascending by
 * the key's unsigned bit pattern). Other snippets are compiled, as the
 * reference compiles its program per sorter, into a per-sorter CUDA
 * program (NVRTC, for this device) that clo_sort_get_program returns; a
 * snippet that does not compile is reported as CLO_ERROR_LIBRARY. */
CloSort *clo_sort_new(const char *type, const char *options,
	CCLContext *ctx, CloType *elem_type, CloType *key_type,
	const char *compare, const char *get_key, const char *compiler_opts,
	GError **err);

void clo_sort_destroy(CloSort *sorter);

/* clo_sort_abstract.c:252 -- asynchronous; returns the event of the last
 * operation (owned by cq_exec), NULL on error. data_out == NULL sorts
 * data_in in place. */
CCLEvent *clo_sort_with_device_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out,
	size_t numel, size_t lws_max, GError **err);

/* clo_sort_abstract.c:296 -- blocking; data_in and data_out are host
 * arrays of numel elements (may alias). */
cl_bool clo_sort_with_host_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLQueue *cq_comm, void *data_in, void *data_out, size_t numel,
	size_t lws_max, GError **err);

CCLContext *clo_sort_get_context(CloSort *sorter);
CCLProgram *clo_sort_get_program(CloSort *sorter);
CloType clo_sort_get_element_type(CloSort *sorter);
size_t clo_sort_get_element_size(CloSort *sorter);
CloType clo_sort_get_key_type(CloSort *sorter);
size_t clo_sort_get_key_size(CloSort *sorter);
void *clo_sort_get_data(CloSort *sorter);
void clo_sort_set_data(CloSort *sorter, void *data);
cl_uint clo_sort_get_num_kernels(CloSort *sorter, GError **err);
const char *clo_sort_get_kernel_name(CloSort *sorter, cl_uint i,
	GError **err);
size_t clo_sort_get_localmem_usage(CloSort *sorter, cl_uint i,
	size_t lws_max, size_t numel, GError **err);

#ifdef __cplusplus
}
#endif

#endif /* CLO_SORT_ABSTRACT_H */
