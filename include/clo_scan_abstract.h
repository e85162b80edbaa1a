/*
 * cl_ops on GB300 -- scanner object API and implementation registry.
 *
 * Same plugin interface and entry points as the reference's
 * src/cl_ops/scan/clo_scan_abstract.in.h:41-162. The only registered
 * implementation is "blelloch" (clo_scan_abstract.c:86-89), an exclusive
 * prefix sum: out[0] = 0, out[i] = sum_{j<i} (SUM_TYPE) in[j], computed
 * here by a single-pass decoupled-lookback kernel.
 */
#ifndef CLO_SCAN_ABSTRACT_H
#define CLO_SCAN_ABSTRACT_H

#include "clo_common.h"
#include "ccl_shim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* clo_scan_abstract.in.h:41-103 */
typedef struct clo_scan_impl_def {
	const char *name;
	const char *(*init)(CloScan *scanner, const char *options, GError **err);
	void (*finalize)(CloScan *scan);
	CCLEvent *(*scan_with_device_data)(CloScan *scanner, CCLQueue *cq_exec,
		CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out,
		size_t numel, size_t lws_max, GError **err);
	cl_uint (*get_num_kernels)(CloScan *scanner, GError **err);
	const char *(*get_kernel_name)(CloScan *scanner, cl_uint i, GError **err);
	size_t (*get_localmem_usage)(CloScan *scanner, cl_uint i, size_t lws_max,
		size_t numel, GError **err);
} CloScanImplDef;

extern const CloScanImplDef clo_scan_blelloch_def;

/* clo_scan_abstract.c:74 -- integer element and sum types of any width
 * and signedness; the element is converted to the sum type with C
 * conversion rules and summed modulo 2^(8*sizeof(sum)). */
CloScan *clo_scan_new(const char *type, const char *options,
	CCLContext *ctx, CloType elem_type, CloType sum_type,
	const char *compiler_opts, GError **err);

void clo_scan_destroy(CloScan *scan);

/* clo_scan_abstract.c:216 -- asynchronous, returns the last event. */
CCLEvent *clo_scan_with_device_data(CloScan *scanner, CCLQueue *cq_exec,
	CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out,
	size_t numel, size_t lws_max, GError **err);

/* clo_scan_abstract.c:255 -- blocking, host arrays. */
cl_bool clo_scan_with_host_data(CloScan *scanner, CCLQueue *cq_exec,
	CCLQueue *cq_comm, void *data_in, void *data_out, size_t numel,
	size_t lws_max, GError **err);

CCLContext *clo_scan_get_context(CloScan *scanner);
CCLProgram *clo_scan_get_program(CloScan *scanner);
CloType clo_scan_get_elem_type(CloScan *scanner);
size_t clo_scan_get_element_size(CloScan *scanner);
CloType clo_scan_get_sum_type(CloScan *scanner);
size_t clo_scan_get_sum_size(CloScan *scanner);
void *clo_scan_get_data(CloScan *scanner);
void clo_scan_set_data(CloScan *scanner, void *data);
cl_uint clo_scan_get_num_kernels(CloScan *scanner, GError **err);
const char *clo_scan_get_kernel_name(CloScan *scanner, cl_uint i,
	GError **err);
size_t clo_scan_get_localmem_usage(CloScan *scanner, cl_uint i,
	size_t lws_max, size_t numel, GError **err);

#ifdef __cplusplus
}
#endif

#endif /* CLO_SCAN_ABSTRACT_H */
