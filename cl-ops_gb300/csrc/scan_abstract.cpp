// Scanner objects: registry and the "blelloch" exclusive scan.
// Reference behaviour: src/cl_ops/scan/clo_scan_abstract.c:74-569 and
// src/cl_ops/scan/clo_scan_blelloch.c:32-343.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "clo_internal.h"

using clo::cuda_ok;
using clo::set_error;

struct clo_scan {
	CloScanImplDef impl_def;
	CCLContext *ctx;
	CCLProgram *prg;
	CloType elem_type;
	CloType sum_type;
	void *data;
	// The host-data pipeline's copy streams and events, made on first use
	// and kept for the scanner's lifetime (no driver object is created or
	// destroyed per call).
	cudaStream_t copy_in = nullptr, copy_out = nullptr;
	std::vector<cudaEvent_t> events;
};

namespace {

const char *blelloch_init(CloScan *scanner, const char *options,
	GError **err) {
	(void)scanner;
	// The reference accepts no option for this scan (clo_scan_blelloch.c:43).
	if (options != nullptr && strlen(options) > 0) {
		set_error(err, CLO_ERROR_ARGS, "Invalid options for blelloch scan.");
		return nullptr;
	}
	if (!clo::type_is_integer(scanner->elem_type) ||
		!clo::type_is_integer(scanner->sum_type)) {
		set_error(err, CLO_ERROR_ARGS,
			"blelloch scan: integer element and sum types only ('%s' -> '%s')",
			clo_type_get_name(scanner->elem_type),
			clo_type_get_name(scanner->sum_type));
		return nullptr;
	}
	return "sm_103a:blelloch(single-pass decoupled lookback)";
}

void blelloch_finalize(CloScan *scan) { (void)scan; }

CCLEvent *blelloch_scan(CloScan *sc, CCLQueue *q, CCLQueue *cq_comm,
	CCLBuffer *in, CCLBuffer *out, size_t numel, size_t lws_max,
	GError **err) {
	(void)cq_comm;
	(void)lws_max;
	size_t ib = clo_type_sizeof(sc->elem_type), ob = clo_type_sizeof(sc->sum_type);
	if (!in || !out || in->size < numel * ib || out->size < numel * ob) {
		set_error(err, CLO_ERROR_ARGS,
			"Scan buffers too small for %zu elements", numel);
		return nullptr;
	}
	ccl_event *ev = clo::event_begin(q, "clo_scan_blelloch");
	if (clo::scan_exclusive(in->ptr, out->ptr, numel, sc->elem_type, (int)ob,
			sc->ctx, q->stream, err) != cudaSuccess)
		return nullptr;
	clo::event_end(ev);
	return ev;
}

const char *kBlellochKernels[] = {"scan_lookback"};

cl_uint blelloch_num_kernels(CloScan *, GError **) { return 1; }

const char *blelloch_kernel_name(CloScan *, cl_uint i, GError **err) {
	if (i >= 1) {
		set_error(err, CLO_ERROR_ARGS, "Kernel index %u out of range", i);
		return nullptr;
	}
	return kBlellochKernels[i];
}

size_t blelloch_localmem(CloScan *sc, cl_uint i, size_t lws_max, size_t numel,
	GError **err) {
	(void)i;
	(void)lws_max;
	(void)numel;
	(void)err;
	// 8 warps x 512 items, staged at the wider of the two types, padded.
	size_t w = clo_type_sizeof(sc->elem_type) > clo_type_sizeof(sc->sum_type)
		? clo_type_sizeof(sc->elem_type) : clo_type_sizeof(sc->sum_type);
	return 8 * 512 * w * 5 / 4;
}

}  // namespace

extern "C" {

const CloScanImplDef clo_scan_blelloch_def = {"blelloch", blelloch_init,
	blelloch_finalize, blelloch_scan, blelloch_num_kernels,
	blelloch_kernel_name, blelloch_localmem};

CloScan *clo_scan_new(const char *type, const char *options, CCLContext *ctx,
	CloType elem_type, CloType sum_type, const char *compiler_opts,
	GError **err) {
	if (!type || !ctx || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_scan_new: bad arguments\n");
		return nullptr;
	}
	const CloScanImplDef *def = nullptr;
	if (strcmp(type, clo_scan_blelloch_def.name) == 0) def = &clo_scan_blelloch_def;
	if (!def) {
		set_error(err, CLO_ERROR_IMPL_NOT_FOUND,
			"The requested scan implementation, '%s', was not found.", type);
		return nullptr;
	}
	if (clo_type_sizeof(elem_type) == 0 || clo_type_sizeof(sum_type) == 0) {
		set_error(err, CLO_ERROR_ARGS, "Invalid element or sum type");
		return nullptr;
	}
	CloScan *s = new clo_scan();
	s->impl_def = *def;
	ccl_context_ref(ctx);
	s->ctx = ctx;
	s->elem_type = elem_type;
	s->sum_type = sum_type;
	s->data = nullptr;
	s->prg = nullptr;
	GError *e2 = nullptr;
	const char *src = def->init(s, options, &e2);
	if (!src) {
		clo::propagate_error(err, e2);
		clo_scan_destroy(s);
		return nullptr;
	}
	s->prg = new ccl_program();
	s->prg->src = src;
	// Same option string the reference builds (clo_scan_abstract.c:122-125).
	s->prg->opts = std::string(" -DCLO_SCAN_ELEM_TYPE=") +
		clo_type_get_name(elem_type) + " -DCLO_SCAN_SUM_TYPE=" +
		clo_type_get_name(sum_type) + (compiler_opts ? compiler_opts : "");
	clo::wrapper_created();
	return s;
}

void clo_scan_destroy(CloScan *scan) {
	if (!scan) return;
	if (scan->copy_in || scan->copy_out || !scan->events.empty()) {
		int prev_dev = -1;
		if (cudaGetDevice(&prev_dev) != cudaSuccess) prev_dev = -1;
		cudaSetDevice(scan->ctx->ordinal);
		for (cudaStream_t st : {scan->copy_in, scan->copy_out}) {
			if (st) {
				cudaStreamSynchronize(st);
				cudaStreamDestroy(st);
			}
		}
		for (cudaEvent_t ev : scan->events) cudaEventDestroy(ev);
		if (prev_dev >= 0) cudaSetDevice(prev_dev);
	}
	scan->impl_def.finalize(scan);
	if (scan->ctx) ccl_context_unref(scan->ctx);
	if (scan->prg) {
		delete scan->prg;
		clo::wrapper_destroyed();
	}
	delete scan;
}

CCLEvent *clo_scan_with_device_data(CloScan *scanner, CCLQueue *cq_exec,
	CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out, size_t numel,
	size_t lws_max, GError **err) {
	if (!scanner || !cq_exec || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_scan_with_device_data: bad arguments\n");
		return nullptr;
	}
	cudaSetDevice(scanner->ctx->ordinal);
	return scanner->impl_def.scan_with_device_data(scanner, cq_exec, cq_comm,
		data_in, data_out, numel, lws_max, err);
}

}  // extern "C"

namespace {

// Host-data scans of large arrays in chunks on three streams: chunk c is
// copied in, scanned continuing from the running sum of the chunks before
// it (a device-side carry), and copied out, while its neighbours are in
// flight the other ways; the two copy directions overlap each other and
// the scans.
constexpr size_t kScanChunk = (size_t)1 << 24;

bool scan_host_pipelined(CloScan *sc, CCLQueue *q, const void *h_in, void *h_out,
	size_t n, GError **err) {
	CCLContext *ctx = sc->ctx;
	const size_t ib = clo_type_sizeof(sc->elem_type), ob = clo_type_sizeof(sc->sum_type);
	const size_t nc = (n + kScanChunk - 1) / kScanChunk;
	cudaStream_t cs = q->stream;
	bool ok = (sc->copy_in || cuda_ok(cudaStreamCreateWithFlags(&sc->copy_in,
		cudaStreamNonBlocking), err, "stream")) &&
		(sc->copy_out || cuda_ok(cudaStreamCreateWithFlags(&sc->copy_out,
		cudaStreamNonBlocking), err, "stream"));
	cudaStream_t si = sc->copy_in, so = sc->copy_out;
	const size_t off_out = (n * ib + 255) / 256 * 256;
	const size_t off_carry = off_out + (n * ob + 255) / 256 * 256;
	char *dev = ok ? (char *)clo::tmp_alloc(ctx, off_carry + (nc + 1) * 8, cs, err) : nullptr;
	ok = ok && dev != nullptr;
	// The call's events, in order, from the scanner's set (grown as needed).
	size_t next_event = 0;
	auto event = [&]() -> cudaEvent_t {
		if (next_event == sc->events.size()) {
			cudaEvent_t e = nullptr;
			if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
			sc->events.push_back(e);
		}
		return sc->events[next_event++];
	};
	cudaEvent_t ready = ok ? event() : nullptr;
	ok = ok && ready && cuda_ok(cudaMemsetAsync(dev + off_carry, 0, (nc + 1) * 8, cs), err,
		"carry") && cuda_ok(cudaEventRecord(ready, cs), err, "event") &&
		cuda_ok(cudaStreamWaitEvent(si, ready, 0), err, "wait");
	for (size_t c = 0; c < nc && ok; ++c) {
		const size_t off = c * kScanChunk;
		const size_t len = n - off < kScanChunk ? n - off : kScanChunk;
		cudaEvent_t ein = event(), esc = event();
		ok = ein && esc &&
			cuda_ok(cudaMemcpyAsync(dev + off * ib, (const char *)h_in + off * ib, len * ib,
				cudaMemcpyHostToDevice, si), err, "copy in") &&
			cuda_ok(cudaEventRecord(ein, si), err, "event") &&
			cuda_ok(cudaStreamWaitEvent(cs, ein, 0), err, "wait");
		ok = ok && clo::scan_exclusive_carry(dev + off * ib, dev + off_out + off * ob, len,
			sc->elem_type, (int)ob, dev + off_carry + c * 8, dev + off_carry + (c + 1) * 8,
			ctx, cs, err) == cudaSuccess;
		ok = ok && cuda_ok(cudaEventRecord(esc, cs), err, "event") &&
			cuda_ok(cudaStreamWaitEvent(so, esc, 0), err, "wait") &&
			cuda_ok(cudaMemcpyAsync((char *)h_out + off * ob, dev + off_out + off * ob,
				len * ob, cudaMemcpyDeviceToHost, so), err, "copy out");
	}
	if (si) cudaStreamSynchronize(si);
	if (so) cudaStreamSynchronize(so);
	cudaStreamSynchronize(cs);
	ok = ok && clo::check_device_status(ctx, err);
	if (dev) clo::tmp_free(dev, cs);
	cudaStreamSynchronize(cs);
	return ok;
}

}  // namespace

extern "C" {

cl_bool clo_scan_with_host_data(CloScan *scanner, CCLQueue *cq_exec,
	CCLQueue *cq_comm, void *data_in, void *data_out, size_t numel,
	size_t lws_max, GError **err) {
	if (!scanner || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_scan_with_host_data: bad arguments\n");
		return CL_FALSE;
	}
	CCLContext *ctx = scanner->ctx;
	cudaSetDevice(ctx->ordinal);
	if (numel >= ((size_t)1 << 22) && strcmp(scanner->impl_def.name, "blelloch") == 0) {
		CCLQueue *q = cq_exec;
		GError *e3 = nullptr;
		if (!q) q = ccl_queue_new(ctx, &ctx->device, 0, &e3);
		bool ok = q && scan_host_pipelined(scanner, q, data_in, data_out, numel, &e3);
		if (q && q != cq_exec) ccl_queue_destroy(q);
		clo::propagate_error(err, e3);
		return ok ? CL_TRUE : CL_FALSE;
	}
	GError *e2 = nullptr;
	CCLQueue *own = nullptr;
	if (cq_exec == nullptr) {
		own = ccl_queue_new(ctx, &ctx->device, 0, &e2);
		if (!own) {
			clo::propagate_error(err, e2);
			return CL_FALSE;
		}
		cq_exec = own;
	}
	if (cq_comm == nullptr) cq_comm = cq_exec;
	size_t ib = numel * clo_type_sizeof(scanner->elem_type);
	size_t ob = numel * clo_type_sizeof(scanner->sum_type);
	cl_bool status = CL_FALSE;
	CCLBuffer *din = nullptr, *dout = nullptr;
	CCLEvent *evt = nullptr;
	CCLEventWaitList ewl = nullptr;
	void *pin = clo::tmp_alloc(ctx, ib, cq_comm->stream, &e2);
	void *pout = pin ? clo::tmp_alloc(ctx, ob, cq_comm->stream, &e2) : nullptr;
	if (!pin || !pout) goto done;
	din = ccl_buffer_new_wrap(ctx, pin, ib, &e2);
	dout = ccl_buffer_new_wrap(ctx, pout, ob, &e2);
	evt = ccl_buffer_enqueue_write(din, cq_comm, CL_FALSE, 0, ib, data_in,
		nullptr, &e2);
	if (!evt) goto done;
	if (cq_comm != cq_exec) ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!clo::wait_ewl(cq_exec, &ewl, &e2)) goto done;
	evt = scanner->impl_def.scan_with_device_data(scanner, cq_exec, cq_comm,
		din, dout, numel, lws_max, &e2);
	if (!evt) goto done;
	if (cq_comm != cq_exec) ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	evt = ccl_buffer_enqueue_read(dout, cq_comm, CL_FALSE, 0, ob, data_out,
		&ewl, &e2);
	if (!evt) goto done;
	ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!ccl_event_wait(&ewl, &e2)) goto done;
	status = CL_TRUE;
done:
	ccl_event_wait_list_clear(&ewl);
	if (din) ccl_buffer_destroy(din);
	if (dout) ccl_buffer_destroy(dout);
	clo::tmp_free(pin, cq_comm->stream);
	clo::tmp_free(pout, cq_comm->stream);
	if (!status) cudaStreamSynchronize(cq_comm->stream);
	if (own) ccl_queue_destroy(own);
	clo::propagate_error(err, e2);
	return status;
}

CCLContext *clo_scan_get_context(CloScan *s) { return s ? s->ctx : nullptr; }
CCLProgram *clo_scan_get_program(CloScan *s) { return s ? s->prg : nullptr; }
CloType clo_scan_get_elem_type(CloScan *s) {
	return s ? s->elem_type : (CloType)-1;
}
size_t clo_scan_get_element_size(CloScan *s) {
	return s ? clo_type_sizeof(s->elem_type) : 0;
}
CloType clo_scan_get_sum_type(CloScan *s) {
	return s ? s->sum_type : (CloType)-1;
}
size_t clo_scan_get_sum_size(CloScan *s) {
	return s ? clo_type_sizeof(s->sum_type) : 0;
}
void *clo_scan_get_data(CloScan *s) { return s ? s->data : nullptr; }
void clo_scan_set_data(CloScan *s, void *data) {
	if (s) s->data = data;
}
cl_uint clo_scan_get_num_kernels(CloScan *s, GError **err) {
	return s ? s->impl_def.get_num_kernels(s, err) : 0;
}
const char *clo_scan_get_kernel_name(CloScan *s, cl_uint i, GError **err) {
	return s ? s->impl_def.get_kernel_name(s, i, err) : nullptr;
}
size_t clo_scan_get_localmem_usage(CloScan *s, cl_uint i, size_t lws_max,
	size_t numel, GError **err) {
	return s ? s->impl_def.get_localmem_usage(s, i, lws_max, numel, err) : 0;
}

}  // extern "C"

// ------------------------------------------------------- segmented scan
extern "C" {

CCLEvent *clo_scan_segmented_with_device_data(CloScan *scanner, CCLQueue *q,
	CCLBuffer *data_in, CCLBuffer *data_out, CCLBuffer *offsets,
	size_t num_segments, GError **err) {
	if (!scanner || !q || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_scan_segmented_with_device_data: bad arguments\n");
		return nullptr;
	}
	if (strcmp(scanner->impl_def.name, "blelloch") != 0) {
		set_error(err, CLO_ERROR_ARGS, "Segmented scan: unknown scanner '%s'",
			scanner->impl_def.name);
		return nullptr;
	}
	cudaSetDevice(scanner->ctx->ordinal);
	const size_t ib = clo_type_sizeof(scanner->elem_type);
	const size_t ob = clo_type_sizeof(scanner->sum_type);
	if (!data_in || !data_out ||
		(num_segments > 0 && (!offsets || offsets->size < (num_segments + 1) * 8))) {
		set_error(err, CLO_ERROR_ARGS,
			"Segmented scan needs input and output buffers and %zu offsets",
			num_segments + 1);
		return nullptr;
	}
	const size_t n_in = data_in->size / ib, n_out = data_out->size / ob;
	ccl_event *ev = clo::event_begin(q, "clo_scan_blelloch_segmented");
	if (clo::seg_scan(data_in->ptr, data_out->ptr, n_in < n_out ? n_in : n_out,
			num_segments ? (const uint64_t *)offsets->ptr : nullptr, num_segments,
			scanner->elem_type, (int)ob, scanner->ctx, q->stream, err) != cudaSuccess)
		return nullptr;
	clo::event_end(ev);
	return ev;
}

cl_bool clo_scan_segmented_with_host_data(CloScan *scanner, CCLQueue *q,
	const void *data_in, void *data_out, size_t numel, const cl_ulong *offsets,
	size_t num_segments, GError **err) {
	if (!scanner || (err && *err)) return CL_FALSE;
	CCLContext *ctx = scanner->ctx;
	cudaSetDevice(ctx->ordinal);
	if (!clo::check_offsets((const uint64_t *)offsets, num_segments, numel, err))
		return CL_FALSE;
	GError *e2 = nullptr;
	CCLQueue *own = nullptr;
	if (!q) {
		own = ccl_queue_new(ctx, &ctx->device, 0, &e2);
		if (!own) {
			clo::propagate_error(err, e2);
			return CL_FALSE;
		}
		q = own;
	}
	const size_t ib = numel * clo_type_sizeof(scanner->elem_type);
	const size_t ob = numel * clo_type_sizeof(scanner->sum_type);
	const size_t obytes = (num_segments + 1) * 8;
	cl_bool status = CL_FALSE;
	CCLBuffer *din = nullptr, *dout = nullptr, *doff = nullptr;
	CCLEventWaitList ewl = nullptr;
	CCLEvent *evt = nullptr;
	void *pin = clo::tmp_alloc(ctx, ib, q->stream, &e2);
	void *pout = pin ? clo::tmp_alloc(ctx, ob, q->stream, &e2) : nullptr;
	void *po = pout ? clo::tmp_alloc(ctx, obytes, q->stream, &e2) : nullptr;
	if (!pin || !pout || !po) goto done;
	din = ccl_buffer_new_wrap(ctx, pin, ib, &e2);
	dout = ccl_buffer_new_wrap(ctx, pout, ob, &e2);
	doff = ccl_buffer_new_wrap(ctx, po, obytes, &e2);
	if (!ccl_buffer_enqueue_write(din, q, CL_FALSE, 0, ib, data_in, nullptr, &e2))
		goto done;
	// Elements outside the segments keep what data_out held.
	if (!ccl_buffer_enqueue_write(dout, q, CL_FALSE, 0, ob, data_out, nullptr, &e2))
		goto done;
	if (num_segments > 0 &&
		!ccl_buffer_enqueue_write(doff, q, CL_FALSE, 0, obytes, offsets, nullptr, &e2))
		goto done;
	if (!clo_scan_segmented_with_device_data(scanner, q, din, dout, doff, num_segments,
			&e2))
		goto done;
	evt = ccl_buffer_enqueue_read(dout, q, CL_FALSE, 0, ob, data_out, nullptr, &e2);
	if (!evt) goto done;
	ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!ccl_event_wait(&ewl, &e2)) goto done;
	status = CL_TRUE;
done:
	ccl_event_wait_list_clear(&ewl);
	if (din) ccl_buffer_destroy(din);
	if (dout) ccl_buffer_destroy(dout);
	if (doff) ccl_buffer_destroy(doff);
	clo::tmp_free(pin, q->stream);
	clo::tmp_free(pout, q->stream);
	clo::tmp_free(po, q->stream);
	if (!status) cudaStreamSynchronize(q->stream);
	if (own) ccl_queue_destroy(own);
	clo::propagate_error(err, e2);
	return status;
}

}  // extern "C"
