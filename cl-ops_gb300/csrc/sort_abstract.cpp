// Sorter objects: registry, option parsing, device-data and host-data
// entry points for "sbitonic", "abitonic", "gselect" and "satradix".
// Reference behaviour: src/cl_ops/sort/clo_sort_abstract.c:91-631 and the
// per-implementation drivers clo_sort_{sbitonic,abitonic,gselect,
// satradix}.c.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "clo_internal.h"
#include "jit.h"

using clo::cuda_ok;
using clo::set_error;

struct clo_sort {
	CloSortImplDef impl_def;
	CCLContext *ctx;
	CCLProgram *prg;
	CloType elem_type;
	CloType key_type;
	void *data;
	// Kernels built by NVRTC for custom compare/get_key macros (or a key
	// type other than the element type); null for the compiled-in path.
	std::shared_ptr<clo::JitSort> jit;
	// The host-data pipeline's copy-out stream and per-group events, made
	// on first use and kept for the sorter's lifetime (no driver object is
	// created or destroyed per call).
	cudaStream_t copy_stream = nullptr;
	std::vector<cudaEvent_t> group_events;
	// Its page-locked scratch: the partition's 256 bucket counts, then the
	// groups' relative offsets (device <-> host copies without staging).
	uint64_t *host_scratch = nullptr;
};

namespace {

// Removes blanks so that "((a) > (b))" and "((a)>(b))" compare equal.
std::string squeeze(const char *s) {
	std::string r;
	for (; s && *s; ++s)
		if (*s != ' ' && *s != '\t' && *s != '\n' && *s != '\r') r += *s;
	return r;
}

bool compare_is_default(const char *c) {
	if (c == nullptr) return true;
	std::string s = squeeze(c);
	return s == "((a)>(b))" || s == "(a>b)" || s == "a>b" || s == "(a)>(b)";
}

bool get_key_is_default(const char *k) {
	if (k == nullptr) return true;
	std::string s = squeeze(k);
	return s == "(x)" || s == "x";
}

// Splits "k1=v1,k2=v2" like the reference's g_strsplit_set(",") then
// g_strsplit_set("=", 2); empty tokens are skipped. Calls f(key, value,
// token) and stops at the first false.
template <typename F>
bool for_each_option(const char *options, F f) {
	if (!options) return true;
	std::string all(options);
	size_t pos = 0;
	while (pos <= all.size()) {
		size_t comma = all.find(',', pos);
		if (comma == std::string::npos) comma = all.size();
		std::string tok = all.substr(pos, comma - pos);
		pos = comma + 1;
		if (tok.empty()) continue;
		size_t eq = tok.find('=');
		std::string key = eq == std::string::npos ? tok : tok.substr(0, eq);
		std::string val = eq == std::string::npos ? std::string() : tok.substr(eq + 1);
		if (!f(key, val, tok, eq != std::string::npos)) return false;
	}
	return true;
}

bool check_numel(CloSort *s, CCLBuffer *b, size_t numel, GError **err) {
	size_t need = numel * clo_type_sizeof(s->elem_type);
	if (b == nullptr) {
		set_error(err, CLO_ERROR_ARGS, "NULL data buffer");
		return false;
	}
	if (need > b->size) {
		set_error(err, CLO_ERROR_ARGS,
			"Buffer of %zu bytes cannot hold %zu elements of type %s",
			b->size, numel, clo_type_get_name(s->elem_type));
		return false;
	}
	return true;
}

// Copies data_in to data_out (when given) and returns the buffer to sort.
CCLBuffer *target_buffer(CloSort *s, CCLQueue *q, CCLBuffer *in,
	CCLBuffer *out, size_t numel, GError **err) {
	if (out == nullptr || out == in) return in;
	if (!check_numel(s, out, numel, err)) return nullptr;
	size_t bytes = numel * clo_type_sizeof(s->elem_type);
	if (bytes && !cuda_ok(cudaMemcpyAsync(out->ptr, in->ptr, bytes,
			cudaMemcpyDeviceToDevice, q->stream), err, "sort copy"))
		return nullptr;
	return out;
}

// ====================================================== built kernels
// Sorts `numel` elements of `src` into `dst` (which may be `src`) with the
// sorter's NVRTC kernels:
// - satradix: keys from get_key with their indices, the compiled-in stable
//   radix sort of (key, index) by the key's low 8 * min(element, key)
//   bytes bits (the passes of clo_sort_satradix.c:167-169 over the key of
//   clo_sort_satradix.cl:58,140), then a gather;
// - bitonic: the reference network (clo_sort_sbitonic.cl:38-69), one step
//   per launch, over the next power of two with padding flags;
// - gselect: rank by counting (clo_sort_gselect.cl:38-57), out of place.
enum JitAlgo { JIT_RADIX, JIT_BITONIC, JIT_GSELECT };

bool jit_sort(CloSort *s, CCLQueue *q, void *src, void *dst, size_t numel,
	JitAlgo algo, GError **err) {
	clo::JitSort &j = *s->jit;
	cudaStream_t st = q->stream;
	const int sms = s->ctx->sm_count;
	const size_t eb = clo_type_sizeof(s->elem_type), kb = clo_type_sizeof(s->key_type);
	unsigned long long n = numel;
	if (numel == 0) return true;
	if (algo == JIT_GSELECT || numel == 1) {
		if (numel == 1 || src == dst) {
			void *tmp = clo::tmp_alloc(s->ctx, numel * eb, st, err);
			if (!tmp) return false;
			bool ok = true;
			if (numel == 1) {
				ok = cuda_ok(cudaMemcpyAsync(tmp, src, eb, cudaMemcpyDeviceToDevice, st),
					err, "copy");
			} else {
				void *args[] = {&src, &tmp, &n};
				ok = cuda_ok(clo::jit_launch(j.gselect, numel, args, st, sms), err, "gselect");
			}
			ok = ok && cuda_ok(cudaMemcpyAsync(dst, tmp, numel * eb,
				cudaMemcpyDeviceToDevice, st), err, "copy back");
			clo::tmp_free(tmp, st);
			return ok;
		}
		void *args[] = {&src, &dst, &n};
		return cuda_ok(clo::jit_launch(j.gselect, numel, args, st, sms), err, "gselect");
	}
	if (algo == JIT_RADIX) {
		if (numel >= (1ull << 32)) {
			set_error(err, CLO_ERROR_ARGS, "Custom get_key sorts take fewer than 2^32 elements");
			return false;
		}
		const size_t off_idx = (numel * kb + 255) / 256 * 256;
		const size_t off_out = off_idx + (numel * 4 + 255) / 256 * 256;
		char *tmp = (char *)clo::tmp_alloc(s->ctx, off_out + numel * eb, st, err);
		if (!tmp) return false;
		void *keys = tmp, *idx = tmp + off_idx, *sorted = tmp + off_out;
		void *a1[] = {&src, &keys, &idx, &n};
		bool ok = cuda_ok(clo::jit_launch(j.keys, numel, a1, st, sms), err, "get_key");
		const int bits = (int)(8 * (eb < kb ? eb : kb));
		ok = ok && clo::radix_sort(keys, idx, numel, (int)kb, 4, bits, s->ctx, st,
			!clo::stream_capturing(st), err) == cudaSuccess;
		void *a2[] = {&src, &idx, &sorted, &n};
		ok = ok && cuda_ok(clo::jit_launch(j.gather, numel, a2, st, sms), err, "gather");
		ok = ok && cuda_ok(cudaMemcpyAsync(dst, sorted, numel * eb,
			cudaMemcpyDeviceToDevice, st), err, "copy back");
		clo::tmp_free(tmp, st);
		return ok;
	}
	size_t N = 1;
	while (N < numel) N <<= 1;
	const size_t off_pad = (N * eb + 255) / 256 * 256;
	char *tmp = (char *)clo::tmp_alloc(s->ctx, off_pad + N, st, err);
	if (!tmp) return false;
	void *data = tmp;
	void *pad = tmp + off_pad;
	bool ok = cuda_ok(cudaMemcpyAsync(data, src, numel * eb, cudaMemcpyDeviceToDevice, st),
		err, "copy");
	ok = ok && cuda_ok(cudaMemsetAsync(pad, 0, numel, st), err, "pad");
	if (N > numel) ok = ok && cuda_ok(cudaMemsetAsync((char *)pad + numel, 1, N - numel, st),
		err, "pad");
	unsigned long long half = N / 2;
	unsigned stages = 0;
	while ((1ull << stages) < N) ++stages;
	for (unsigned stage = 1; stage <= stages && ok; ++stage)
		for (unsigned step = stage; step > 0 && ok; --step) {
			void *args[] = {&data, &pad, &stage, &step, &half};
			ok = cuda_ok(clo::jit_launch(j.bitonic_step, half, args, st, sms), err,
				"bitonic step");
		}
	ok = ok && cuda_ok(cudaMemcpyAsync(dst, data, numel * eb, cudaMemcpyDeviceToDevice, st),
		err, "copy back");
	clo::tmp_free(tmp, st);
	return ok;
}

// ============================================================ satradix
struct SatradixData {
	unsigned radix;
	std::string scan_type;
	std::string scan_opts;
	CloScan *scanner;
	// Shape of segmented sorts (segvariant= option, or the autotuner's
	// choice).
	int seg_variant;
};

const char *kSatradixKernels[] = {"satradix_upsweep", "satradix_onesweep"};

CloScan *satradix_get_scanner(CloSort *s, GError **err) {
	SatradixData *d = (SatradixData *)s->data;
	if (d->scanner == nullptr) {
		d->scanner = clo_scan_new(d->scan_type.c_str(), d->scan_opts.c_str(),
			s->ctx, CLO_UINT, CLO_UINT, s->prg ? s->prg->opts.c_str() : nullptr,
			err);
	}
	return d->scanner;
}

// Number of low key bits the reference's satradix passes actually order:
// passes run over the *element* width (clo_sort_satradix.c:167-169) but
// shift the *key*, whose shift count OpenCL masks to the key width, so
// the sorted bits are the low min(key, element) bits of the key.
int satradix_sort_bits(CloSort *s) {
	size_t eb = clo_type_sizeof(s->elem_type), kb = clo_type_sizeof(s->key_type);
	return (int)(8 * (eb < kb ? eb : kb));
}

const char *satradix_init(CloSort *s, const char *options, GError **err) {
	SatradixData *d = new SatradixData();
	d->radix = 16;
	d->scanner = nullptr;
	d->seg_variant = 0;
	s->data = d;
	bool ok = for_each_option(options, [&](const std::string &k,
		const std::string &v, const std::string &tok, bool has_eq) {
		if (!has_eq) {
			set_error(err, CLO_ERROR_ARGS,
				"Invalid option '%s' for satradix sort.", tok.c_str());
			return false;
		}
		if (k == "radix") {
			d->radix = (unsigned)atoi(v.c_str());
			if (clo_ones32(d->radix) != 1) {
				set_error(err, CLO_ERROR_ARGS, "Radix must be a power of 2.");
				return false;
			}
		} else if (k == "segvariant") {
			d->seg_variant = atoi(v.c_str());
			if (d->seg_variant < 0 || d->seg_variant >= clo::seg_sort_num_variants()) {
				set_error(err, CLO_ERROR_ARGS, "segvariant must be in [0, %d).",
					clo::seg_sort_num_variants());
				return false;
			}
		} else if (k.size() >= 4 && strncasecmp(k.c_str(), "scan", 4) == 0) {
			if (k.size() == 4) d->scan_type = v;
			else d->scan_opts += tok.substr(4) + ",";
		} else {
			set_error(err, CLO_ERROR_ARGS,
				"Invalid option key '%s' for satradix sort.", k.c_str());
			return false;
		}
		return true;
	});
	if (!ok) return nullptr;
	if (d->scan_type.empty()) d->scan_type = "blelloch";
	if (!clo::type_is_integer(s->elem_type) ||
		!clo::type_is_integer(s->key_type)) {
		set_error(err, CLO_ERROR_ARGS,
			"satradix sorts integer keys only (element '%s', key '%s')",
			clo_type_get_name(s->elem_type), clo_type_get_name(s->key_type));
		return nullptr;
	}
	return "sm_103a:satradix(onesweep, 8-bit digits)";
}

void satradix_finalize(CloSort *s) {
	SatradixData *d = (SatradixData *)s->data;
	if (!d) return;
	if (d->scanner) clo_scan_destroy(d->scanner);
	delete d;
	s->data = nullptr;
}

CCLEvent *satradix_sort(CloSort *s, CCLQueue *cq_exec, CCLQueue *cq_comm,
	CCLBuffer *in, CCLBuffer *out, size_t numel, size_t lws_max,
	GError **err) {
	(void)cq_comm;
	(void)lws_max;
	if (!check_numel(s, in, numel, err)) return nullptr;
	GError *e2 = nullptr;
	// The reference creates its scanner on the first sort; doing the same
	// validates the scan= options at the same point.
	if (!satradix_get_scanner(s, &e2)) {
		clo::propagate_error(err, e2);
		return nullptr;
	}
	ccl_event *ev = clo::event_begin(cq_exec, "satradix");
	CCLBuffer *tgt = target_buffer(s, cq_exec, in, out, numel, err);
	if (!tgt) return nullptr;
	if (s->jit) {
		if (!jit_sort(s, cq_exec, tgt->ptr, tgt->ptr, numel, JIT_RADIX, err)) return nullptr;
		clo::event_end(ev);
		return ev;
	}
	int kb = (int)clo_type_sizeof(s->elem_type);
	bool skip = !clo::stream_capturing(cq_exec->stream);
	if (clo::radix_sort(tgt->ptr, nullptr, numel, kb, 0, satradix_sort_bits(s),
			s->ctx, cq_exec->stream, skip, err) != cudaSuccess)
		return nullptr;
	clo::event_end(ev);
	return ev;
}

cl_uint satradix_num_kernels(CloSort *s, GError **err) {
	CloScan *sc = satradix_get_scanner(s, err);
	if (!sc) return 0;
	return 2 + clo_scan_get_num_kernels(sc, err);
}

const char *satradix_kernel_name(CloSort *s, cl_uint i, GError **err) {
	if (i < 2) return kSatradixKernels[i];
	CloScan *sc = satradix_get_scanner(s, err);
	if (!sc) return nullptr;
	return clo_scan_get_kernel_name(sc, i - 2, err);
}

// Shared-memory footprint of the onesweep kernels (fixed tile shapes).
size_t radix_localmem(size_t elem, cl_uint i) {
	if (i == 0) return 4 * 256 * sizeof(cl_uint);
	size_t tile = elem <= 4 ? 8192 : 4096;
	return tile * elem + 16 * 256 * sizeof(cl_uint) + 4 * 256 * sizeof(cl_uint);
}

size_t satradix_localmem(CloSort *s, cl_uint i, size_t lws_max, size_t numel,
	GError **err) {
	if (i < 2) return radix_localmem(clo_sort_get_element_size(s), i);
	CloScan *sc = satradix_get_scanner(s, err);
	if (!sc) return 0;
	return clo_scan_get_localmem_usage(sc, i - 2, lws_max, numel, err);
}

// ============================================================ bitonic
struct AbitonicData {
	unsigned max_ps;
	unsigned min_ps;
	unsigned max_sfs;
};

const char *sbitonic_init(CloSort *s, const char *options, GError **err) {
	(void)options;
	s->data = nullptr;
	return "sm_103a:sbitonic(one network step per launch)";
}

const char *abitonic_init(CloSort *s, const char *options, GError **err) {
	AbitonicData *d = new AbitonicData{4, 1, 0xffffffffu};
	s->data = d;
	bool ok = for_each_option(options, [&](const std::string &k,
		const std::string &v, const std::string &tok, bool has_eq) {
		if (!has_eq) {
			set_error(err, CLO_ERROR_ARGS,
				"Invalid option '%s' for abitonic sort.", tok.c_str());
			return false;
		}
		unsigned value = (unsigned)atoi(v.c_str());
		if (k == "minps") {
			if (value > 4 || value < 1) {
				set_error(err, CLO_ERROR_ARGS,
					"Option 'minps' must be between 1 and 4.");
				return false;
			}
			d->min_ps = value;
		} else if (k == "maxps") {
			if (value > 4 || value < 1) {
				set_error(err, CLO_ERROR_ARGS,
					"Option 'maxps' must be between 1 and 4.");
				return false;
			}
			d->max_ps = value;
		} else if (k == "maxsfs") {
			d->max_sfs = value;
		} else {
			set_error(err, CLO_ERROR_ARGS,
				"Invalid option key '%s' for abitonic sort.", k.c_str());
			return false;
		}
		return true;
	});
	if (!ok) return nullptr;
	if (options && d->max_ps < d->min_ps) {
		set_error(err, CLO_ERROR_ARGS,
			"'minps' (%u) must be less or equal than 'maxps' (%u).",
			d->min_ps, d->max_ps);
		return nullptr;
	}
	return "sm_103a:abitonic(shared-memory tiles + register passes)";
}

void bitonic_finalize(CloSort *s) {
	delete (AbitonicData *)s->data;
	s->data = nullptr;
}

}  // namespace

namespace clo {
// Implemented in bitonic.cu: one global compare-exchange step per launch,
// and the grouped form with explicit grouping limits.
cudaError_t bitonic_sort_simple(void *data, size_t n, CloType type,
	CCLContext *ctx, cudaStream_t s, GError **err);
cudaError_t bitonic_sort_tuned(void *data, size_t n, CloType type, int max_ps,
	int max_sfs, CCLContext *ctx, cudaStream_t s, GError **err);
}

namespace {

CCLEvent *bitonic_sort_common(CloSort *s, CCLQueue *q, CCLBuffer *in,
	CCLBuffer *out, size_t numel, bool simple, GError **err) {
	if (!check_numel(s, in, numel, err)) return nullptr;
	ccl_event *ev = clo::event_begin(q, simple ? "sbitonic" : "abitonic");
	CCLBuffer *tgt = target_buffer(s, q, in, out, numel, err);
	if (!tgt) return nullptr;
	// abitonic's maxps bounds the steps grouped per global pass and maxsfs
	// the largest step finished in shared memory (clo_sort_abitonic.c:
	// 155-157); neither changes the result.
	if (s->jit) {
		if (!jit_sort(s, q, tgt->ptr, tgt->ptr, numel, JIT_BITONIC, err)) return nullptr;
		clo::event_end(ev);
		return ev;
	}
	AbitonicData *d = (AbitonicData *)s->data;
	cudaError_t e = simple
		? clo::bitonic_sort_simple(tgt->ptr, numel, s->elem_type, s->ctx,
			q->stream, err)
		: clo::bitonic_sort_tuned(tgt->ptr, numel, s->elem_type,
			d ? (int)d->max_ps : 4,
			d && d->max_sfs < 64 ? (int)d->max_sfs : 0, s->ctx, q->stream, err);
	if (e != cudaSuccess) return nullptr;
	clo::event_end(ev);
	return ev;
}

CCLEvent *sbitonic_sort(CloSort *s, CCLQueue *cq_exec, CCLQueue *cq_comm,
	CCLBuffer *in, CCLBuffer *out, size_t numel, size_t lws_max,
	GError **err) {
	(void)cq_comm;
	(void)lws_max;
	return bitonic_sort_common(s, cq_exec, in, out, numel, true, err);
}

CCLEvent *abitonic_sort(CloSort *s, CCLQueue *cq_exec, CCLQueue *cq_comm,
	CCLBuffer *in, CCLBuffer *out, size_t numel, size_t lws_max,
	GError **err) {
	(void)cq_comm;
	(void)lws_max;
	return bitonic_sort_common(s, cq_exec, in, out, numel, false, err);
}

const char *kSbitonicKernels[] = {"sbitonic_step"};
const char *kAbitonicKernels[] = {"abitonic_tile_sort", "abitonic_global_steps",
	"abitonic_tile_finish"};

cl_uint sbitonic_num_kernels(CloSort *, GError **) { return 1; }
const char *sbitonic_kernel_name(CloSort *, cl_uint i, GError **err) {
	if (i >= 1) {
		set_error(err, CLO_ERROR_ARGS, "Kernel index %u out of range", i);
		return nullptr;
	}
	return kSbitonicKernels[0];
}
size_t sbitonic_localmem(CloSort *, cl_uint, size_t, size_t, GError **) {
	return 0;
}

cl_uint abitonic_num_kernels(CloSort *, GError **) { return 3; }
const char *abitonic_kernel_name(CloSort *, cl_uint i, GError **err) {
	if (i >= 3) {
		set_error(err, CLO_ERROR_ARGS, "Kernel index %u out of range", i);
		return nullptr;
	}
	return kAbitonicKernels[i];
}
size_t abitonic_localmem(CloSort *s, cl_uint i, size_t, size_t,
	GError **) {
	size_t eb = clo_sort_get_element_size(s);
	size_t tile = eb >= 8 ? 8192 : 16384;
	return i == 1 ? 0 : tile * eb + tile / 32 * eb;
}

// ============================================================ gselect
const char *gselect_init(CloSort *s, const char *options, GError **err) {
	(void)options;
	s->data = nullptr;
	return "sm_103a:gselect(rank by counting)";
}

void gselect_finalize(CloSort *s) { (void)s; }

CCLEvent *gselect_sort(CloSort *s, CCLQueue *q, CCLQueue *cq_comm,
	CCLBuffer *in, CCLBuffer *out, size_t numel, size_t lws_max,
	GError **err) {
	(void)cq_comm;
	(void)lws_max;
	if (!check_numel(s, in, numel, err)) return nullptr;
	ccl_event *ev = clo::event_begin(q, "gselect");
	size_t bytes = numel * clo_type_sizeof(s->elem_type);
	if (s->jit) {
		CCLBuffer *dst = out != nullptr ? out : in;
		if (out != nullptr && out != in && !check_numel(s, out, numel, err)) return nullptr;
		if (!jit_sort(s, q, in->ptr, dst->ptr, numel, JIT_GSELECT, err)) return nullptr;
		clo::event_end(ev);
		return ev;
	}
	if (out != nullptr && out != in) {
		if (!check_numel(s, out, numel, err)) return nullptr;
		if (clo::gselect_sort(in->ptr, out->ptr, numel, s->elem_type, nullptr,
				nullptr, 0, s->ctx, q->stream, err) != cudaSuccess)
			return nullptr;
	} else {
		// No output buffer: sort into a temporary and copy back, as the
		// reference does (clo_sort_gselect.c:82-124).
		void *tmp = clo::tmp_alloc(s->ctx, bytes, q->stream, err);
		if (!tmp) return nullptr;
		if (clo::gselect_sort(in->ptr, tmp, numel, s->elem_type, nullptr,
				nullptr, 0, s->ctx, q->stream, err) != cudaSuccess) {
			clo::tmp_free(tmp, q->stream);
			return nullptr;
		}
		bool ok = cuda_ok(cudaMemcpyAsync(in->ptr, tmp, bytes,
			cudaMemcpyDeviceToDevice, q->stream), err, "gselect copy back");
		clo::tmp_free(tmp, q->stream);
		if (!ok) return nullptr;
	}
	clo::event_end(ev);
	return ev;
}

cl_uint gselect_num_kernels(CloSort *, GError **) { return 1; }
const char *gselect_kernel_name(CloSort *, cl_uint i, GError **err) {
	if (i >= 1) {
		set_error(err, CLO_ERROR_ARGS, "Kernel index %u out of range", i);
		return nullptr;
	}
	return "gselect";
}
size_t gselect_localmem(CloSort *s, cl_uint, size_t, size_t, GError **) {
	return 2048 * clo_sort_get_element_size(s);
}

}  // namespace

extern "C" {

const CloSortImplDef clo_sort_sbitonic_def = {"sbitonic", CL_TRUE,
	sbitonic_init, bitonic_finalize, sbitonic_sort, sbitonic_num_kernels,
	sbitonic_kernel_name, sbitonic_localmem};

const CloSortImplDef clo_sort_abitonic_def = {"abitonic", CL_TRUE,
	abitonic_init, bitonic_finalize, abitonic_sort, abitonic_num_kernels,
	abitonic_kernel_name, abitonic_localmem};

const CloSortImplDef clo_sort_gselect_def = {"gselect", CL_FALSE,
	gselect_init, gselect_finalize, gselect_sort, gselect_num_kernels,
	gselect_kernel_name, gselect_localmem};

const CloSortImplDef clo_sort_satradix_def = {"satradix", CL_TRUE,
	satradix_init, satradix_finalize, satradix_sort, satradix_num_kernels,
	satradix_kernel_name, satradix_localmem};

CloSort *clo_sort_new(const char *type, const char *options, CCLContext *ctx,
	CloType *elem_type, CloType *key_type, const char *compare,
	const char *get_key, const char *compiler_opts, GError **err) {
	if (err != nullptr && *err != nullptr) return nullptr;
	const CloSortImplDef *impls[] = {&clo_sort_sbitonic_def,
		&clo_sort_abitonic_def, &clo_sort_gselect_def, &clo_sort_satradix_def};
	const CloSortImplDef *def = nullptr;
	for (const CloSortImplDef *d : impls)
		if (type && strcmp(type, d->name) == 0) def = d;
	if (!def) {
		set_error(err, CLO_ERROR_IMPL_NOT_FOUND,
			"The requested sort implementation, '%s', was not found.",
			type ? type : "(null)");
		return nullptr;
	}
	if (!ctx || !elem_type || clo_type_sizeof(*elem_type) == 0 ||
		(key_type && clo_type_sizeof(*key_type) == 0)) {
		set_error(err, CLO_ERROR_ARGS, "Invalid context or element/key type");
		return nullptr;
	}
	CloSort *s = new clo_sort();
	s->impl_def = *def;
	ccl_context_ref(ctx);
	s->ctx = ctx;
	s->prg = nullptr;
	s->elem_type = *elem_type;
	s->key_type = key_type ? *key_type : *elem_type;
	s->data = nullptr;
	GError *e2 = nullptr;
	const char *src = s->impl_def.init(s, options, &e2);
	if (!src) {
		clo::propagate_error(err, e2);
		clo_sort_destroy(s);
		return nullptr;
	}
	// satradix ignores the compare macro (it always orders by the key's
	// unsigned bits, clo_sort_satradix.cl:58,140) and handles a narrower or
	// wider key type through its sort bits; it needs built kernels only for
	// a custom get_key. The other sorters use them for any custom macro or
	// a key type other than the element type.
	const bool is_radix = def == &clo_sort_satradix_def;
	const bool custom = is_radix ? !get_key_is_default(get_key)
		: (!compare_is_default(compare) || !get_key_is_default(get_key) ||
			s->key_type != s->elem_type);
	if (custom) {
		s->jit = clo::jit_sort_get(s->elem_type, s->key_type, compare, get_key,
			ctx->ordinal, &e2);
		if (!s->jit) {
			clo::propagate_error(err, e2);
			clo_sort_destroy(s);
			return nullptr;
		}
	}
	s->prg = new ccl_program();
	char macros[512];
	snprintf(macros, sizeof macros,
		"#define CLO_SORT_ELEM_TYPE %s\n#define CLO_SORT_KEY_TYPE %s\n"
		"#define CLO_SORT_COMPARE(a, b) %s\n#define CLO_SORT_KEY_GET(x) %s\n",
		clo_type_get_name(s->elem_type), clo_type_get_name(s->key_type),
		compare ? compare : "((a) > (b))", get_key ? get_key : "(x)");
	s->prg->src = s->jit ? s->jit->source : std::string(macros) + src;
	s->prg->opts = compiler_opts ? compiler_opts : "";
	clo::wrapper_created();
	return s;
}

void clo_sort_destroy(CloSort *sorter) {
	if (!sorter) return;
	if (sorter->copy_stream || !sorter->group_events.empty()) {
		int prev_dev = -1;
		if (cudaGetDevice(&prev_dev) != cudaSuccess) prev_dev = -1;
		cudaSetDevice(sorter->ctx->ordinal);
		if (sorter->copy_stream) {
			cudaStreamSynchronize(sorter->copy_stream);
			cudaStreamDestroy(sorter->copy_stream);
		}
		for (cudaEvent_t ev : sorter->group_events) cudaEventDestroy(ev);
		if (prev_dev >= 0) cudaSetDevice(prev_dev);
	}
	if (sorter->host_scratch) cudaFreeHost(sorter->host_scratch);
	if (sorter->impl_def.finalize) sorter->impl_def.finalize(sorter);
	if (sorter->ctx) ccl_context_unref(sorter->ctx);
	if (sorter->prg) {
		delete sorter->prg;
		clo::wrapper_destroyed();
	}
	delete sorter;
}

CCLEvent *clo_sort_with_device_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLQueue *cq_comm, CCLBuffer *data_in, CCLBuffer *data_out,
	size_t numel, size_t lws_max, GError **err) {
	if (!sorter || !cq_exec || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_sort_with_device_data: bad arguments\n");
		return nullptr;
	}
	cudaSetDevice(sorter->ctx->ordinal);
	return sorter->impl_def.sort_with_device_data(sorter, cq_exec, cq_comm,
		data_in, data_out, numel, lws_max, err);
}

}  // extern "C"

namespace {

// Host-data satradix for large arrays, with the copy back overlapped by
// the sort: after the copy in, one stable partition pass by the top digit
// splits the keys into 256 ordered groups; groups of kBucketsPerGroup are
// then sorted (each group's buckets as segments, by the remaining bits)
// one after the other, and each group's copy to the host starts, on a
// second stream, as soon as it is sorted. Stable throughout, so the result
// is the single satradix sort's.
constexpr int kBucketsPerGroup = 16;

bool satradix_host_pipelined(CloSort *s, CCLQueue *q, const void *h_in, void *h_out,
	size_t n, GError **err) {
	CCLContext *ctx = s->ctx;
	const size_t eb = clo_type_sizeof(s->elem_type);
	const int bits = satradix_sort_bits(s);
	const int groups = 256 / kBucketsPerGroup;
	cudaStream_t cs = q->stream;
	if (!s->copy_stream &&
		!cuda_ok(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), err, "stream"))
		return false;
	while ((int)s->group_events.size() < groups) {
		cudaEvent_t ev = nullptr;
		if (!cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), err, "event"))
			return false;
		s->group_events.push_back(ev);
	}
	cudaStream_t xs = s->copy_stream;
	const size_t rel_words = (size_t)groups * (kBucketsPerGroup + 1);
	if (!s->host_scratch &&
		!cuda_ok(cudaMallocHost(&s->host_scratch, (128 + rel_words) * sizeof(uint64_t)), err,
			"cudaMallocHost"))
		return false;
	uint32_t *counts = reinterpret_cast<uint32_t *>(s->host_scratch);  // 256 words
	uint64_t *h_rel = s->host_scratch + 128;
	const size_t off_b = (n * eb + 255) / 256 * 256;
	const size_t off_rel = off_b + (n * eb + 255) / 256 * 256;
	char *dev = (char *)clo::tmp_alloc(ctx, off_rel + rel_words * 8, cs, err);
	bool ok = dev != nullptr;
	char *da = dev, *db = dev + off_b;
	uint64_t *d_rel = (uint64_t *)(dev + off_rel);
	ok = ok && cuda_ok(cudaMemcpyAsync(da, h_in, n * eb, cudaMemcpyHostToDevice, cs), err,
		"copy in");
	ok = ok && clo::radix_msd_partition(da, db, n, (int)eb, bits, counts, ctx, cs, err) ==
		cudaSuccess;
	uint64_t off[257];
	off[0] = 0;
	for (int d = 0; d < 256; ++d) off[d + 1] = off[d] + (ok ? counts[d] : 0);
	if (ok) {
		for (int g = 0; g < groups; ++g)
			for (int j = 0; j <= kBucketsPerGroup; ++j)
				h_rel[(size_t)g * (kBucketsPerGroup + 1) + j] =
					off[g * kBucketsPerGroup + j] - off[g * kBucketsPerGroup];
		ok = cuda_ok(cudaMemcpyAsync(d_rel, h_rel, rel_words * 8,
			cudaMemcpyHostToDevice, cs), err, "offsets");
	}
	for (int g = 0; g < groups && ok; ++g) {
		const uint64_t base = off[g * kBucketsPerGroup];
		const uint64_t len = off[(g + 1) * kBucketsPerGroup] - base;
		if (len == 0) continue;
		char *gp = db + base * eb;
		// The input buffer is free after the partition: it is the groups'
		// second buffer, and a group whose passes end there is copied from
		// there.
		bool in_alt = false;
		if (bits > 8)
			ok = clo::seg_sort(gp, len, d_rel + (size_t)g * (kBucketsPerGroup + 1),
				kBucketsPerGroup, (int)eb, bits - 8, 0, ctx, cs, err, da + base * eb,
				&in_alt) == cudaSuccess;
		if (in_alt) gp = da + base * eb;
		if (!ok) break;
		cudaEvent_t ev = s->group_events[g];
		ok = cuda_ok(cudaEventRecord(ev, cs), err, "event") &&
			cuda_ok(cudaStreamWaitEvent(xs, ev, 0), err, "wait") &&
			cuda_ok(cudaMemcpyAsync((char *)h_out + base * eb, gp, len * eb,
				cudaMemcpyDeviceToHost, xs), err, "copy out");
	}
	cudaStreamSynchronize(xs);
	cudaStreamSynchronize(cs);
	ok = ok && clo::check_device_status(ctx, err);
	clo::tmp_free(dev, cs);
	cudaStreamSynchronize(cs);
	return ok;
}

}  // namespace

extern "C" {

cl_bool clo_sort_with_host_data(CloSort *sorter, CCLQueue *cq_exec,
	CCLQueue *cq_comm, void *data_in, void *data_out, size_t numel,
	size_t lws_max, GError **err) {
	if (!sorter || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_sort_with_host_data: bad arguments\n");
		return CL_FALSE;
	}
	CCLContext *ctx = sorter->ctx;
	cudaSetDevice(ctx->ordinal);
	// Large satradix sorts overlap the copy back with the sort.
	if (strcmp(sorter->impl_def.name, "satradix") == 0 && !sorter->jit &&
		numel >= ((size_t)1 << 22) && numel < ((size_t)1 << 30) &&
		satradix_sort_bits(sorter) >= 16 && clo_type_sizeof(sorter->elem_type) >= 2) {
		CCLQueue *q = cq_exec;
		GError *e3 = nullptr;
		if (!q) q = ccl_queue_new(ctx, &ctx->device, 0, &e3);
		bool ok = q && satradix_host_pipelined(sorter, q, data_in, data_out, numel, &e3);
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
	size_t bytes = numel * clo_type_sizeof(sorter->elem_type);
	cl_bool status = CL_FALSE;
	CCLBuffer *din = nullptr, *dout = nullptr;
	CCLEvent *evt = nullptr;
	CCLEventWaitList ewl = nullptr;
	void *pin = clo::tmp_alloc(ctx, bytes, cq_comm->stream, &e2);
	void *pout = nullptr;
	if (!pin) goto done;
	din = ccl_buffer_new_wrap(ctx, pin, bytes, &e2);
	if (!sorter->impl_def.in_place) {
		pout = clo::tmp_alloc(ctx, bytes, cq_comm->stream, &e2);
		if (!pout) goto done;
		dout = ccl_buffer_new_wrap(ctx, pout, bytes, &e2);
	}
	evt = ccl_buffer_enqueue_write(din, cq_comm, CL_FALSE, 0, bytes, data_in,
		nullptr, &e2);
	if (!evt) goto done;
	if (cq_comm != cq_exec)
		ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!clo::wait_ewl(cq_exec, &ewl, &e2)) goto done;
	evt = sorter->impl_def.sort_with_device_data(sorter, cq_exec, cq_comm, din,
		dout, numel, lws_max, &e2);
	if (!evt) goto done;
	if (cq_comm != cq_exec) ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	evt = ccl_buffer_enqueue_read(dout ? dout : din, cq_comm, CL_FALSE, 0,
		bytes, data_out, &ewl, &e2);
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

CCLContext *clo_sort_get_context(CloSort *s) { return s ? s->ctx : nullptr; }
CCLProgram *clo_sort_get_program(CloSort *s) { return s ? s->prg : nullptr; }
CloType clo_sort_get_element_type(CloSort *s) {
	return s ? s->elem_type : (CloType)-1;
}
size_t clo_sort_get_element_size(CloSort *s) {
	return s ? clo_type_sizeof(s->elem_type) : 0;
}
CloType clo_sort_get_key_type(CloSort *s) {
	return s ? s->key_type : (CloType)-1;
}
size_t clo_sort_get_key_size(CloSort *s) {
	return s ? clo_type_sizeof(s->key_type) : 0;
}
void *clo_sort_get_data(CloSort *s) { return s ? s->data : nullptr; }
void clo_sort_set_data(CloSort *s, void *data) {
	if (s) s->data = data;
}
cl_uint clo_sort_get_num_kernels(CloSort *s, GError **err) {
	return s ? s->impl_def.get_num_kernels(s, err) : 0;
}
const char *clo_sort_get_kernel_name(CloSort *s, cl_uint i, GError **err) {
	return s ? s->impl_def.get_kernel_name(s, i, err) : nullptr;
}
size_t clo_sort_get_localmem_usage(CloSort *s, cl_uint i, size_t lws_max,
	size_t numel, GError **err) {
	return s ? s->impl_def.get_localmem_usage(s, i, lws_max, numel, err) : 0;
}

// ------------------------------------------------------- key-value sort
CCLEvent *clo_sort_kv_with_device_data(CloSort *sorter, CCLQueue *q,
	CCLBuffer *keys, CCLBuffer *values, CloType value_type, size_t numel,
	GError **err) {
	if (!sorter || !q || (err && *err)) {
		fprintf(stderr, "cl_ops: clo_sort_kv_with_device_data: bad arguments\n");
		return nullptr;
	}
	cudaSetDevice(sorter->ctx->ordinal);
	size_t vb = clo_type_sizeof(value_type);
	const char *name = sorter->impl_def.name;
	bool radix = strcmp(name, "satradix") == 0;
	bool gsel = strcmp(name, "gselect") == 0;
	if (!radix && !gsel) {
		set_error(err, CLO_ERROR_ARGS,
			"Key-value sorting needs a stable sorter (satradix or gselect), "
			"not '%s'", name);
		return nullptr;
	}
	if (vb != 4 && vb != 8) {
		set_error(err, CLO_ERROR_ARGS, "Value type must be 4 or 8 bytes wide");
		return nullptr;
	}
	if (sorter->jit) {
		set_error(err, CLO_ERROR_ARGS,
			"Key-value sorting takes the default compare and get_key only");
		return nullptr;
	}
	if (!check_numel(sorter, keys, numel, err)) return nullptr;
	if (!values || values->size < numel * vb) {
		set_error(err, CLO_ERROR_ARGS, "Value buffer too small");
		return nullptr;
	}
	ccl_event *ev = clo::event_begin(q, radix ? "satradix_kv" : "gselect_kv");
	size_t kb = clo_type_sizeof(sorter->elem_type);
	if (radix) {
		bool skip = !clo::stream_capturing(q->stream);
		if (clo::radix_sort(keys->ptr, values->ptr, numel, (int)kb, (int)vb,
				satradix_sort_bits(sorter), sorter->ctx, q->stream, skip,
				err) != cudaSuccess)
			return nullptr;
	} else {
		void *tk = clo::tmp_alloc(sorter->ctx, numel * kb, q->stream, err);
		if (!tk) return nullptr;
		void *tv = clo::tmp_alloc(sorter->ctx, numel * vb, q->stream, err);
		if (!tv) {
			clo::tmp_free(tk, q->stream);
			return nullptr;
		}
		bool ok = clo::gselect_sort(keys->ptr, tk, numel, sorter->elem_type,
			values->ptr, tv, (int)vb, sorter->ctx, q->stream, err) == cudaSuccess;
		ok = ok && cuda_ok(cudaMemcpyAsync(keys->ptr, tk, numel * kb,
			cudaMemcpyDeviceToDevice, q->stream), err, "kv copy back");
		ok = ok && cuda_ok(cudaMemcpyAsync(values->ptr, tv, numel * vb,
			cudaMemcpyDeviceToDevice, q->stream), err, "kv copy back");
		clo::tmp_free(tk, q->stream);
		clo::tmp_free(tv, q->stream);
		if (!ok) return nullptr;
	}
	clo::event_end(ev);
	return ev;
}

cl_bool clo_sort_kv_with_host_data(CloSort *sorter, CCLQueue *q, void *keys,
	void *values, CloType value_type, size_t numel, GError **err) {
	if (!sorter || (err && *err)) return CL_FALSE;
	CCLContext *ctx = sorter->ctx;
	cudaSetDevice(ctx->ordinal);
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
	size_t kbytes = numel * clo_type_sizeof(sorter->elem_type);
	size_t vbytes = numel * clo_type_sizeof(value_type);
	cl_bool status = CL_FALSE;
	CCLBuffer *dk = nullptr, *dv = nullptr;
	CCLEventWaitList ewl = nullptr;
	CCLEvent *evt = nullptr;
	void *pk = clo::tmp_alloc(ctx, kbytes, q->stream, &e2);
	void *pv = pk ? clo::tmp_alloc(ctx, vbytes, q->stream, &e2) : nullptr;
	if (!pk || !pv) goto done;
	dk = ccl_buffer_new_wrap(ctx, pk, kbytes, &e2);
	dv = ccl_buffer_new_wrap(ctx, pv, vbytes, &e2);
	if (!ccl_buffer_enqueue_write(dk, q, CL_FALSE, 0, kbytes, keys, nullptr, &e2))
		goto done;
	if (!ccl_buffer_enqueue_write(dv, q, CL_FALSE, 0, vbytes, values, nullptr, &e2))
		goto done;
	if (!clo_sort_kv_with_device_data(sorter, q, dk, dv, value_type, numel, &e2))
		goto done;
	if (!ccl_buffer_enqueue_read(dk, q, CL_FALSE, 0, kbytes, keys, nullptr, &e2))
		goto done;
	evt = ccl_buffer_enqueue_read(dv, q, CL_FALSE, 0, vbytes, values, nullptr, &e2);
	if (!evt) goto done;
	ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!ccl_event_wait(&ewl, &e2)) goto done;
	status = CL_TRUE;
done:
	ccl_event_wait_list_clear(&ewl);
	if (dk) ccl_buffer_destroy(dk);
	if (dv) ccl_buffer_destroy(dv);
	clo::tmp_free(pk, q->stream);
	clo::tmp_free(pv, q->stream);
	if (!status) cudaStreamSynchronize(q->stream);
	if (own) ccl_queue_destroy(own);
	clo::propagate_error(err, e2);
	return status;
}

}  // extern "C"

// ------------------------------------------------------- segmented sort
namespace {

bool seg_args_ok(CloSort *sorter, CCLQueue *q, const char *what, GError **err) {
	if (!sorter || !q || (err && *err)) {
		fprintf(stderr, "cl_ops: %s: bad arguments\n", what);
		return false;
	}
	if (strcmp(sorter->impl_def.name, "satradix") != 0) {
		set_error(err, CLO_ERROR_ARGS,
			"Segmented sorting is implemented for the satradix sorter (stable, "
			"unsigned key order), not '%s'", sorter->impl_def.name);
		return false;
	}
	if (sorter->jit) {
		set_error(err, CLO_ERROR_ARGS,
			"Segmented sorting takes the default get_key only");
		return false;
	}
	return true;
}

CCLEvent *seg_sort_device(CloSort *sorter, CCLQueue *q, CCLBuffer *data,
	CCLBuffer *offsets, size_t nseg, int variant, GError **err) {
	const size_t eb = clo_type_sizeof(sorter->elem_type);
	if (!data || (nseg > 0 && (!offsets || offsets->size < (nseg + 1) * 8))) {
		set_error(err, CLO_ERROR_ARGS,
			"Segmented sort needs a data buffer and %zu offsets", nseg + 1);
		return nullptr;
	}
	ccl_event *ev = clo::event_begin(q, "satradix_segmented");
	if (nseg > 0 && clo::seg_sort(data->ptr, data->size / eb,
			(const uint64_t *)offsets->ptr, nseg, (int)eb, satradix_sort_bits(sorter),
			variant, sorter->ctx, q->stream, err) != cudaSuccess)
		return nullptr;
	clo::event_end(ev);
	return ev;
}

}  // namespace

extern "C" {

CCLEvent *clo_sort_segmented_with_device_data(CloSort *sorter, CCLQueue *q,
	CCLBuffer *data, CCLBuffer *offsets, size_t num_segments, GError **err) {
	if (!seg_args_ok(sorter, q, "clo_sort_segmented_with_device_data", err))
		return nullptr;
	cudaSetDevice(sorter->ctx->ordinal);
	SatradixData *d = (SatradixData *)sorter->data;
	return seg_sort_device(sorter, q, data, offsets, num_segments, d->seg_variant, err);
}

cl_bool clo_sort_segmented_with_host_data(CloSort *sorter, CCLQueue *q, void *data,
	size_t numel, const cl_ulong *offsets, size_t num_segments, GError **err) {
	if (!sorter || (err && *err)) return CL_FALSE;
	CCLContext *ctx = sorter->ctx;
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
	const size_t bytes = numel * clo_type_sizeof(sorter->elem_type);
	const size_t obytes = (num_segments + 1) * 8;
	cl_bool status = CL_FALSE;
	CCLBuffer *dd = nullptr, *doff = nullptr;
	CCLEventWaitList ewl = nullptr;
	CCLEvent *evt = nullptr;
	void *pd = clo::tmp_alloc(ctx, bytes, q->stream, &e2);
	void *po = pd ? clo::tmp_alloc(ctx, obytes, q->stream, &e2) : nullptr;
	if (!pd || !po) goto done;
	dd = ccl_buffer_new_wrap(ctx, pd, bytes, &e2);
	doff = ccl_buffer_new_wrap(ctx, po, obytes, &e2);
	if (!ccl_buffer_enqueue_write(dd, q, CL_FALSE, 0, bytes, data, nullptr, &e2))
		goto done;
	if (num_segments > 0 &&
		!ccl_buffer_enqueue_write(doff, q, CL_FALSE, 0, obytes, offsets, nullptr, &e2))
		goto done;
	if (!clo_sort_segmented_with_device_data(sorter, q, dd, doff, num_segments, &e2))
		goto done;
	evt = ccl_buffer_enqueue_read(dd, q, CL_FALSE, 0, bytes, data, nullptr, &e2);
	if (!evt) goto done;
	ccl_ewl(&ewl, evt, (CCLEvent *)nullptr);
	if (!ccl_event_wait(&ewl, &e2)) goto done;
	status = CL_TRUE;
done:
	ccl_event_wait_list_clear(&ewl);
	if (dd) ccl_buffer_destroy(dd);
	if (doff) ccl_buffer_destroy(doff);
	clo::tmp_free(pd, q->stream);
	clo::tmp_free(po, q->stream);
	if (!status) cudaStreamSynchronize(q->stream);
	if (own) ccl_queue_destroy(own);
	clo::propagate_error(err, e2);
	return status;
}

cl_int clo_sort_segmented_tune(CloSort *sorter, CCLQueue *q, CCLBuffer *data,
	CCLBuffer *offsets, size_t num_segments, double *times_ms, GError **err) {
	if (!seg_args_ok(sorter, q, "clo_sort_segmented_tune", err)) return -1;
	if (!data) {
		set_error(err, CLO_ERROR_ARGS, "NULL data buffer");
		return -1;
	}
	CCLContext *ctx = sorter->ctx;
	cudaSetDevice(ctx->ordinal);
	SatradixData *d = (SatradixData *)sorter->data;
	const int nv = clo::seg_sort_num_variants();
	// Each variant sorts a fresh copy of the caller's data; the best of two
	// runs counts. The caller's data is left as it was.
	void *work = clo::tmp_alloc(ctx, data->size, q->stream, err);
	if (!work) return -1;
	CCLBuffer *wb = ccl_buffer_new_wrap(ctx, work, data->size, err);
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	int best = -1;
	double best_ms = 0.0;
	GError *e2 = nullptr;
	for (int v = 0; v < nv && !e2; ++v) {
		double vbest = -1.0;
		for (int rep = 0; rep < 2 && !e2; ++rep) {
			if (!cuda_ok(cudaMemcpyAsync(work, data->ptr, data->size,
					cudaMemcpyDeviceToDevice, q->stream), &e2, "tune copy"))
				break;
			cudaEventRecord(e0, q->stream);
			if (!seg_sort_device(sorter, q, wb, offsets, num_segments, v, &e2)) break;
			cudaEventRecord(e1, q->stream);
			if (!cuda_ok(cudaEventSynchronize(e1), &e2, "tune wait")) break;
			if (!clo::check_device_status(ctx, &e2)) break;
			float ms = 0.f;
			cudaEventElapsedTime(&ms, e0, e1);
			if (vbest < 0 || ms < vbest) vbest = ms;
		}
		if (e2) break;
		if (times_ms) times_ms[v] = vbest;
		if (best < 0 || vbest < best_ms) {
			best = v;
			best_ms = vbest;
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	ccl_buffer_destroy(wb);
	clo::tmp_free(work, q->stream);
	cudaStreamSynchronize(q->stream);
	if (e2) {
		clo::propagate_error(err, e2);
		return -1;
	}
	d->seg_variant = best;
	return best;
}

cl_int clo_sort_segmented_get_variant(CloSort *sorter) {
	if (!sorter || strcmp(sorter->impl_def.name, "satradix") != 0) return -1;
	return ((SatradixData *)sorter->data)->seg_variant;
}

}  // extern "C"
