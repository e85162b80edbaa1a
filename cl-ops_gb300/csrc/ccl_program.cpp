// Programs and kernels built from a caller's source text: the cf4ocl2
// calls a cl_ops client makes to run its own kernel against a CloRng
// (src/tests/test_rng.c:79-115: ccl_program_new_from_source,
// ccl_program_build, ccl_program_get_kernel, ccl_kernel_suggest_worksizes,
// ccl_kernel_set_args_and_enqueue_ndrange). The source is CUDA (the text
// clo_rng_get_source returns, plus the client's kernels declared
// extern "C" __global__), compiled by NVRTC for the context's device.
//
// NDRange mapping: one dimension, global size G in work-groups of L
// (G a multiple of L, as OpenCL requires) -> G / L blocks of L threads, so
// blockIdx.x * blockDim.x + threadIdx.x is OpenCL's get_global_id(0).
// Kernel arguments follow cf4ocl2: a CCLBuffer passes its device pointer,
// a ccl_arg_priv / ccl_arg_full value passes its bytes, and a
// ccl_arg_local size adds to the launch's dynamic shared memory (which
// the kernel reaches through extern __shared__) without taking a
// parameter slot.
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "clo_internal.h"
#include "jit.h"

struct ccl_kernel {
	CCLProgram *prg;
	cudaKernel_t k;
	std::string name;
};

struct ccl_arg {
	std::vector<unsigned char> bytes;  // empty with local_size set: local memory
	size_t local_size;
	bool local;
};

namespace {

std::mutex g_arg_mu;
std::set<const void *> g_args;  // live CCLArg objects (told apart from buffers)

bool is_arg(const void *p) {
	std::lock_guard<std::mutex> lk(g_arg_mu);
	return g_args.count(p) != 0;
}

void arg_free(CCLArg *a) {
	{
		std::lock_guard<std::mutex> lk(g_arg_mu);
		g_args.erase(a);
	}
	delete a;
}

// Program state beyond the descriptor fields (src, opts): the built
// library, its build log and the kernels handed out.
struct Built {
	CCLContext *ctx = nullptr;
	cudaLibrary_t lib = nullptr;
	std::string log;
	std::map<std::string, ccl_kernel *> kernels;
};
std::mutex g_prg_mu;
std::map<CCLProgram *, Built> g_built;

}  // namespace

using clo::cuda_ok;
using clo::set_error;

extern "C" {

CCLProgram *ccl_program_new_from_source(CCLContext *ctx, const char *string,
	GError **err) {
	if (err && *err) return nullptr;
	if (!ctx || !string) {
		set_error(err, CLO_ERROR_ARGS, "ccl_program_new_from_source: NULL context or source");
		return nullptr;
	}
	CCLProgram *prg = new ccl_program();
	prg->src = string;
	{
		std::lock_guard<std::mutex> lk(g_prg_mu);
		g_built[prg].ctx = ctx;
	}
	ccl_context_ref(ctx);
	clo::wrapper_created();
	return prg;
}

CCLProgram *ccl_program_new_from_sources(CCLContext *ctx, cl_uint count,
	const char **strings, const size_t *lengths, GError **err) {
	if (err && *err) return nullptr;
	std::string all;
	for (cl_uint i = 0; i < count; ++i) {
		if (!strings || !strings[i]) {
			set_error(err, CLO_ERROR_ARGS, "ccl_program_new_from_sources: NULL source %u", i);
			return nullptr;
		}
		if (lengths && lengths[i]) all.append(strings[i], lengths[i]);
		else all += strings[i];
	}
	return ccl_program_new_from_source(ctx, all.c_str(), err);
}

cl_bool ccl_program_build(CCLProgram *prg, const char *options, GError **err) {
	if (err && *err) return CL_FALSE;
	std::lock_guard<std::mutex> lk(g_prg_mu);
	auto it = prg ? g_built.find(prg) : g_built.end();
	if (it == g_built.end()) {
		set_error(err, CLO_ERROR_ARGS, "ccl_program_build: not a program built from source");
		return CL_FALSE;
	}
	Built &b = it->second;
	if (b.lib) {
		set_error(err, CLO_ERROR_ARGS, "ccl_program_build: program already built");
		return CL_FALSE;
	}
	prg->opts = options ? options : "";
	b.lib = clo::jit_build(prg->src, "ccl_program.cu", prg->opts, b.ctx->ordinal, &b.log, err);
	return b.lib ? CL_TRUE : CL_FALSE;
}

const char *ccl_program_get_build_log(CCLProgram *prg, GError **err) {
	(void)err;
	std::lock_guard<std::mutex> lk(g_prg_mu);
	auto it = prg ? g_built.find(prg) : g_built.end();
	return it == g_built.end() ? nullptr : it->second.log.c_str();
}

CCLKernel *ccl_program_get_kernel(CCLProgram *prg, const char *kernel_name, GError **err) {
	if (err && *err) return nullptr;
	std::lock_guard<std::mutex> lk(g_prg_mu);
	auto it = prg ? g_built.find(prg) : g_built.end();
	if (it == g_built.end() || !it->second.lib || !kernel_name) {
		set_error(err, CLO_ERROR_ARGS,
			"ccl_program_get_kernel: program not built or NULL kernel name");
		return nullptr;
	}
	Built &b = it->second;
	auto f = b.kernels.find(kernel_name);
	if (f != b.kernels.end()) return f->second;
	cudaKernel_t k = nullptr;
	cudaSetDevice(b.ctx->ordinal);
	if (!cuda_ok(cudaLibraryGetKernel(&k, b.lib, kernel_name), err,
			"ccl_program_get_kernel (kernels must be extern \"C\" __global__)"))
		return nullptr;
	ccl_kernel *kr = new ccl_kernel{prg, k, kernel_name};
	b.kernels[kernel_name] = kr;
	return kr;
}

void ccl_program_destroy(CCLProgram *prg) {
	if (!prg) return;
	CCLContext *ctx = nullptr;
	{
		std::lock_guard<std::mutex> lk(g_prg_mu);
		auto it = g_built.find(prg);
		if (it == g_built.end()) return;  // a sorter's or scanner's descriptor
		for (auto &kv : it->second.kernels) delete kv.second;
		if (it->second.lib) {
			cudaSetDevice(it->second.ctx->ordinal);
			cudaLibraryUnload(it->second.lib);
		}
		ctx = it->second.ctx;
		g_built.erase(it);
	}
	delete prg;
	clo::wrapper_destroyed();
	ccl_context_unref(ctx);
}

CCLArg *ccl_arg_new(void *value, size_t size) {
	CCLArg *a = new ccl_arg();
	a->local = value == nullptr;
	a->local_size = a->local ? size : 0;
	if (!a->local) a->bytes.assign((unsigned char *)value, (unsigned char *)value + size);
	std::lock_guard<std::mutex> lk(g_arg_mu);
	g_args.insert(a);
	return a;
}

void ccl_arg_destroy(CCLArg *arg) {
	if (arg && is_arg(arg)) arg_free(arg);
}

// cf4ocl2 leaves the choice to the device; here: the largest work-group of
// at most 256 work-items that divides the real size when no global size
// is asked for (so the NDRange is exactly the real size), else 256 (or
// the real size, if smaller) with the global size rounded up to it.
cl_bool ccl_kernel_suggest_worksizes(CCLKernel *krnl, CCLDevice *dev, cl_uint dims,
	const size_t *real_worksize, size_t *gws, size_t *lws, GError **err) {
	(void)krnl;
	(void)dev;
	if (err && *err) return CL_FALSE;
	if (dims != 1 || !real_worksize || !lws || real_worksize[0] == 0) {
		set_error(err, CLO_ERROR_ARGS,
			"ccl_kernel_suggest_worksizes: one dimension with a nonzero size only");
		return CL_FALSE;
	}
	const size_t real = real_worksize[0];
	if (gws) {
		lws[0] = real < 256 ? real : 256;
		gws[0] = (real + lws[0] - 1) / lws[0] * lws[0];
	} else {
		size_t l = real < 256 ? real : 256;
		while (real % l) --l;
		lws[0] = l;
	}
	return CL_TRUE;
}

CCLEvent *ccl_kernel_set_args_and_enqueue_ndrange(CCLKernel *krnl, CCLQueue *cq,
	cl_uint work_dim, const size_t *global_work_offset, const size_t *global_work_size,
	const size_t *local_work_size, CCLEventWaitList *evt_wait_lst, GError **err, ...) {
	// Collect the arguments first, so that every CCLArg is released on
	// every path.
	std::vector<void *> items;
	va_list ap;
	va_start(ap, err);
	for (void *p = va_arg(ap, void *); p != nullptr; p = va_arg(ap, void *)) items.push_back(p);
	va_end(ap);
	std::vector<std::vector<unsigned char>> store;
	std::vector<CCLArg *> owned;
	size_t shared_bytes = 0;
	store.reserve(items.size());
	for (void *p : items) {
		if (is_arg(p)) {
			CCLArg *a = (CCLArg *)p;
			owned.push_back(a);
			if (a->local) shared_bytes += a->local_size;
			else store.push_back(a->bytes);
		} else {
			void *dptr = ccl_buffer_unwrap((CCLBuffer *)p);
			store.emplace_back((unsigned char *)&dptr, (unsigned char *)&dptr + sizeof dptr);
		}
	}
	for (CCLArg *a : owned) arg_free(a);
	if (err && *err) return nullptr;
	if (!krnl || !cq || work_dim != 1 || !global_work_size || global_work_size[0] == 0) {
		set_error(err, CLO_ERROR_ARGS,
			"ccl_kernel_set_args_and_enqueue_ndrange: kernel, queue and a one-dimensional "
			"nonzero global size are required");
		return nullptr;
	}
	if (global_work_offset && global_work_offset[0] != 0) {
		set_error(err, CLO_ERROR_ARGS, "ccl_kernel_set_args_and_enqueue_ndrange: "
			"global work offsets are not supported");
		return nullptr;
	}
	const size_t g = global_work_size[0];
	size_t l = 0;
	if (local_work_size) {
		l = local_work_size[0];
	} else if (!ccl_kernel_suggest_worksizes(krnl, nullptr, 1, &g, nullptr, &l, err)) {
		return nullptr;
	}
	if (l == 0 || l > 1024 || g % l != 0 || g / l > 0x7FFFFFFFull) {
		set_error(err, CLO_ERROR_ARGS,
			"ccl_kernel_set_args_and_enqueue_ndrange: global size %zu is not a multiple of "
			"a local size of 1..1024 (%zu)", g, l);
		return nullptr;
	}
	if (!clo::wait_ewl(cq, evt_wait_lst, err)) return nullptr;
	std::vector<void *> params;
	for (auto &b : store) params.push_back(b.data());
	cudaSetDevice(cq->ctx->ordinal);
	if (shared_bytes > 48 * 1024 &&
		!cuda_ok(cudaKernelSetAttributeForDevice(krnl->k,
				cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared_bytes,
				cq->ctx->ordinal),
			err, "ccl_kernel_set_args_and_enqueue_ndrange: shared memory"))
		return nullptr;
	ccl_event *e = clo::event_begin(cq, krnl->name.c_str());
	cudaError_t ce = cudaLaunchKernel((const void *)krnl->k, dim3((unsigned)(g / l)),
		dim3((unsigned)l), params.data(), shared_bytes, cq->stream);
	clo::event_end(e);
	clo::count_launches(1);
	if (!cuda_ok(ce, err, "ccl_kernel_set_args_and_enqueue_ndrange")) return nullptr;
	return e;
}

}  // extern "C"
