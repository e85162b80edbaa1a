// Custom compare / get_key snippets: the reference builds each sorter's
// OpenCL program with
//   #define CLO_SORT_ELEM_TYPE, CLO_SORT_KEY_TYPE, CLO_SORT_COMPARE(a, b),
//   #define CLO_SORT_KEY_GET(x)
// prepended to its kernels (src/cl_ops/sort/clo_sort_abstract.c:141-179).
// Here the same macros are prepended to a small CUDA program that NVRTC
// compiles for sm_103a when the sorter is created; its kernels extract
// keys, gather by index, run one bitonic network step and rank-by-count
// (gselect). Programs are cached by source text. NVRTC is loaded on first
// use, so the library has no link-time dependency on it.
#include <dlfcn.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "clo_internal.h"
#include "jit.h"

namespace clo {
namespace {

// NVRTC entry points used (nvrtc.h signatures, loaded with dlsym).
typedef int nvrtcResult_t;
typedef struct _nvrtcProgram *nvrtcProgram_t;
struct Nvrtc {
	nvrtcResult_t (*create)(nvrtcProgram_t *, const char *, const char *, int,
		const char *const *, const char *const *);
	nvrtcResult_t (*compile)(nvrtcProgram_t, int, const char *const *);
	nvrtcResult_t (*log_size)(nvrtcProgram_t, size_t *);
	nvrtcResult_t (*log)(nvrtcProgram_t, char *);
	nvrtcResult_t (*cubin_size)(nvrtcProgram_t, size_t *);
	nvrtcResult_t (*cubin)(nvrtcProgram_t, char *);
	nvrtcResult_t (*destroy)(nvrtcProgram_t *);
	bool ok = false;
};

Nvrtc *nvrtc(GError **err) {
	static Nvrtc n;
	static std::once_flag once;
	std::call_once(once, [] {
		const char *names[] = {"libnvrtc.so.13", "libnvrtc.so",
			"/usr/local/cuda/lib64/libnvrtc.so.13", "/usr/local/cuda/lib64/libnvrtc.so"};
		void *h = nullptr;
		for (const char *nm : names)
			if ((h = dlopen(nm, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
		if (!h) return;
		n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
		n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
		n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
		n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
		n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
		n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
		n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
		n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin &&
			n.destroy;
	});
	if (!n.ok) {
		set_error(err, CLO_ERROR_LIBRARY,
			"Custom compare/get_key need NVRTC (libnvrtc.so), which could not be loaded");
		return nullptr;
	}
	return &n;
}

// CUDA spelling of each CloType for the program's macros.
const char *cuda_type(CloType t) {
	switch (t) {
	case CLO_CHAR: return "cl_char";
	case CLO_UCHAR: return "uchar";
	case CLO_SHORT: return "short";
	case CLO_USHORT: return "ushort";
	case CLO_INT: return "int";
	case CLO_UINT: return "uint";
	case CLO_LONG: return "cl_long";
	case CLO_ULONG: return "ulong";
	case CLO_FLOAT: return "float";
	case CLO_DOUBLE: return "double";
	default: return nullptr;
	}
}

// The kernels (the macros come first). OpenCL scalar names are typedefs
// so that snippets written for the reference compile unchanged.
const char kProgram[] = R"CLO(
typedef signed char cl_char;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef long long cl_long;
typedef unsigned long long ulong;
typedef CLO_SORT_ELEM_TYPE clo_elem_t;
typedef CLO_SORT_KEY_TYPE clo_key_t;

extern "C" __global__ void clo_jit_keys(const clo_elem_t *in, clo_key_t *keys,
		uint *idx, ulong n) {
	for (ulong i = blockIdx.x * (ulong)blockDim.x + threadIdx.x; i < n;
			i += (ulong)gridDim.x * blockDim.x) {
		clo_elem_t x = in[i];
		keys[i] = (clo_key_t)(CLO_SORT_KEY_GET(x));
		idx[i] = (uint)i;
	}
}

extern "C" __global__ void clo_jit_gather(const clo_elem_t *in, const uint *idx,
		clo_elem_t *out, ulong n) {
	for (ulong i = blockIdx.x * (ulong)blockDim.x + threadIdx.x; i < n;
			i += (ulong)gridDim.x * blockDim.x)
		out[i] = in[idx[i]];
}

// One step of the reference bitonic network (clo_sort_sbitonic.cl:38-69):
// work-item g compares i1 = g + (g / s) * s and i2 = i1 + s (s = 2^(step-1))
// and swaps iff COMPARE(key1, key2) XOR desc, desc = bit (stage - 1) of g.
// Positions past the real elements (pad != 0) compare as greater than
// every element and equal to each other.
extern "C" __global__ void clo_jit_bitonic_step(clo_elem_t *d, uchar *pad,
		uint stage, uint step, ulong half) {
	for (ulong g = blockIdx.x * (ulong)blockDim.x + threadIdx.x; g < half;
			g += (ulong)gridDim.x * blockDim.x) {
		const ulong s = 1ull << (step - 1);
		const ulong i1 = g + (g / s) * s, i2 = i1 + s;
		const bool desc = (g >> (stage - 1)) & 1ull;
		const uchar p1 = pad[i1], p2 = pad[i2];
		bool gt;
		if (p1 | p2) {
			gt = p1 && !p2;
		} else {
			clo_elem_t x1 = d[i1], x2 = d[i2];
			clo_key_t k1 = (clo_key_t)(CLO_SORT_KEY_GET(x1));
			clo_key_t k2 = (clo_key_t)(CLO_SORT_KEY_GET(x2));
			gt = (CLO_SORT_COMPARE(k1, k2)) ? true : false;
		}
		if (gt ^ desc) {
			clo_elem_t t = d[i1];
			d[i1] = d[i2];
			d[i2] = t;
			pad[i1] = p2;
			pad[i2] = p1;
		}
	}
}

// gselect rank (clo_sort_gselect.cl:38-57): the element goes to the number
// of elements before it in (COMPARE, then index) order.
extern "C" __global__ void clo_jit_gselect(const clo_elem_t *in, clo_elem_t *out,
		ulong n) {
	for (ulong g = blockIdx.x * (ulong)blockDim.x + threadIdx.x; g < n;
			g += (ulong)gridDim.x * blockDim.x) {
		clo_elem_t xg = in[g];
		clo_key_t kg = (clo_key_t)(CLO_SORT_KEY_GET(xg));
		ulong pos = 0;
		for (ulong i = 0; i < n; ++i) {
			clo_elem_t xi = in[i];
			clo_key_t ki = (clo_key_t)(CLO_SORT_KEY_GET(xi));
			if ((CLO_SORT_COMPARE(kg, ki)) || ((ki == kg) && (i < g))) pos++;
		}
		out[pos] = xg;
	}
}
)CLO";

std::mutex g_mu;
std::map<std::string, std::shared_ptr<JitSort>> g_cache;

}  // namespace

std::string jit_sort_source(CloType elem, CloType key, const char *compare,
	const char *get_key) {
	std::string s;
	s += "#define CLO_SORT_ELEM_TYPE ";
	s += cuda_type(elem) ? cuda_type(elem) : "?";
	s += "\n#define CLO_SORT_KEY_TYPE ";
	s += cuda_type(key) ? cuda_type(key) : "?";
	s += "\n#define CLO_SORT_COMPARE(a, b) ";
	s += compare ? compare : "((a) > (b))";
	s += "\n#define CLO_SORT_KEY_GET(x) ";
	s += get_key ? get_key : "(x)";
	s += "\n";
	s += kProgram;
	return s;
}

std::shared_ptr<JitSort> jit_sort_get(CloType elem, CloType key, const char *compare,
	const char *get_key, int ordinal, GError **err) {
	if (!cuda_type(elem) || !cuda_type(key)) {
		set_error(err, CLO_ERROR_ARGS,
			"Custom compare/get_key: element and key types must be integer, float or double");
		return nullptr;
	}
	const std::string src = jit_sort_source(elem, key, compare, get_key);
	const std::string cache_key = std::to_string(ordinal) + "\n" + src;
	std::lock_guard<std::mutex> lk(g_mu);
	auto f = g_cache.find(cache_key);
	if (f != g_cache.end()) return f->second;
	Nvrtc *nv = nvrtc(err);
	if (!nv) return nullptr;
	nvrtcProgram_t prog = nullptr;
	if (nv->create(&prog, src.c_str(), "clo_sort_custom.cu", 0, nullptr, nullptr) != 0) {
		set_error(err, CLO_ERROR_LIBRARY, "nvrtcCreateProgram failed");
		return nullptr;
	}
	const char *opts[] = {"-arch=sm_103a", "-std=c++17", "-default-device"};
	const int rc = nv->compile(prog, 3, opts);
	if (rc != 0) {
		size_t ls = 0;
		nv->log_size(prog, &ls);
		std::string log(ls, '\0');
		if (ls) nv->log(prog, &log[0]);
		nv->destroy(&prog);
		set_error(err, CLO_ERROR_LIBRARY,
			"Building the custom compare/get_key program failed:\n%s", log.c_str());
		return nullptr;
	}
	size_t cs = 0;
	nv->cubin_size(prog, &cs);
	std::vector<char> cubin(cs);
	nv->cubin(prog, cubin.data());
	nv->destroy(&prog);
	auto js = std::make_shared<JitSort>();
	js->source = src;
	cudaSetDevice(ordinal);
	cudaError_t e = cudaLibraryLoadData(&js->lib, cubin.data(), nullptr, nullptr, 0,
		nullptr, nullptr, 0);
	if (e == cudaSuccess) e = cudaLibraryGetKernel(&js->keys, js->lib, "clo_jit_keys");
	if (e == cudaSuccess) e = cudaLibraryGetKernel(&js->gather, js->lib, "clo_jit_gather");
	if (e == cudaSuccess)
		e = cudaLibraryGetKernel(&js->bitonic_step, js->lib, "clo_jit_bitonic_step");
	if (e == cudaSuccess) e = cudaLibraryGetKernel(&js->gselect, js->lib, "clo_jit_gselect");
	if (e != cudaSuccess) {
		cuda_ok(e, err, "loading the custom compare/get_key program");
		return nullptr;
	}
	g_cache[cache_key] = js;
	return js;
}

cudaLibrary_t jit_build(const std::string &src, const char *file_name,
	const std::string &options, int ordinal, std::string *log, GError **err) {
	Nvrtc *nv = nvrtc(err);
	if (!nv) return nullptr;
	std::vector<std::string> words;
	{
		std::string w;
		for (char c : options) {
			if (c == ' ' || c == '\t' || c == '\n') {
				if (!w.empty()) words.push_back(w);
				w.clear();
			} else {
				w += c;
			}
		}
		if (!w.empty()) words.push_back(w);
	}
	std::vector<const char *> opts = {"-arch=sm_103a", "-std=c++17"};
	for (const std::string &w : words) opts.push_back(w.c_str());
	nvrtcProgram_t prog = nullptr;
	std::lock_guard<std::mutex> lk(g_mu);
	if (nv->create(&prog, src.c_str(), file_name, 0, nullptr, nullptr) != 0) {
		set_error(err, CLO_ERROR_LIBRARY, "nvrtcCreateProgram failed");
		return nullptr;
	}
	const int rc = nv->compile(prog, (int)opts.size(), opts.data());
	size_t ls = 0;
	nv->log_size(prog, &ls);
	std::string text(ls, '\0');
	if (ls) nv->log(prog, &text[0]);
	if (log) *log = text.c_str();
	if (rc != 0) {
		nv->destroy(&prog);
		set_error(err, CLO_ERROR_LIBRARY, "Program build failed:\n%s", text.c_str());
		return nullptr;
	}
	size_t cs = 0;
	nv->cubin_size(prog, &cs);
	std::vector<char> cubin(cs);
	nv->cubin(prog, cubin.data());
	nv->destroy(&prog);
	cudaLibrary_t lib = nullptr;
	cudaError_t e = cudaSetDevice(ordinal);
	if (e == cudaSuccess)
		e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
	if (e != cudaSuccess) {
		cuda_ok(e, err, "loading the built program");
		return nullptr;
	}
	return lib;
}

cudaError_t jit_launch(cudaKernel_t k, size_t work, void **args, cudaStream_t s,
	int sm_count) {
	size_t blocks = (work + 255) / 256;
	const size_t cap = (size_t)sm_count * 16;
	if (blocks > cap) blocks = cap;
	if (blocks == 0) blocks = 1;
	count_launches(1);
	return cudaLaunchKernel((const void *)k, dim3((unsigned)blocks), dim3(256), args, 0, s);
}

}  // namespace clo
