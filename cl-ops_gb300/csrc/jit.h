// NVRTC-built kernels for sorters with custom compare / get_key snippets.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>

#include "clo_internal.h"

namespace clo {

struct JitSort {
	std::string source;
	cudaLibrary_t lib = nullptr;
	cudaKernel_t keys = nullptr;          // keys[i] = KEY_GET(in[i]), idx[i] = i
	cudaKernel_t gather = nullptr;        // out[i] = in[idx[i]]
	cudaKernel_t bitonic_step = nullptr;  // one network step with padding flags
	cudaKernel_t gselect = nullptr;       // rank-by-count
};

// The program text for these macros (also what clo_sort_get_program's
// source returns).
std::string jit_sort_source(CloType elem, CloType key, const char *compare,
	const char *get_key);

// Compiled (and cached) program for these macros on device `ordinal`.
std::shared_ptr<JitSort> jit_sort_get(CloType elem, CloType key, const char *compare,
	const char *get_key, int ordinal, GError **err);

// Compiles CUDA source text with NVRTC for sm_103a (plus `options`,
// whitespace-separated) and loads it on device `ordinal`. On a compile
// error, *log (when given) receives NVRTC's log and err says why.
cudaLibrary_t jit_build(const std::string &src, const char *file_name,
	const std::string &options, int ordinal, std::string *log, GError **err);

// Grid-stride launch of a JIT kernel over `work` items, 256 threads.
cudaError_t jit_launch(cudaKernel_t k, size_t work, void **args, cudaStream_t s,
	int sm_count);

}  // namespace clo
