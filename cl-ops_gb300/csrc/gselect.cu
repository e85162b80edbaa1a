// "gselect": rank-by-counting selection sort, stable and out of place.
//
// Reference (src/cl_ops/sort/clo_sort_gselect.cl:38-57): element gid goes
// to position #{i : COMPARE(key_gid, key_i) || (key_i == key_gid && i <
// gid)} with COMPARE(a, b) = a > b, i.e. a stable ascending sort for any
// input without NaN. Here each thread ranks four elements against tiles
// of 2048 keys staged in shared memory. O(n^2) compares: meant for small
// arrays, like the reference.
#include <cuda_fp16.h>

#include "clo_internal.h"

namespace clo {
namespace {

struct Half16 {
	uint16_t bits;
};

template <typename T>
struct GT {
	using C = T;
	__device__ __forceinline__ static C key(T v) { return v; }
};
template <>
struct GT<Half16> {
	using C = float;
	__device__ __forceinline__ static C key(Half16 v) {
		return __half2float(__ushort_as_half(v.bits));
	}
};

constexpr int kThreads = 256;
constexpr int kPer = 4;
constexpr int kChunk = 2048;

template <typename T, typename V, bool HAS_V>
__global__ void __launch_bounds__(kThreads)
gselect_kernel(const T *__restrict__ in, T *__restrict__ out, size_t n,
	const V *__restrict__ vin, V *__restrict__ vout) {
	using C = typename GT<T>::C;
	__shared__ C s_key[kChunk];
	size_t mine[kPer];
	C k[kPer];
	size_t pos[kPer];
	bool valid[kPer];
#pragma unroll
	for (int q = 0; q < kPer; ++q) {
		mine[q] = ((size_t)blockIdx.x * kPer + q) * kThreads + threadIdx.x;
		valid[q] = mine[q] < n;
		k[q] = valid[q] ? GT<T>::key(in[mine[q]]) : C(0);
		pos[q] = 0;
	}
	for (size_t c0 = 0; c0 < n; c0 += kChunk) {
		size_t cn = n - c0 < (size_t)kChunk ? n - c0 : (size_t)kChunk;
		__syncthreads();
		for (size_t i = threadIdx.x; i < cn; i += kThreads)
			s_key[i] = GT<T>::key(in[c0 + i]);
		__syncthreads();
		for (size_t i = 0; i < cn; ++i) {
			C ki = s_key[i];
			size_t gi = c0 + i;
#pragma unroll
			for (int q = 0; q < kPer; ++q)
				pos[q] += (k[q] > ki) || ((ki == k[q]) && (gi < mine[q]));
		}
	}
#pragma unroll
	for (int q = 0; q < kPer; ++q) {
		if (!valid[q]) continue;
		out[pos[q]] = in[mine[q]];
		if (HAS_V) vout[pos[q]] = vin[mine[q]];
	}
}

template <typename T>
cudaError_t gselect_typed(const void *in, void *out, size_t n, const void *vin,
	void *vout, int vb, cudaStream_t s) {
	unsigned blocks = (unsigned)((n + kThreads * kPer - 1) / (kThreads * kPer));
	if (vb == 0)
		gselect_kernel<T, uint32_t, false><<<blocks, kThreads, 0, s>>>(
			(const T *)in, (T *)out, n, nullptr, nullptr);
	else if (vb == 4)
		gselect_kernel<T, uint32_t, true><<<blocks, kThreads, 0, s>>>(
			(const T *)in, (T *)out, n, (const uint32_t *)vin, (uint32_t *)vout);
	else
		gselect_kernel<T, uint64_t, true><<<blocks, kThreads, 0, s>>>(
			(const T *)in, (T *)out, n, (const uint64_t *)vin, (uint64_t *)vout);
	count_launches(1);
	return cudaGetLastError();
}

}  // namespace

cudaError_t gselect_sort(const void *in, void *out, size_t n, CloType type,
	const void *vals_in, void *vals_out, int val_bytes, CCLContext *ctx,
	cudaStream_t s, GError **err) {
	(void)ctx;
	if (n == 0) return cudaSuccess;
	cudaError_t e;
	switch (type) {
	case CLO_CHAR: e = gselect_typed<int8_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_UCHAR: e = gselect_typed<uint8_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_SHORT: e = gselect_typed<int16_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_USHORT: e = gselect_typed<uint16_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_INT: e = gselect_typed<int32_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_UINT: e = gselect_typed<uint32_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_LONG: e = gselect_typed<int64_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_ULONG: e = gselect_typed<uint64_t>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_HALF: e = gselect_typed<Half16>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_FLOAT: e = gselect_typed<float>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	case CLO_DOUBLE: e = gselect_typed<double>(in, out, n, vals_in, vals_out, val_bytes, s); break;
	default:
		set_error(err, CLO_ERROR_ARGS, "Unsupported element type %d", (int)type);
		return cudaErrorInvalidValue;
	}
	if (e != cudaSuccess) cuda_ok(e, err, "gselect");
	return e;
}

}  // namespace clo
