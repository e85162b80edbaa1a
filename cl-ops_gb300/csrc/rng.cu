// RNG kernels: DEV_GID seed initialisation and the batched draw ("fill").
//
// Seed init (src/cl_ops/rng/clo_rng_init.cl:47-60): state[gid] =
// convert(hash(gid + main_seed)) where `hash` is a compiled stack program
// (rng.cpp) and `convert` is the generator's clo_ulong2statetype:
// identity for lcg/xorshift64, (s, s>>16, s>>32, s>>46) masked to 32 bits
// for xorshift128 (clo_rng_xorshift128.cl:30), (low, high) words for
// mwc64x (clo_rng_mwc64x.cl:32), the low word as int for parkmiller
// (clo_rng_parkmiller.cl:31) and as_uint4((ulong2)(s, s)) for tauslcg
// (clo_rng_tauslcg.cl:35).
//
// Fill (the draw loop of src/benchmarks/clo_rng_bench.c:302-324 with the
// kernel of clo_rng_bench.cl:23-37, moved on device): out[r * count + i]
// = next(state i) >> (32 - bits), or % maxint, for r = 0..draws-1. Each
// thread keeps 4 consecutive states in registers for all draws and writes
// one 16-byte vector per draw, so the states are read and written once.
//
// HBM roofline: 4 B per draw + 2 x state size per state.
#include "clo_internal.h"
#include "clo_rng_device.cuh"
#include "dev_common.cuh"
#include "timing.h"

namespace clo {
namespace {

__device__ __forceinline__ uint64_t run_hash(const HashProgram &hp, uint64_t x) {
	uint64_t st[16];
	int sp = 0;
	for (int i = 0; i < hp.n_ops; ++i) {
		uint8_t op = hp.op[i];
		uint64_t a = 0, b = 0;
		if (op >= 4 && op != 14 && op != 15 && op != 16 && sp >= 2) {
			b = st[--sp];
			a = st[--sp];
		}
		switch (op) {
		case 0: if (sp < 16) st[sp++] = hp.imm[i]; break;     // IMM
		case 1: if (sp < 16) st[sp++] = x; break;             // X
		case 2: if (sp > 0) x = st[--sp]; break;              // STORE
		case 3: if (sp > 0) --sp; break;                      // POP
		case 4: st[sp++] = a + b; break;
		case 5: st[sp++] = a - b; break;
		case 6: st[sp++] = a * b; break;
		case 7: st[sp++] = b ? a / b : 0; break;
		case 8: st[sp++] = b ? a % b : 0; break;
		case 9: st[sp++] = a & b; break;
		case 10: st[sp++] = a | b; break;
		case 11: st[sp++] = a ^ b; break;
		case 12: st[sp++] = a << (b & 63); break;
		case 13: st[sp++] = a >> (b & 63); break;
		case 14: if (sp > 0) st[sp - 1] = 0 - st[sp - 1]; break;  // NEG
		case 15: if (sp > 0) st[sp - 1] = ~st[sp - 1]; break;     // NOT
		case 16: if (sp > 0) st[sp - 1] = !st[sp - 1]; break;     // LNOT
		case 17: st[sp++] = a == b; break;
		case 18: st[sp++] = a != b; break;
		case 19: st[sp++] = a < b; break;
		case 20: st[sp++] = a > b; break;
		case 21: st[sp++] = a <= b; break;
		case 22: st[sp++] = a >= b; break;
		case 23: st[sp++] = a && b; break;
		case 24: st[sp++] = a || b; break;
		}
	}
	return x;
}

__global__ void rng_init_kernel(void *states, size_t count, int gen,
	uint64_t main_seed, HashProgram hp) {
	size_t gid = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	if (gid >= count) return;
	// The reference adds the work-item id (a size_t) to the ulong seed.
	uint64_t seed = run_hash(hp, (uint64_t)gid + main_seed);
	switch (gen) {
	case RNG_LCG:
	case RNG_XS64:
		((uint64_t *)states)[gid] = seed;
		break;
	case RNG_XS128:
		((uint4 *)states)[gid] = make_uint4((uint32_t)seed, (uint32_t)(seed >> 16),
			(uint32_t)(seed >> 32), (uint32_t)(seed >> 46));
		break;
	case RNG_MWC64X:
		((uint2 *)states)[gid] = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
		break;
	case RNG_PARKMILLER:
		((int32_t *)states)[gid] = (int32_t)(uint32_t)seed;
		break;
	case RNG_TAUSLCG:
		((uint4 *)states)[gid] = make_uint4((uint32_t)seed, (uint32_t)(seed >> 32),
			(uint32_t)seed, (uint32_t)(seed >> 32));
		break;
	}
}

template <int GEN>
struct Gen;
template <>
struct Gen<RNG_LCG> {
	using S = uint64_t;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_lcg(&s); }
};
template <>
struct Gen<RNG_XS64> {
	using S = uint64_t;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_xorshift64(&s); }
};
template <>
struct Gen<RNG_XS128> {
	using S = uint4;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_xorshift128(&s); }
};
template <>
struct Gen<RNG_MWC64X> {
	using S = uint2;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_mwc64x(&s); }
};
template <>
struct Gen<RNG_PARKMILLER> {
	using S = int32_t;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_parkmiller(&s); }
};
template <>
struct Gen<RNG_TAUSLCG> {
	using S = uint4;
	__device__ __forceinline__ static uint32_t next(S &s) { return clo_rng_step_tauslcg(&s); }
};

constexpr int kFillThreads = 256;

// 4 consecutive states per thread; one uint4 store per draw.
template <int GEN, bool MAXINT>
__global__ void __launch_bounds__(kFillThreads)
rng_fill_kernel(typename Gen<GEN>::S *__restrict__ states, size_t count,
	uint32_t *__restrict__ out, size_t draws, uint32_t shift, uint32_t maxint,
	bool vec) {
	using S = typename Gen<GEN>::S;
	const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
	const size_t i0 = q * 4;
	if (i0 >= count) return;
	auto emit = [&](uint32_t v) -> uint32_t {
		return MAXINT ? v % maxint : (v >> shift);
	};
	if (vec) {
		S s0 = states[i0], s1 = states[i0 + 1], s2 = states[i0 + 2], s3 = states[i0 + 3];
		uint4 *o = reinterpret_cast<uint4 *>(out) + q;
		const size_t row = count / 4;
		for (size_t r = 0; r < draws; ++r) {
			uint4 v;
			v.x = emit(Gen<GEN>::next(s0));
			v.y = emit(Gen<GEN>::next(s1));
			v.z = emit(Gen<GEN>::next(s2));
			v.w = emit(Gen<GEN>::next(s3));
			dev::st_stream_v4(o + r * row, v);
		}
		states[i0] = s0;
		states[i0 + 1] = s1;
		states[i0 + 2] = s2;
		states[i0 + 3] = s3;
	} else {
		for (size_t i = i0; i < i0 + 4 && i < count; ++i) {
			S s = states[i];
			for (size_t r = 0; r < draws; ++r) out[r * count + i] = emit(Gen<GEN>::next(s));
			states[i] = s;
		}
	}
}

template <int GEN>
cudaError_t fill_gen(void *states, size_t count, uint32_t *out, size_t draws,
	unsigned bits, unsigned maxint, cudaStream_t s) {
	using S = typename Gen<GEN>::S;
	size_t threads = (count + 3) / 4;
	unsigned blocks = (unsigned)((threads + kFillThreads - 1) / kFillThreads);
	uint32_t shift = 32u - bits;
	// Whole rows of 16-byte stores need count % 4 == 0 and an aligned out.
	bool vec = (count % 4) == 0 && ((uintptr_t)out % 16) == 0;
	KernelTimer t("rng_fill", s, (double)count * (4.0 * draws + 2.0 * sizeof(S)));
	if (maxint)
		rng_fill_kernel<GEN, true><<<blocks, kFillThreads, 0, s>>>((S *)states, count,
			out, draws, shift, maxint, vec);
	else
		rng_fill_kernel<GEN, false><<<blocks, kFillThreads, 0, s>>>((S *)states, count,
			out, draws, shift, maxint, vec);
	t.stop();
	count_launches(1);
	return cudaGetLastError();
}

}  // namespace

cudaError_t rng_init_gid(void *states, size_t count, int gen,
	uint64_t main_seed, const HashProgram &hp, cudaStream_t s) {
	if (count == 0) return cudaSuccess;
	rng_init_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(states, count,
		gen, main_seed, hp);
	count_launches(1);
	return cudaGetLastError();
}

cudaError_t rng_fill(void *states, size_t count, int gen, uint32_t *out,
	size_t draws, unsigned bits, unsigned maxint, cudaStream_t s) {
	if (count == 0 || draws == 0) return cudaSuccess;
	switch (gen) {
	case RNG_LCG: return fill_gen<RNG_LCG>(states, count, out, draws, bits, maxint, s);
	case RNG_XS64: return fill_gen<RNG_XS64>(states, count, out, draws, bits, maxint, s);
	case RNG_XS128: return fill_gen<RNG_XS128>(states, count, out, draws, bits, maxint, s);
	case RNG_MWC64X: return fill_gen<RNG_MWC64X>(states, count, out, draws, bits, maxint, s);
	case RNG_PARKMILLER: return fill_gen<RNG_PARKMILLER>(states, count, out, draws, bits, maxint, s);
	case RNG_TAUSLCG: return fill_gen<RNG_TAUSLCG>(states, count, out, draws, bits, maxint, s);
	}
	return cudaErrorInvalidValue;
}

}  // namespace clo
