/*
 * cl_ops on GB300 -- device-side generator API for client CUDA kernels.
 *
 * CUDA counterpart of the OpenCL source the reference hands to client
 * kernels through clo_rng_get_source(): src/cl_ops/rng/clo_rng_workitem.cl,
 * clo_rng_api.cl and one of clo_rng_{lcg,xorshift64,xorshift128,mwc64x,
 * parkmiller,tauslcg}.cl. Select the generator with one of
 *   CLO_RNG_LCG, CLO_RNG_XORSHIFT64, CLO_RNG_XORSHIFT128, CLO_RNG_MWC64X,
 *   CLO_RNG_PARKMILLER, CLO_RNG_TAUSLCG
 * before including this header (clo_rng_get_source() returns the text
 * with that definition prepended). Without a selection only the
 * per-generator step functions are declared.
 *
 * State layouts match the reference's clo_statetype, byte for byte, so a
 * state buffer can be filled on the host exactly as for the reference:
 *   lcg, xorshift64  uint64
 *   xorshift128      uint4 {x, y, z, w}
 *   mwc64x           uint2 {x = multiplier state, y = carry}
 *   parkmiller       int32
 *   tauslcg          uint4 {x, y, z, w}
 */
#ifndef CLO_RNG_DEVICE_CUH
#define CLO_RNG_DEVICE_CUH

#ifdef __CUDACC_RTC__
/* NVRTC (a client program built with ccl_program_build) has no C library
 * headers: the fixed-width types it needs here. */
typedef unsigned char uint8_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
#else
#include <stdint.h>
#endif

#define CLO_RNG_HD __host__ __device__ __forceinline__

/* ---- per-generator steps: advance the state, return the 32-bit draw ---- */

/* clo_rng_lcg.cl:43-59 -- 48-bit LCG (Java Random constants). */
CLO_RNG_HD uint32_t clo_rng_step_lcg(uint64_t *s) {
	uint64_t v = (*s * 0x5DEECE66DULL + 0xBULL) & ((1ULL << 48) - 1ULL);
	*s = v;
	return (uint32_t)(v >> 16);
}

/* clo_rng_xorshift64.cl:40-63 -- shifts 21, 35, 4; low 32 bits out. */
CLO_RNG_HD uint32_t clo_rng_step_xorshift64(uint64_t *s) {
	uint64_t v = *s;
	v ^= v << 21;
	v ^= v >> 35;
	v ^= v << 4;
	*s = v;
	return (uint32_t)v;
}

/* clo_rng_xorshift128.cl:41-59 -- Marsaglia xorshift128, w out. */
CLO_RNG_HD uint32_t clo_rng_step_xorshift128(uint4 *s) {
	uint32_t t = s->x ^ (s->x << 11);
	s->x = s->y;
	s->y = s->z;
	s->z = s->w;
	s->w = s->w ^ (s->w >> 19) ^ (t ^ (t >> 8));
	return s->w;
}

/* clo_rng_mwc64x.cl:43-63 -- multiply-with-carry, A = 4294883355; the
 * output is taken before the step. */
CLO_RNG_HD uint32_t clo_rng_step_mwc64x(uint2 *s) {
	const uint32_t A = 4294883355u;
	uint32_t x = s->x, c = s->y;
	uint32_t res = x ^ c;
	uint32_t hi = (uint32_t)(((uint64_t)x * A) >> 32);
	x = x * A + c;
	c = hi + (x < c);
	s->x = x;
	s->y = c;
	return res;
}

/* clo_rng_parkmiller.cl:43-59 -- minimal standard, a = 16807,
 * m = 2^31 - 1, with C's truncating signed remainder; output shifted left
 * by one. */
CLO_RNG_HD uint32_t clo_rng_step_parkmiller(int32_t *s) {
	// p = s * 16807; |p| = |s| * 16807 < 2^46 as one 32x32->64 product.
	// |p| mod (2^31 - 1) by folding (2^31 = 1 modulo 2^31 - 1):
	// a*2^31 + b = a + b, in 32 bits, then at most one subtraction. The
	// sign follows the dividend (the sign of s), as C's truncating % does.
	const int32_t x = *s;
	const uint32_t a = x < 0 ? 0u - (uint32_t)x : (uint32_t)x;
	const uint64_t w = (uint64_t)a * 16807u;
	const uint32_t lo = (uint32_t)w, hi = (uint32_t)(w >> 32);
	uint32_t q = (lo & 0x7FFFFFFFu) + ((hi << 1) | (lo >> 31));
	if (q >= 0x7FFFFFFFu) q -= 0x7FFFFFFFu;
	const int32_t v = x < 0 ? -(int32_t)q : (int32_t)q;
	*s = v;
	return ((uint32_t)v) << 1;
}

/* clo_rng_tauslcg.cl:52-100 -- three Tausworthe steps fed from y, z, w
 * plus an LCG on the old x; returns the new x. */
CLO_RNG_HD uint32_t clo_rng_taus_step(uint32_t z, int s1, int s2, int s3,
	uint32_t m) {
	uint32_t b = (((z << s1) ^ z) >> s2);
	return (((z & m) << s3) ^ b);
}
CLO_RNG_HD uint32_t clo_rng_step_tauslcg(uint4 *s) {
	uint32_t x = s->x;
	s->x = clo_rng_taus_step(s->y, 13, 19, 12, 4294967294u);
	s->y = clo_rng_taus_step(s->z, 2, 25, 4, 4294967288u);
	s->z = clo_rng_taus_step(s->w, 3, 11, 17, 4294967294u);
	s->w = 1664525u * x + 1013904223u;
	return s->x;
}

/* ---- client API (clo_rng_api.cl:33-105, clo_rng_workitem.cl:24-32):
 * next_int, next_int2, next_int4, next_int8 ---- */
#if defined(CLO_RNG_LCG)
typedef uint64_t clo_statetype;
#define CLO_RNG_STEP clo_rng_step_lcg
#elif defined(CLO_RNG_XORSHIFT64)
typedef uint64_t clo_statetype;
#define CLO_RNG_STEP clo_rng_step_xorshift64
#elif defined(CLO_RNG_XORSHIFT128)
typedef uint4 clo_statetype;
#define CLO_RNG_STEP clo_rng_step_xorshift128
#elif defined(CLO_RNG_MWC64X)
typedef uint2 clo_statetype;
#define CLO_RNG_STEP clo_rng_step_mwc64x
#elif defined(CLO_RNG_PARKMILLER)
typedef int32_t clo_statetype;
#define CLO_RNG_STEP clo_rng_step_parkmiller
#elif defined(CLO_RNG_TAUSLCG)
typedef uint4 clo_statetype;
#define CLO_RNG_STEP clo_rng_step_tauslcg
#endif

#ifdef CLO_RNG_STEP
#ifdef __CUDACC__
/* Flattened 1-D global id and size, as OpenCL's get_global_id(0). */
__device__ __forceinline__ uint32_t clo_rng_gid(void) {
	return blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ uint32_t clo_rng_global_size(void) {
	return gridDim.x * blockDim.x;
}

/* Next draw from state `index` (read-modify-write in global memory). */
__device__ __forceinline__ uint32_t clo_rng_next(clo_statetype *states,
	uint32_t index) {
	clo_statetype s = states[index];
	uint32_t r = CLO_RNG_STEP(&s);
	states[index] = s;
	return r;
}

/* next % n from the work-item's own state. */
__device__ __forceinline__ uint32_t clo_rng_next_int(clo_statetype *states,
	uint32_t n) {
	return clo_rng_next(states, clo_rng_gid()) % n;
}

/* Vector forms: lane k uses state k * global_size + gid. */
__device__ __forceinline__ uint2 clo_rng_next_int2(clo_statetype *states,
	uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	return make_uint2(clo_rng_next(states, g) % n,
		clo_rng_next(states, w + g) % n);
}

__device__ __forceinline__ uint4 clo_rng_next_int4(clo_statetype *states,
	uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	return make_uint4(clo_rng_next(states, g) % n,
		clo_rng_next(states, w + g) % n, clo_rng_next(states, 2 * w + g) % n,
		clo_rng_next(states, 3 * w + g) % n);
}

/* OpenCL's uint8 (eight uints, .s0 - .s7); CUDA has no 8-wide vector. */
typedef struct {
	uint32_t s0, s1, s2, s3, s4, s5, s6, s7;
} clo_uint8;

__device__ __forceinline__ clo_uint8 clo_rng_next_int8(clo_statetype *states,
	uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	clo_uint8 r;
	r.s0 = clo_rng_next(states, g) % n;
	r.s1 = clo_rng_next(states, w + g) % n;
	r.s2 = clo_rng_next(states, 2 * w + g) % n;
	r.s3 = clo_rng_next(states, 3 * w + g) % n;
	r.s4 = clo_rng_next(states, 4 * w + g) % n;
	r.s5 = clo_rng_next(states, 5 * w + g) % n;
	r.s6 = clo_rng_next(states, 6 * w + g) % n;
	r.s7 = clo_rng_next(states, 7 * w + g) % n;
	return r;
}
#endif /* __CUDACC__ */
#endif /* CLO_RNG_STEP */

#endif /* CLO_RNG_DEVICE_CUH */
