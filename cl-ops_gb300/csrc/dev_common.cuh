// Device helpers shared by the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace clo {
namespace dev {

__device__ __forceinline__ uint32_t lanemask_lt() {
	uint32_t m;
	asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}

// Relaxed accesses at GPU scope for the lookback status words (each word
// carries its own ready bits, so no ordering beyond the word is needed).
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p) {
	uint32_t v;
	asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t *p) {
	uint64_t v;
	asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
	return v;
}
__device__ __forceinline__ void st_relaxed_u32(uint32_t *p, uint32_t v) {
	asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t *p, uint64_t v) {
	asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

// Streaming (evict-first) 16-byte load/store for data touched once.
__device__ __forceinline__ uint4 ld_stream_v4(const uint4 *p) {
	uint4 v;
	asm volatile("ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];"
		: "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
	return v;
}
__device__ __forceinline__ void st_stream_v4(uint4 *p, uint4 v) {
	asm volatile("st.global.cs.v4.u32 [%0], {%1,%2,%3,%4};"
		:: "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w) : "memory");
}

// 32-byte vector load/store (eight 32-bit words; 32-byte aligned address).
__device__ __forceinline__ void ld_v8(const void *p, uint32_t (&w)[8]) {
	asm volatile("ld.global.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
		: "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]),
		  "=r"(w[6]), "=r"(w[7]) : "l"(p));
}
__device__ __forceinline__ void st_v8(void *p, const uint32_t (&w)[8]) {
	asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
		:: "l"(p), "r"(w[0]), "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]),
		   "r"(w[6]), "r"(w[7]) : "memory");
}

// Spin budget of every bounded wait: with the nanosleep back-off below and
// the re-read of the flag each round this is about a second of waiting
// before a wait gives up.
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ __forceinline__ void backoff(uint32_t iter) {
	if (iter > 8) __nanosleep(iter < 64 ? 64 : 256);
}

// Records a watchdog failure (first writer wins) in the context's status.
__device__ __forceinline__ void report_timeout(int *status, int code,
	int detail) {
	if (atomicCAS(status, 0, code) == 0) atomicExch(status + 1, detail);
}

// ---------------------------------------------------------------- bulk copies
// One-dimensional bulk copies global -> shared (the copy engine, not the
// load/store pipe), completing on a CTA-local mbarrier. Addresses 16-byte
// aligned, sizes multiples of 16 bytes. No multicast.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
	return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count)
		: "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
		:: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
	uint64_t *bar) {
	asm volatile(
		"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
		:: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
	return ok != 0;
}
// Waits for phase `parity` of the barrier with a bounded number of tries;
// false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
	for (uint32_t iter = 0; iter < kSpinLimit; ++iter) {
		if (mbar_try_wait(bar, parity)) return true;
		backoff(iter);
	}
	return false;
}

// old = atomicAdd(p, v) on shared memory for the lanes where `pred` holds,
// as a predicated instruction (no branch around it).
__device__ __forceinline__ uint32_t atomic_add_shared_if(bool pred, uint32_t *p,
	uint32_t v) {
	uint32_t old = 0;
	const uint32_t addr = (uint32_t)__cvta_generic_to_shared(p);
	asm volatile(
		"{\n\t.reg .pred q;\n\t"
		"setp.ne.u32 q, %1, 0;\n\t"
		"@q atom.shared.add.u32 %0, [%2], %3;\n\t}"
		: "+r"(old) : "r"((uint32_t)pred), "r"(addr), "r"(v) : "memory");
	return old;
}

// Stable rank of a key among the lanes of its warp holding the same digit
// `d` in this round, and the warp's run position for it: peers are found
// through a shared-memory OR into match[d] (cleared again by the lowest
// peer), the lowest peer advances the warp's counter hist[d] by the number
// of peers, and the counter's old value reaches the peers by shuffle.
// Returns the key's position (old counter + lanes below it with d).
__device__ __forceinline__ uint32_t warp_rank_digit(uint32_t *match, uint32_t *hist,
	uint32_t d, uint32_t lane, uint32_t lt) {
	atomicOr(match + d, 1u << lane);
	__syncwarp();
	const uint32_t peers = match[d];
	__syncwarp();
	const uint32_t below = __popc(peers & lt);
	uint32_t start = atomic_add_shared_if(below == 0, hist + d, __popc(peers));
	if (below == 0) match[d] = 0;
	start = __shfl_sync(0xffffffffu, start, __ffs(peers) - 1);
	__syncwarp();
	return start + below;
}

// Stable rank of a key within its half-warp unit (16 lanes) for one round:
// w is the unit's word for the key's digit (next position << 16 | peer
// mask). Lanes OR in their bit and read the word back; the lowest peer
// stores the advanced position with the mask cleared. Returns the key's
// position.
__device__ __forceinline__ uint32_t unit_rank_digit(uint32_t *w, uint32_t l16,
	uint32_t lt16) {
	atomicOr(w, 1u << l16);
	__syncwarp();
	const uint32_t v = *w;
	__syncwarp();
	const uint32_t peers = v & 0xFFFFu;
	const uint32_t below = __popc(peers & lt16);
	if (below == 0) *w = (v & 0xFFFF0000u) + ((uint32_t)__popc(peers) << 16);
	__syncwarp();
	return (v >> 16) + below;
}

}  // namespace dev
}  // namespace clo
