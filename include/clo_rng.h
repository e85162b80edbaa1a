/*
 * cl_ops on GB300 -- pseudo-random number generators.
 *
 * Same entry points as the reference's src/cl_ops/rng/clo_rng.in.h:50-111.
 * A CloRng owns a device buffer of per-work-item generator states. The
 * reference hands client kernels OpenCL source (clo_rng_get_source); here
 * client CUDA kernels include "clo_rng_device.cuh", and
 * clo_rng_get_source returns that header's text. The batched draw kernel
 * the reference runs from its benchmark (src/benchmarks/clo_rng_bench.cl)
 * is exported as clo_rng_fill in clo_gb300.h.
 *
 * Generators and seed sizes (clo_rng.c:60-68): lcg 8, xorshift64 8,
 * xorshift128 16, mwc64x 8, parkmiller 4, tauslcg 16 bytes.
 */
#ifndef CLO_RNG_H
#define CLO_RNG_H

#include "clo_common.h"
#include "ccl_shim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CLO_RNG_IMPLS "lcg, xorshift64, xorshift128, mwc64x, parkmiller, tauslcg"

/* clo_rng.in.h:50-63 -- `src` holds the device source text of the
 * generator (a CUDA header fragment here). */
struct clo_rng_info {
	const char *name;
	const char *src;
	const size_t seed_size;
};

/* clo_rng.c:60-68 -- NULL-terminated. */
extern const struct clo_rng_info clo_rng_infos[];

/* clo_rng.in.h:78-92 */
typedef enum clo_rng_seed_type {
	CLO_RNG_SEED_DEV_GID = 0,
	CLO_RNG_SEED_HOST_MT = 1,
	CLO_RNG_SEED_EXT_DEV = 2,
	CLO_RNG_SEED_EXT_HOST = 3
} CloRngSeedType;

/* clo_rng.c:262 -- DEV_GID: state i = convert(hash(i + main_seed));
 * `hash` is the reference's macro body over `x` (NULL/""/"x": none,
 * "KNUTH(x)", "XS1(x)", or C statements assigning x from integer
 * expressions). HOST_MT: MT19937 seeded with (uint32)main_seed fills the
 * state bytes 32 bits at a time. EXT_DEV: `seeds` is a CCLBuffer* holding
 * at least seeds_count states (referenced, not copied). EXT_HOST: `seeds`
 * points at seeds_count raw states in host memory (copied). */
CloRng *clo_rng_new(const char *type, CloRngSeedType seed_type,
	void *seeds, size_t seeds_count, cl_ulong main_seed,
	const char *hash, CCLContext *ctx, CCLQueue *cq, GError **err);

void clo_rng_destroy(CloRng *rng);

/* clo_rng.c:439 -- device source for client kernels. */
const char *clo_rng_get_source(CloRng *rng);

/* clo_rng.c:452 -- the state buffer. */
CCLBuffer *clo_rng_get_device_seeds(CloRng *rng);

/* clo_rng.c:465 -- state buffer size in bytes. */
size_t clo_rng_get_size(CloRng *rng);

#ifdef __cplusplus
}
#endif

#endif /* CLO_RNG_H */
