/*
 * TEST INFRASTRUCTURE -- CPU oracle for the cl_ops hot path.
 *
 * A plain-C restatement of the reference's algorithms, used only by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU baseline leg to
 * check (or time beside) the CUDA library. Nothing in the product links
 * or calls it. Each function cites the reference code it restates
 * (paths inside the FakenMC/cl-ops source tree).
 *
 * Type codes are the CloType values (0 char .. 10 double).
 */
#ifndef CLO_ORACLE_H
#define CLO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

/* Stable sort ascending by bits [0, sort_bits) of the unsigned key
 * (src/cl_ops/sort/clo_sort_satradix.c:117-335, clo_sort_satradix.cl).
 * Values (val_bytes 0, 4 or 8) follow their keys. In place. */
void oracle_radix_sort(void *keys, void *vals, size_t n, int key_bytes,
	int val_bytes, int sort_bits);

/* Bitonic network replay (src/cl_ops/sort/clo_sort_sbitonic.c:86-108 with
 * clo_sort_sbitonic.cl:38-69): stages 1..log2 N, steps s..1, swap iff
 * (key1 > key2) XOR desc. N = next power of two of n; the missing
 * elements are the type's maximum. In place. */
void oracle_bitonic_sort(void *data, size_t n, int type);
/* The same replay by `threads` host threads (identical results): steps
 * split by gid range, the short-stride steps of each stage run block by
 * block. For full-size checks. */
void oracle_bitonic_sort_threaded(void *data, size_t n, int type, int threads);

/* Rank-by-counting sort (src/cl_ops/sort/clo_sort_gselect.cl:38-57):
 * out[#{i : k_g > k_i || (k_i == k_g && i < g)}] = in[g]. */
void oracle_gselect_sort(const void *in, void *out, size_t n, int type,
	const void *vals_in, void *vals_out, int val_bytes);

/* Exclusive scan (src/cl_ops/scan/clo_scan_blelloch.cl:49-211 semantics;
 * the reference benchmark's serial check, clo_scan_bench.c:253-270):
 * out[i] = sum_{j<i} (SUM)in[j] modulo 2^(8 out_bytes). */
void oracle_scan(const void *in, void *out, size_t n, int in_type,
	int out_bytes);

/* DEV_GID seeds (src/cl_ops/rng/clo_rng_init.cl:47-60): hash_kind 0 =
 * none, 1 = KNUTH, 2 = XS1 (clo_rng_init.cl:27-33), then the generator's
 * ulong-to-state conversion. gen: 0 lcg, 1 xorshift64, 2 xorshift128,
 * 3 mwc64x, 4 parkmiller, 5 tauslcg. */
void oracle_rng_init_gid(void *states, size_t count, int gen,
	uint64_t main_seed, int hash_kind);

/* Draws (src/benchmarks/clo_rng_bench.cl:23-37 repeated `draws` times):
 * out[r * count + i] = next_i >> (32 - bits), or next_i % maxint. */
void oracle_rng_fill(void *states, size_t count, int gen, uint32_t *out,
	size_t draws, unsigned bits, unsigned maxint);

/* The LSD scheme of oracle_radix_sort for 32-bit keys with `bits`-bit
 * digits (4 or 8) on `threads` host threads (the timed CPU baseline). */
void oracle_radix_sort_u32_threaded(uint32_t *keys, size_t n, int threads,
	int bits);

/* First `nwords` outputs of MT19937 seeded with init_genrand(seed). */
void oracle_mt19937(uint32_t seed, uint32_t *out, size_t nwords);

/* splitmix64 stream (Steele, Lea, Flood 2014): the synthetic-input
 * generator of the tests and the benchmark. */
void oracle_splitmix64(uint64_t seed, uint64_t *out, size_t n);

/* Segmented forms: each segment [off[i], off[i+1]) (i < nseg) handled as
 * a separate oracle_radix_sort / oracle_scan call on it would handle it
 * -- i.e. as a separate clo_sort_with_device_data ("satradix",
 * src/cl_ops/sort/clo_sort_satradix.c:117-335) or clo_scan_with_device_data
 * ("blelloch", src/cl_ops/scan/clo_scan_blelloch.c:78-214) call on that
 * segment. Elements outside every segment are left alone. */
void oracle_seg_sort(void *keys, const uint64_t *off, size_t nseg, int key_bytes,
	int sort_bits);
void oracle_seg_scan(const void *in, void *out, const uint64_t *off, size_t nseg,
	int in_type, int out_bytes);

#endif
