/*
 * TEST INFRASTRUCTURE -- CPU oracle for the cl_ops hot path.
 *
 * Plain-C restatement of the reference's sort, scan and RNG algorithms.
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU baseline use
 * it, as the checker; the library never links it. See clo_oracle.h for
 * the per-function reference citations.
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers under -std=c11 */
#include "clo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ helpers */

static uint64_t load_u(const void *p, int bytes) {
	uint64_t v = 0;
	memcpy(&v, p, (size_t)bytes); /* little-endian hosts (x86-64, aarch64) */
	return v;
}

/* Half (binary16) to float, exact, from the IEEE 754 field layout. */
static float half_to_float(uint16_t h) {
	int s = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
	float v;
	if (e == 0) v = ldexpf((float)m, -24);
	else if (e == 31) v = m ? NAN : INFINITY;
	else v = ldexpf((float)(m + 1024), e - 25);
	return s ? -v : v;
}

/* ------------------------------------------------ satradix (LSD, stable)
 * The reference sorts with log2(radix)-bit digits, least significant
 * first, each pass a stable split (clo_sort_satradix.cl:34-258); the
 * composition is a stable sort by the unsigned key. This restatement runs
 * the same LSD scheme with 4-bit digits (radix 16, the reference default,
 * clo_sort_satradix.c:353) as serial counting sorts. */
void oracle_radix_sort(void *keys, void *vals, size_t n, int kb, int vb,
	int sort_bits) {
	const int bits = 4, R = 1 << bits;
	if (n < 2) return;
	unsigned char *k0 = (unsigned char *)keys, *v0 = (unsigned char *)vals;
	unsigned char *k1 = malloc(n * (size_t)kb);
	unsigned char *v1 = vb ? malloc(n * (size_t)vb) : NULL;
	unsigned char *ks = k0, *kd = k1, *vs = v0, *vd = v1;
	size_t count[16];
	int passes = (sort_bits + bits - 1) / bits;
	for (int p = 0; p < passes; ++p) {
		int shift = p * bits;
		memset(count, 0, sizeof count);
		for (size_t i = 0; i < n; ++i)
			count[(load_u(ks + i * kb, kb) >> shift) & (R - 1)]++;
		size_t sum = 0;
		for (int d = 0; d < R; ++d) {
			size_t c = count[d];
			count[d] = sum;
			sum += c;
		}
		for (size_t i = 0; i < n; ++i) {
			size_t o = count[(load_u(ks + i * kb, kb) >> shift) & (R - 1)]++;
			memcpy(kd + o * kb, ks + i * kb, (size_t)kb);
			if (vb) memcpy(vd + o * vb, vs + i * vb, (size_t)vb);
		}
		unsigned char *t = ks; ks = kd; kd = t;
		t = vs; vs = vd; vd = t;
	}
	if (ks != k0) {
		memcpy(k0, ks, n * (size_t)kb);
		if (vb) memcpy(v0, vs, n * (size_t)vb);
	}
	free(k1);
	free(v1);
}

/* ------------------------------------------------------------ bitonic */
#define DEFINE_BITONIC(NAME, T, GT, MAXV)                                  \
	static void NAME(T *a, size_t n) {                                       \
		size_t N = 1;                                                        \
		int logN = 0;                                                        \
		while (N < n) { N <<= 1; logN++; }                                   \
		T *d = a;                                                            \
		if (N != n) {                                                        \
			d = malloc(N * sizeof(T));                                       \
			memcpy(d, a, n * sizeof(T));                                     \
			for (size_t i = n; i < N; ++i) d[i] = (MAXV);                    \
		}                                                                    \
		for (int stage = 1; stage <= logN; ++stage)                          \
			for (int step = stage; step >= 1; --step) {                      \
				size_t stride = (size_t)1 << (step - 1);                     \
				for (size_t gid = 0; gid < N / 2; ++gid) {                   \
					size_t i1 = gid + (gid / stride) * stride;               \
					size_t i2 = i1 + stride;                                 \
					int desc = (int)((gid >> (stage - 1)) & 1);              \
					T x = d[i1], y = d[i2];                                  \
					if ((GT(x, y) ? 1 : 0) ^ desc) { d[i1] = y; d[i2] = x; } \
				}                                                            \
			}                                                                \
		if (d != a) {                                                        \
			memcpy(a, d, n * sizeof(T));                                     \
			free(d);                                                         \
		}                                                                    \
	}

#define PLAIN_GT(x, y) ((x) > (y))
#define HALF_GT(x, y) (half_to_float(x) > half_to_float(y))
DEFINE_BITONIC(bit_i8, int8_t, PLAIN_GT, INT8_MAX)
DEFINE_BITONIC(bit_u8, uint8_t, PLAIN_GT, UINT8_MAX)
DEFINE_BITONIC(bit_i16, int16_t, PLAIN_GT, INT16_MAX)
DEFINE_BITONIC(bit_u16, uint16_t, PLAIN_GT, UINT16_MAX)
DEFINE_BITONIC(bit_i32, int32_t, PLAIN_GT, INT32_MAX)
DEFINE_BITONIC(bit_u32, uint32_t, PLAIN_GT, UINT32_MAX)
DEFINE_BITONIC(bit_i64, int64_t, PLAIN_GT, INT64_MAX)
DEFINE_BITONIC(bit_u64, uint64_t, PLAIN_GT, UINT64_MAX)
DEFINE_BITONIC(bit_f16, uint16_t, HALF_GT, 0x7c00)
DEFINE_BITONIC(bit_f32, float, PLAIN_GT, INFINITY)
DEFINE_BITONIC(bit_f64, double, PLAIN_GT, INFINITY)

/* The same network replayed by host threads, for full-size checks. A step
 * is N/2 independent compare-exchanges, split over the threads by gid
 * range; once a stage's stride is below half a block of kBitBlock
 * elements, every remaining step of the stage pairs elements inside
 * aligned blocks, so each thread runs those steps block by block (a
 * block's gids are [b B/2, (b + 1) B/2)). Every pair is compared in the
 * same step order as the serial replay, so the results are identical. */
#define DEFINE_BITONIC_STEP(NAME, T, GT, MAXV)                               \
	static void NAME##_step(void *dv, size_t glo, size_t ghi, int stage,      \
		int step) {                                                           \
		T *d = dv;                                                            \
		size_t stride = (size_t)1 << (step - 1);                              \
		for (size_t gid = glo; gid < ghi; ++gid) {                            \
			size_t i1 = gid + (gid / stride) * stride;                        \
			size_t i2 = i1 + stride;                                          \
			int desc = (int)((gid >> (stage - 1)) & 1);                       \
			T x = d[i1], y = d[i2];                                           \
			if ((GT(x, y) ? 1 : 0) ^ desc) { d[i1] = y; d[i2] = x; }          \
		}                                                                     \
	}                                                                         \
	static void NAME##_pad(void *dv, size_t from, size_t to) {               \
		T *d = dv;                                                            \
		for (size_t i = from; i < to; ++i) d[i] = (MAXV);                     \
	}
DEFINE_BITONIC_STEP(bit_i8, int8_t, PLAIN_GT, INT8_MAX)
DEFINE_BITONIC_STEP(bit_u8, uint8_t, PLAIN_GT, UINT8_MAX)
DEFINE_BITONIC_STEP(bit_i16, int16_t, PLAIN_GT, INT16_MAX)
DEFINE_BITONIC_STEP(bit_u16, uint16_t, PLAIN_GT, UINT16_MAX)
DEFINE_BITONIC_STEP(bit_i32, int32_t, PLAIN_GT, INT32_MAX)
DEFINE_BITONIC_STEP(bit_u32, uint32_t, PLAIN_GT, UINT32_MAX)
DEFINE_BITONIC_STEP(bit_i64, int64_t, PLAIN_GT, INT64_MAX)
DEFINE_BITONIC_STEP(bit_u64, uint64_t, PLAIN_GT, UINT64_MAX)
DEFINE_BITONIC_STEP(bit_f16, uint16_t, HALF_GT, 0x7c00)
DEFINE_BITONIC_STEP(bit_f32, float, PLAIN_GT, INFINITY)
DEFINE_BITONIC_STEP(bit_f64, double, PLAIN_GT, INFINITY)

typedef void (*BitStepFn)(void *, size_t, size_t, int, int);
typedef void (*BitPadFn)(void *, size_t, size_t);
static const BitStepFn kBitStep[11] = {bit_i8_step, bit_u8_step, bit_i16_step,
	bit_u16_step, bit_i32_step, bit_u32_step, bit_i64_step, bit_u64_step, bit_f16_step,
	bit_f32_step, bit_f64_step};
static const BitPadFn kBitPad[11] = {bit_i8_pad, bit_u8_pad, bit_i16_pad, bit_u16_pad,
	bit_i32_pad, bit_u32_pad, bit_i64_pad, bit_u64_pad, bit_f16_pad, bit_f32_pad,
	bit_f64_pad};
static const int kBitSize[11] = {1, 1, 2, 2, 4, 4, 8, 8, 2, 4, 8};
#define kBitBlock ((size_t)1 << 14)

typedef struct {
	void *d;
	size_t N, B;
	int logN, t, threads;
	BitStepFn step;
	pthread_barrier_t *bar;
} BitJob;

static void *bitonic_job(void *arg) {
	BitJob *j = arg;
	const size_t half = j->N / 2, T = (size_t)j->threads, t = (size_t)j->t;
	const size_t blocks = j->N / j->B;
	for (int stage = 1; stage <= j->logN; ++stage) {
		int step = stage;
		for (; step >= 1 && ((size_t)1 << step) > j->B; --step) {
			j->step(j->d, half * t / T, half * (t + 1) / T, stage, step);
			pthread_barrier_wait(j->bar);
		}
		if (step >= 1) {
			for (size_t b = blocks * t / T; b < blocks * (t + 1) / T; ++b)
				for (int s = step; s >= 1; --s)
					j->step(j->d, b * (j->B / 2), (b + 1) * (j->B / 2), stage, s);
			pthread_barrier_wait(j->bar);
		}
	}
	return NULL;
}

void oracle_bitonic_sort_threaded(void *data, size_t n, int type, int threads) {
	if (n < 2 || type < 0 || type > 10) return;
	if (threads < 1) threads = 1;
	if (threads > 256) threads = 256;
	const size_t es = (size_t)kBitSize[type];
	size_t N = 1;
	int logN = 0;
	while (N < n) { N <<= 1; logN++; }
	unsigned char *d = data;
	if (N != n) {
		d = malloc(N * es);
		memcpy(d, data, n * es);
		kBitPad[type](d, n, N);
	}
	pthread_barrier_t bar;
	pthread_barrier_init(&bar, NULL, (unsigned)threads);
	BitJob jobs[256];
	pthread_t th[256];
	for (int t = 0; t < threads; ++t) {
		jobs[t].d = d;
		jobs[t].N = N;
		jobs[t].B = N < kBitBlock ? N : kBitBlock;
		jobs[t].logN = logN;
		jobs[t].t = t;
		jobs[t].threads = threads;
		jobs[t].step = kBitStep[type];
		jobs[t].bar = &bar;
		if (t > 0) pthread_create(&th[t], NULL, bitonic_job, &jobs[t]);
	}
	bitonic_job(&jobs[0]);
	for (int t = 1; t < threads; ++t) pthread_join(th[t], NULL);
	pthread_barrier_destroy(&bar);
	if (d != (unsigned char *)data) {
		memcpy(data, d, n * es);
		free(d);
	}
}

void oracle_bitonic_sort(void *data, size_t n, int type) {
	if (n < 2) return;
	switch (type) {
	case 0: bit_i8(data, n); break;
	case 1: bit_u8(data, n); break;
	case 2: bit_i16(data, n); break;
	case 3: bit_u16(data, n); break;
	case 4: bit_i32(data, n); break;
	case 5: bit_u32(data, n); break;
	case 6: bit_i64(data, n); break;
	case 7: bit_u64(data, n); break;
	case 8: bit_f16(data, n); break;
	case 9: bit_f32(data, n); break;
	case 10: bit_f64(data, n); break;
	}
}

/* ------------------------------------------------------------ gselect */
#define DEFINE_GSELECT(NAME, T, KEY, KT)                                     \
	static void NAME(const T *in, T *out, size_t n, const unsigned char *vin, \
		unsigned char *vout, int vb) {                                        \
		for (size_t g = 0; g < n; ++g) {                                      \
			KT kg = KEY(in[g]);                                               \
			size_t pos = 0;                                                   \
			for (size_t i = 0; i < n; ++i) {                                  \
				KT ki = KEY(in[i]);                                           \
				if ((kg > ki) || ((ki == kg) && (i < g))) pos++;              \
			}                                                                 \
			out[pos] = in[g];                                                 \
			if (vb) memcpy(vout + pos * vb, vin + g * vb, (size_t)vb);        \
		}                                                                     \
	}
#define ID_KEY(x) (x)
DEFINE_GSELECT(gs_i8, int8_t, ID_KEY, int8_t)
DEFINE_GSELECT(gs_u8, uint8_t, ID_KEY, uint8_t)
DEFINE_GSELECT(gs_i16, int16_t, ID_KEY, int16_t)
DEFINE_GSELECT(gs_u16, uint16_t, ID_KEY, uint16_t)
DEFINE_GSELECT(gs_i32, int32_t, ID_KEY, int32_t)
DEFINE_GSELECT(gs_u32, uint32_t, ID_KEY, uint32_t)
DEFINE_GSELECT(gs_i64, int64_t, ID_KEY, int64_t)
DEFINE_GSELECT(gs_u64, uint64_t, ID_KEY, uint64_t)
DEFINE_GSELECT(gs_f16, uint16_t, half_to_float, float)
DEFINE_GSELECT(gs_f32, float, ID_KEY, float)
DEFINE_GSELECT(gs_f64, double, ID_KEY, double)

void oracle_gselect_sort(const void *in, void *out, size_t n, int type,
	const void *vin, void *vout, int vb) {
	const unsigned char *vi = vin;
	unsigned char *vo = vout;
	switch (type) {
	case 0: gs_i8(in, out, n, vi, vo, vb); break;
	case 1: gs_u8(in, out, n, vi, vo, vb); break;
	case 2: gs_i16(in, out, n, vi, vo, vb); break;
	case 3: gs_u16(in, out, n, vi, vo, vb); break;
	case 4: gs_i32(in, out, n, vi, vo, vb); break;
	case 5: gs_u32(in, out, n, vi, vo, vb); break;
	case 6: gs_i64(in, out, n, vi, vo, vb); break;
	case 7: gs_u64(in, out, n, vi, vo, vb); break;
	case 8: gs_f16(in, out, n, vi, vo, vb); break;
	case 9: gs_f32(in, out, n, vi, vo, vb); break;
	case 10: gs_f64(in, out, n, vi, vo, vb); break;
	}
}

/* --------------------------------------------------------------- scan */
void oracle_scan(const void *in, void *out, size_t n, int in_type,
	int out_bytes) {
	static const int sizes[] = {1, 1, 2, 2, 4, 4, 8, 8};
	int ib = sizes[in_type];
	int is_signed = (in_type % 2) == 0;
	uint64_t mask = out_bytes == 8 ? ~0ull : ((1ull << (8 * out_bytes)) - 1);
	uint64_t acc = 0;
	const unsigned char *src = in;
	unsigned char *dst = out;
	for (size_t i = 0; i < n; ++i) {
		uint64_t o = acc & mask;
		memcpy(dst + i * out_bytes, &o, (size_t)out_bytes);
		uint64_t v = load_u(src + i * ib, ib);
		if (is_signed && ib < 8 && (v >> (8 * ib - 1)) & 1)
			v |= ~0ull << (8 * ib); /* C conversion sign-extends */
		acc += v;
	}
}

/* ---------------------------------------------------------------- RNG */
static const size_t kSeedSize[] = {8, 8, 16, 8, 4, 16};

static void to_state(void *states, size_t i, int gen, uint64_t s) {
	unsigned char *p = (unsigned char *)states + i * kSeedSize[gen];
	uint32_t w[4];
	int32_t pm;
	switch (gen) {
	case 0: case 1: memcpy(p, &s, 8); break;              /* ulong */
	case 2:                                               /* uint4 split */
		w[0] = (uint32_t)(s & 0xFFFFFFFFull);
		w[1] = (uint32_t)((s >> 16) & 0xFFFFFFFFull);
		w[2] = (uint32_t)((s >> 32) & 0xFFFFFFFFull);
		w[3] = (uint32_t)((s >> 46) & 0xFFFFFFFFull);
		memcpy(p, w, 16);
		break;
	case 3: memcpy(p, &s, 8); break;                      /* as_uint2 */
	case 4:                                               /* as_int(low) */
		pm = (int32_t)(uint32_t)(s & 0xFFFFFFFFull);
		memcpy(p, &pm, 4);
		break;
	case 5: memcpy(p, &s, 8); memcpy(p + 8, &s, 8); break; /* as_uint4(ulong2) */
	}
}

void oracle_rng_init_gid(void *states, size_t count, int gen,
	uint64_t main_seed, int hash_kind) {
	for (size_t i = 0; i < count; ++i) {
		uint64_t x = (uint64_t)i + main_seed;
		if (hash_kind == 1) {
			x = (x * 2654435761ull) % 0x100000000ull;
		} else if (hash_kind == 2) {
			x = ((x >> 16) ^ x) * 0x45d9f3bull;
			x = ((x >> 16) ^ x) * 0x45d9f3bull;
			x = ((x >> 16) ^ x);
		}
		to_state(states, i, gen, x);
	}
}

static uint32_t next_draw(unsigned char *p, int gen) {
	uint64_t s;
	uint32_t w[4], t, res;
	int32_t pm;
	switch (gen) {
	case 0: /* clo_rng_lcg.cl:43-59 */
		memcpy(&s, p, 8);
		s = (s * 0x5DEECE66Dull + 0xBull) & ((1ull << 48) - 1);
		memcpy(p, &s, 8);
		return (uint32_t)(s >> 16);
	case 1: /* clo_rng_xorshift64.cl:40-63 */
		memcpy(&s, p, 8);
		s ^= s << 21;
		s ^= s >> 35;
		s ^= s << 4;
		memcpy(p, &s, 8);
		return (uint32_t)s;
	case 2: /* clo_rng_xorshift128.cl:41-59 */
		memcpy(w, p, 16);
		t = w[0] ^ (w[0] << 11);
		w[0] = w[1];
		w[1] = w[2];
		w[2] = w[3];
		w[3] = w[3] ^ (w[3] >> 19) ^ (t ^ (t >> 8));
		memcpy(p, w, 16);
		return w[3];
	case 3: { /* clo_rng_mwc64x.cl:43-63 */
		memcpy(w, p, 8);
		uint32_t x = w[0], c = w[1];
		res = x ^ c;
		uint32_t hi = (uint32_t)(((uint64_t)x * 4294883355ull) >> 32);
		x = x * 4294883355u + c;
		c = hi + (x < c);
		w[0] = x;
		w[1] = c;
		memcpy(p, w, 8);
		return res;
	}
	case 4: /* clo_rng_parkmiller.cl:43-59 */
		memcpy(&pm, p, 4);
		pm = (int32_t)(((int64_t)pm * 16807) % 2147483647);
		memcpy(p, &pm, 4);
		return ((uint32_t)pm) << 1;
	case 5: { /* clo_rng_tauslcg.cl:52-100 */
		memcpy(w, p, 16);
		uint32_t x = w[0], z;
		z = w[1]; w[0] = (((z & 4294967294u) << 12) ^ (((z << 13) ^ z) >> 19));
		z = w[2]; w[1] = (((z & 4294967288u) << 4) ^ (((z << 2) ^ z) >> 25));
		z = w[3]; w[2] = (((z & 4294967294u) << 17) ^ (((z << 3) ^ z) >> 11));
		w[3] = 1664525u * x + 1013904223u;
		memcpy(p, w, 16);
		return w[0];
	}
	}
	return 0;
}

void oracle_rng_fill(void *states, size_t count, int gen, uint32_t *out,
	size_t draws, unsigned bits, unsigned maxint) {
	unsigned char *st = states;
	for (size_t r = 0; r < draws; ++r)
		for (size_t i = 0; i < count; ++i) {
			uint32_t v = next_draw(st + i * kSeedSize[gen], gen);
			out[r * count + i] = maxint ? v % maxint : (v >> (32 - bits));
		}
}

void oracle_mt19937(uint32_t seed, uint32_t *out, size_t nwords) {
	uint32_t mt[624];
	int mti;
	mt[0] = seed;
	for (mti = 1; mti < 624; ++mti)
		mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti;
	for (size_t k = 0; k < nwords; ++k) {
		if (mti >= 624) {
			for (int i = 0; i < 624; ++i) {
				uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
				mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
			}
			mti = 0;
		}
		uint32_t y = mt[mti++];
		y ^= y >> 11;
		y ^= (y << 7) & 0x9d2c5680u;
		y ^= (y << 15) & 0xefc60000u;
		y ^= y >> 18;
		out[k] = y;
	}
}

void oracle_splitmix64(uint64_t seed, uint64_t *out, size_t n) {
	uint64_t x = seed;
	for (size_t i = 0; i < n; ++i) {
		uint64_t z = (x += 0x9E3779B97F4A7C15ull);
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		out[i] = z ^ (z >> 31);
	}
}

/* ------------------------------------------- threaded CPU radix baseline
 * The same LSD scheme run by `threads` host threads with `bits`-bit digits
 * (4 = the reference's default radix 16, 8 passes; or 8): per-thread
 * digit counts, a serial prefix over (digit, thread), a stable scatter.
 * The timed CPU baseline of bench.py; results equal oracle_radix_sort. */
typedef struct {
	const uint32_t *src;
	uint32_t *dst;
	size_t lo, hi;
	int shift;
	int bits;
	size_t *count; /* 256 per thread */
	int phase;
} RadixJob;

static void *radix_job(void *arg) {
	RadixJob *j = arg;
	const uint32_t m = (1u << j->bits) - 1u;
	if (j->phase == 0) {
		memset(j->count, 0, 256 * sizeof(size_t));
		for (size_t i = j->lo; i < j->hi; ++i) j->count[(j->src[i] >> j->shift) & m]++;
	} else {
		for (size_t i = j->lo; i < j->hi; ++i) {
			uint32_t v = j->src[i];
			j->dst[j->count[(v >> j->shift) & m]++] = v;
		}
	}
	return NULL;
}

void oracle_radix_sort_u32_threaded(uint32_t *keys, size_t n, int threads,
	int bits) {
	if (bits != 4 && bits != 8) bits = 8;
	const int R = 1 << bits, passes = 32 / bits;
	if (threads < 1) threads = 1;
	if (threads > 256) threads = 256;
	uint32_t *tmp = malloc(n * sizeof(uint32_t));
	size_t *count = malloc((size_t)threads * 256 * sizeof(size_t));
	RadixJob jobs[256];
	pthread_t th[256];
	uint32_t *src = keys, *dst = tmp;
	for (int p = 0; p < passes; ++p) {
		for (int ph = 0; ph < 2; ++ph) {
			for (int t = 0; t < threads; ++t) {
				jobs[t].src = src;
				jobs[t].dst = dst;
				jobs[t].lo = n * (size_t)t / (size_t)threads;
				jobs[t].hi = n * (size_t)(t + 1) / (size_t)threads;
				jobs[t].shift = bits * p;
				jobs[t].bits = bits;
				jobs[t].count = count + (size_t)t * 256;
				jobs[t].phase = ph;
				pthread_create(&th[t], NULL, radix_job, &jobs[t]);
			}
			for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
			if (ph == 0) {
				size_t sum = 0;
				for (int d = 0; d < R; ++d)
					for (int t = 0; t < threads; ++t) {
						size_t c = count[(size_t)t * 256 + d];
						count[(size_t)t * 256 + d] = sum;
						sum += c;
					}
			}
		}
		uint32_t *x = src; src = dst; dst = x;
	}
	free(tmp);
	free(count);
}

void oracle_seg_sort(void *keys, const uint64_t *off, size_t nseg, int kb,
	int sort_bits) {
	for (size_t i = 0; i < nseg; ++i)
		oracle_radix_sort((unsigned char *)keys + off[i] * (size_t)kb, NULL,
			(size_t)(off[i + 1] - off[i]), kb, 0, sort_bits);
}

void oracle_seg_scan(const void *in, void *out, const uint64_t *off, size_t nseg,
	int in_type, int out_bytes) {
	static const int sizes[] = {1, 1, 2, 2, 4, 4, 8, 8};
	const int ib = sizes[in_type];
	for (size_t i = 0; i < nseg; ++i)
		oracle_scan((const unsigned char *)in + off[i] * (size_t)ib,
			(unsigned char *)out + off[i] * (size_t)out_bytes,
			(size_t)(off[i + 1] - off[i]), in_type, out_bytes);
}
