/*
 * Shared pieces of the benchmark programs (ports of the reference's
 * src/benchmarks/clo_{sort,scan,rng}_bench.c command lines): option
 * parsing helpers, a Mersenne Twister for host data (the reference draws
 * its data with GLib's GRand, an MT19937), per-type random values and
 * comparisons (clo_bench.c:30-200), and device timing with queue markers.
 */
#ifndef CLO_CLI_H
#define CLO_CLI_H

#include <float.h>
#include <limits.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cl_ops.h"

/* ---- MT19937 (Matsumoto & Nishimura 1998), init_genrand seeding ------ */
typedef struct {
	uint32_t mt[624];
	int mti;
} CliMt;

static void cli_mt_seed(CliMt *r, uint32_t seed) {
	r->mt[0] = seed;
	for (int i = 1; i < 624; ++i)
		r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
	r->mti = 624;
}

static uint32_t cli_mt_next(CliMt *r) {
	if (r->mti >= 624) {
		for (int k = 0; k < 624; ++k) {
			uint32_t y = (r->mt[k] & 0x80000000u) | (r->mt[(k + 1) % 624] & 0x7fffffffu);
			r->mt[k] = r->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
		}
		r->mti = 0;
	}
	uint32_t y = r->mt[r->mti++];
	y ^= y >> 11;
	y ^= (y << 7) & 0x9d2c5680u;
	y ^= (y << 15) & 0xefc60000u;
	y ^= y >> 18;
	return y;
}

/* Uniform double in [0, 1) from two 32-bit words. */
static double cli_mt_double(CliMt *r) {
	for (;;) {
		double v = cli_mt_next(r) * (1.0 / 4294967296.0);
		v = (v + cli_mt_next(r)) * (1.0 / 4294967296.0);
		if (v < 1.0) return v;
	}
}

/* Integer in [begin, end). */
static int64_t cli_mt_range(CliMt *r, int64_t begin, int64_t end) {
	uint64_t span = (uint64_t)(end - begin);
	return begin + (int64_t)(span ? (uint64_t)cli_mt_next(r) % span : 0);
}

/* One random element of `type` at `loc`, over the ranges of the
 * reference's clo_bench_rand (clo_bench.c:105-200). */
static void cli_rand(CliMt *r, CloType type, void *loc) {
	switch (type) {
	case CLO_CHAR: { int8_t v = (int8_t)cli_mt_range(r, SCHAR_MIN, SCHAR_MAX); memcpy(loc, &v, 1); break; }
	case CLO_UCHAR: { uint8_t v = (uint8_t)cli_mt_range(r, 0, UCHAR_MAX); memcpy(loc, &v, 1); break; }
	case CLO_SHORT: { int16_t v = (int16_t)cli_mt_range(r, SHRT_MIN, SHRT_MAX); memcpy(loc, &v, 2); break; }
	case CLO_USHORT: { uint16_t v = (uint16_t)cli_mt_range(r, 0, USHRT_MAX); memcpy(loc, &v, 2); break; }
	case CLO_INT: { int32_t v = (int32_t)cli_mt_range(r, INT_MIN, INT_MAX); memcpy(loc, &v, 4); break; }
	case CLO_UINT: { uint32_t v = (uint32_t)(cli_mt_double(r) * (double)UINT_MAX); memcpy(loc, &v, 4); break; }
	case CLO_LONG: {
		double d = cli_mt_double(r);
		int64_t v = (int64_t)(d * ((cli_mt_next(r) & 1u) ? (double)INT64_MIN : (double)INT64_MAX));
		memcpy(loc, &v, 8);
		break;
	}
	case CLO_ULONG: {
		double d = cli_mt_double(r) * 18446744073709549568.0;  /* largest double < 2^64 */
		uint64_t v = (uint64_t)d;
		memcpy(loc, &v, 8);
		break;
	}
	case CLO_FLOAT: { float v = (float)(FLT_MIN + cli_mt_double(r) * (FLT_MAX - FLT_MIN)); memcpy(loc, &v, 4); break; }
	case CLO_DOUBLE: { double v = DBL_MIN + cli_mt_double(r) * (DBL_MAX - DBL_MIN); memcpy(loc, &v, 8); break; }
	default: { uint16_t v = (uint16_t)cli_mt_next(r); memcpy(loc, &v, 2); break; }
	}
}

#define CLI_CMP(T, a, b) ((*(const T *)(a) > *(const T *)(b)) - (*(const T *)(a) < *(const T *)(b)))

/* Sign of a - b in the type's own order (clo_bench.c:30-75). */
static int cli_compare(CloType type, const void *a, const void *b) {
	switch (type) {
	case CLO_CHAR: return CLI_CMP(int8_t, a, b);
	case CLO_UCHAR: return CLI_CMP(uint8_t, a, b);
	case CLO_SHORT: return CLI_CMP(int16_t, a, b);
	case CLO_USHORT: return CLI_CMP(uint16_t, a, b);
	case CLO_INT: return CLI_CMP(int32_t, a, b);
	case CLO_UINT: return CLI_CMP(uint32_t, a, b);
	case CLO_LONG: return CLI_CMP(int64_t, a, b);
	case CLO_ULONG: return CLI_CMP(uint64_t, a, b);
	case CLO_FLOAT: return CLI_CMP(float, a, b);
	case CLO_DOUBLE: return CLI_CMP(double, a, b);
	default: return CLI_CMP(uint16_t, a, b);
	}
}

/* Long option table entry: name, short letter, takes a value. */
typedef struct {
	const char *name;
	char letter;
	int has_value;
	const char *help;
} CliOpt;

/* Parses argv against opts; calls set(letter, value) for each. Accepts
 * "-x VALUE", "-xVALUE", "--name VALUE" and "--name=VALUE". Returns 0, or
 * 1 after printing help (--help, or -h when no option takes that
 * letter), or -1 on an unknown option. */
static int cli_parse(int argc, char **argv, const CliOpt *opts, const char *usage,
	void (*set)(char, const char *)) {
	for (int i = 1; i < argc; ++i) {
		const char *a = argv[i];
		const CliOpt *o = NULL;
		const char *val = NULL;
		int h_taken = 0;
		for (const CliOpt *p = opts; p->name; ++p) h_taken |= p->letter == 'h';
		if (!strcmp(a, "--help") || (!h_taken && !strcmp(a, "-h"))) {
			printf("Usage:\n  %s [OPTION...] - %s\n\nOptions:\n", argv[0], usage);
			for (const CliOpt *p = opts; p->name; ++p)
				printf("  -%c, --%-14s %s\n", p->letter, p->name, p->help);
			return 1;
		}
		if (a[0] == '-' && a[1] == '-') {
			const char *eq = strchr(a + 2, '=');
			size_t len = eq ? (size_t)(eq - (a + 2)) : strlen(a + 2);
			for (const CliOpt *p = opts; p->name; ++p)
				if (strlen(p->name) == len && !strncmp(p->name, a + 2, len)) o = p;
			if (o && eq) val = eq + 1;
		} else if (a[0] == '-' && a[1]) {
			for (const CliOpt *p = opts; p->name; ++p)
				if (p->letter == a[1]) o = p;
			if (o && a[2]) val = a + 2;
		}
		if (!o) {
			fprintf(stderr, "Error: Unknown option %s\n", a);
			return -1;
		}
		if (o->has_value && !val) {
			if (i + 1 >= argc) {
				fprintf(stderr, "Error: Missing argument for %s\n", a);
				return -1;
			}
			val = argv[++i];
		}
		set(o->letter, val);
	}
	return 0;
}

/* Device nanoseconds between two markers on a profiling queue. */
static unsigned long long cli_elapsed_ns(CCLEvent *m0, CCLEvent *m1) {
	GError *err = NULL;
	unsigned long long ns = ccl_event_elapsed_ns(m0, m1, &err);
	if (err) clo_error_free(err);
	return ns;
}

#endif
