/*
 * clo_rng_bench: random-number benchmark with the command line and output
 * formats of the reference's src/benchmarks/clo_rng_bench.c (options
 * :40-90, outputs :180-275, draw loop :302-324). Per run, every one of the
 * gws generator states produces one number (next >> (32 - bits), or
 * next % max); the run's numbers are written as a TSV line, a dieharder
 * input file, raw binary or decimal lines on stdout. runs = 0 generates
 * continuously (stdout only). The states are seeded on the host with the
 * Mersenne Twister, or per work-item (GID-based) with a hash (--gid-hash).
 */
#include <time.h>

#include "clo_cli.h"

static const char *rng = "lcg";
static const char *output = "file-tsv";
static size_t gws = 262144;
static size_t lws = 256;
static unsigned runs = 10;
static int dev_idx = -1;
static unsigned rng_seed = 0;
static const char *gid_hash = NULL;
static unsigned bits = 32;
static unsigned maxint = 0;

static const CliOpt opts[] = {
	{"rng", 'r', 1, "Random number generator: " CLO_RNG_IMPLS " (default is lcg)"},
	{"output", 'o', 1, "Output: file-tsv, file-dh, stdout-bin, stdout-uint (default: file-tsv)"},
	{"globalsize", 'g', 1, "Global work size (default is 262144)"},
	{"localsize", 'l', 1, "Local work size (default is 256)"},
	{"runs", 'n', 1, "Random numbers per workitem (default is 10, 0 means continuous generation)"},
	{"device", 'd', 1, "Device index"},
	{"rng-seed", 's', 1, "Seed for random number generator (default is 0)"},
	{"gid-hash", 'h', 1, "Use workitem GID-based seeds instead of MT derived seeds from host. The option value is the hash to apply to seeds (KNUTH, XS1 or source code modifying variable x, e.g. x = x << 2)."},
	{"bits", 'b', 1, "Number of bits in unsigned integers to produce (default 32)"},
	{"max", 'm', 1, "Maximum integer to produce, overrides --bits option"},
	{NULL, 0, 0, NULL}};

static void set(char c, const char *v) {
	switch (c) {
	case 'r': rng = v; break;
	case 'o': output = v; break;
	case 'g': gws = (size_t)strtoull(v, NULL, 0); break;
	case 'l': lws = (size_t)strtoull(v, NULL, 0); break;
	case 'n': runs = (unsigned)strtoul(v, NULL, 0); break;
	case 'd': dev_idx = atoi(v); break;
	case 's': rng_seed = (unsigned)strtoul(v, NULL, 0); break;
	case 'h': gid_hash = v; break;
	case 'b': bits = (unsigned)strtoul(v, NULL, 0); break;
	case 'm': maxint = (unsigned)strtoul(v, NULL, 0); break;
	}
}

static double now_s(void) {
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int main(int argc, char **argv) {
	int pr = cli_parse(argc, argv, opts, "Test RNGs", set);
	if (pr) return pr > 0 ? CLO_SUCCESS : CLO_ERROR_ARGS;
	GError *err = NULL;
	int status = CLO_SUCCESS;
	CCLContext *ctx = NULL;
	CCLQueue *q = NULL;
	CloRng *r = NULL;
	CCLBuffer *dev_out = NULL;
	uint32_t *host = NULL;
	FILE *fp = NULL;
	char fname[512];
	int to_stdout = !strncmp(output, "stdout", 6), raw = 0, dh = 0;
	const char *sep_field = "\t", *sep_line = "\n";
	if (strcmp(output, "file-tsv") && strcmp(output, "file-dh") &&
		strcmp(output, "stdout-bin") && strcmp(output, "stdout-uint")) {
		fprintf(stderr, "Error: Unknown output '%s'.\n", output);
		return CLO_ERROR_ARGS;
	}
	if (bits > 32 || bits < 1) {
		fprintf(stderr, "Error: Number of bits must be between 1 and 32.\n");
		return CLO_ERROR_ARGS;
	}
	if (runs == 0 && !to_stdout) {
		fprintf(stderr, "Error: Continuous generation can only be performed to stdout.\n");
		return CLO_ERROR_ARGS;
	}
	if (gws == 0) {
		fprintf(stderr, "Error: The global work size must be positive.\n");
		return CLO_ERROR_ARGS;
	}
	if (dev_idx < 0) dev_idx = 0;
	ctx = ccl_context_new_from_menu_full(&dev_idx, &err);
	if (err) goto error;
	q = ccl_queue_new(ctx, ccl_context_get_device(ctx, 0, NULL), 0, &err);
	if (err) goto error;
	r = clo_rng_new(rng, gid_hash ? CLO_RNG_SEED_DEV_GID : CLO_RNG_SEED_HOST_MT, NULL, gws,
		rng_seed, gid_hash, ctx, q, &err);
	if (err) goto error;
	dev_out = ccl_buffer_new(ctx, CL_MEM_READ_WRITE, gws * sizeof(uint32_t), NULL, &err);
	if (err) goto error;
	host = clo_host_alloc(gws * sizeof(uint32_t), &err);
	if (err) goto error;
	if (to_stdout) {
		fp = stdout;
		raw = !strcmp(output, "stdout-bin");
		sep_field = "\n";
		sep_line = "";
	} else {
		dh = !strcmp(output, "file-dh");
		snprintf(fname, sizeof fname, "out_%s_%s%s%s", rng, gid_hash ? "gid_" : "host_",
			gid_hash ? gid_hash : "mt", dh ? ".dh.txt" : ".tsv");
		fp = fopen(fname, "w");
		if (!fp) {
			fprintf(stderr, "Error: Unable to create output file '%s'.\n", fname);
			status = CLO_ERROR_OPENFILE;
			goto cleanup;
		}
		if (dh) {
			sep_field = "\n";
			sep_line = "";
			fprintf(fp, "type: d\n");
			fprintf(fp, "count: %d\n", (int)(gws * runs));
			fprintf(fp, "numbit: %d\n", bits);
		}
	}
	if (!to_stdout) {
		printf("\n   =========================== Selected options ============================\n\n");
		printf("     Random number generator (seed): %s (%u)\n", rng, rng_seed);
		printf("     Seeds in workitems: %s %s\n", gid_hash ? "GID-based, hash:" : "Host-based,",
			gid_hash ? gid_hash : "Mersenne Twister");
		printf("     Global/local worksizes: %d/%d\n", (int)gws, (int)lws);
		printf("     Number of runs: %d\n", runs);
		printf("     Number of bits / Maximum integer: %d / %u\n", bits,
			(unsigned)((1ul << bits) - 1));
		printf("     Compiler Options: %s\n", maxint ? " -D CLO_RNG_BENCHMARK_MAXINT" : "");
		printf("\n   =========================== Execution status ============================\n\n");
		printf("     Producing random numbers...\n");
	}
	double t0 = now_s();
	for (unsigned i = 0; i != runs || runs == 0; ++i) {
		CCLEvent *e = clo_rng_fill(r, q, dev_out, 1, bits, maxint, &err);
		if (err || !e) goto error;
		ccl_buffer_enqueue_read(dev_out, q, CL_TRUE, 0, gws * sizeof(uint32_t), host, NULL,
			&err);
		if (err) goto error;
		ccl_queue_gc(q);
		if (raw) {
			if (fwrite(host, sizeof(uint32_t), gws, fp) != gws) break;
		} else {
			for (size_t k = 0; k < gws; ++k) fprintf(fp, "%u%s", host[k], sep_field);
			fprintf(fp, "%s", sep_line);
		}
		if (ferror(fp)) break;
	}
	if (!to_stdout) {
		printf("     Finished, ellapsed time: %lfs\n", now_s() - t0);
		printf("     Done...\n");
	}
	goto cleanup;
error:
	fprintf(stderr, "Error: %s\n", err ? err->message : "unknown");
	status = err && err->code ? err->code : CLO_ERROR_LIBRARY;
	if (err) clo_error_free(err);
cleanup:
	if (fp && fp != stdout) fclose(fp);
	if (host) clo_host_free(host);
	if (dev_out) ccl_buffer_destroy(dev_out);
	if (r) clo_rng_destroy(r);
	if (q) ccl_queue_destroy(q);
	if (ctx) ccl_context_destroy(ctx);
	return status;
}
