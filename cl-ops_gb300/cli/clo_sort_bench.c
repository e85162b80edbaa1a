/*
 * clo_sort_bench: sorting benchmark with the command line and output of
 * the reference's src/benchmarks/clo_sort_bench.c (options :50-80, loop
 * and report :160-250), running this library's sorters. For every size
 * 2^4 .. 2^maxpo2 and run: random host data, a blocking host-data sort,
 * the device time between markers on the exec queue, a sortedness check
 * in the element type's order.
 */
#include "clo_cli.h"

static const char *algorithm = "sbitonic";
static const char *alg_options = "";
static unsigned runs = 1;
static size_t lws = 0;
static int dev_idx = -1;
static unsigned rng_seed = 0;
static const char *type = "uint";
static unsigned maxpo2 = 24;
static const char *out = NULL;
static const char *compiler_opts = NULL;

static const CliOpt opts[] = {
	{"algorithm", 'a', 1, "Sorting algorithm to use (default is sbitonic)"},
	{"alg-opts", 'g', 1, "Algorithm options"},
	{"runs", 'r', 1, "Number of runs (default is 1)"},
	{"localsize", 'l', 1, "Maximum local work size (default is auto-select)"},
	{"device", 'd', 1, "Device index"},
	{"rng-seed", 's', 1, "Seed for random number generator (default is 0)"},
	{"type", 't', 1, "Type of elements to sort (default uint)"},
	{"maxpo2", 'n', 1, "Log2 of the maximum number of elements to sort, e.g. 2^N (default N=24)"},
	{"out", 'o', 1, "File where to output sorting benchmarks (default is no file output)"},
	{"compiler", 'c', 1, "Compiler options"},
	{NULL, 0, 0, NULL}};

static void set(char c, const char *v) {
	switch (c) {
	case 'a': algorithm = v; break;
	case 'g': alg_options = v; break;
	case 'r': runs = (unsigned)strtoul(v, NULL, 0); break;
	case 'l': lws = (size_t)strtoull(v, NULL, 0); break;
	case 'd': dev_idx = atoi(v); break;
	case 's': rng_seed = (unsigned)strtoul(v, NULL, 0); break;
	case 't': type = v; break;
	case 'n': maxpo2 = (unsigned)strtoul(v, NULL, 0); break;
	case 'o': out = v; break;
	case 'c': compiler_opts = v; break;
	}
}

int main(int argc, char **argv) {
	int pr = cli_parse(argc, argv, opts, "Test sorting algorithms", set);
	if (pr) return pr > 0 ? CLO_SUCCESS : CLO_ERROR_ARGS;
	GError *err = NULL;
	int status = CLO_SUCCESS;
	CloSort *sorter = NULL;
	CCLQueue *cq_exec = NULL, *cq_comm = NULL;
	CCLContext *ctx = NULL;
	unsigned char *host = NULL;
	unsigned long long **bench = NULL;
	CliMt rng;
	CloType t = clo_type_by_name(type, &err);
	if (err) goto error;
	if (maxpo2 < 4 || maxpo2 > 32 || runs == 0) {
		fprintf(stderr, "Error: maxpo2 must be in [4, 32] and runs positive\n");
		return CLO_ERROR_ARGS;
	}
	size_t bytes = clo_type_sizeof(t);
	cli_mt_seed(&rng, rng_seed);
	if (dev_idx < 0) dev_idx = 0;
	ctx = ccl_context_new_from_menu_full(&dev_idx, &err);
	if (err) goto error;
	sorter = clo_sort_new(algorithm, alg_options, ctx, &t, NULL, NULL, NULL,
		compiler_opts, &err);
	if (err) goto error;
	cq_exec = ccl_queue_new(ctx, ccl_context_get_device(ctx, 0, NULL),
		CL_QUEUE_PROFILING_ENABLE, &err);
	if (err) goto error;
	cq_comm = ccl_queue_new(ctx, ccl_context_get_device(ctx, 0, NULL), 0, &err);
	if (err) goto error;
	bench = calloc(maxpo2, sizeof *bench);
	for (unsigned i = 0; i < maxpo2; ++i) bench[i] = calloc(runs, sizeof **bench);

	printf("\n   =========================== Selected options ============================\n\n");
	printf("     Random number generator seed: %u\n", rng_seed);
	printf("     Maximum local worksize (0 is auto-select): %d\n", (int)lws);
	printf("     Type of elements to sort: %s\n", clo_type_get_name(t));
	printf("     Number of runs: %d\n", runs);
	printf("     Compiler Options: %s\n", compiler_opts ? compiler_opts : "(null)");

	host = clo_host_alloc(bytes * ((size_t)1 << maxpo2), &err);
	if (err) goto error;
	for (unsigned N = 4; N <= maxpo2; ++N) {
		size_t n = (size_t)1 << N;
		int sorted_ok = 1;
		for (unsigned r = 0; r < runs; ++r) {
			for (size_t i = 0; i < n; ++i) cli_rand(&rng, t, host + bytes * i);
			CCLEvent *m0 = ccl_enqueue_marker(cq_exec, NULL, &err);
			if (err) goto error;
			clo_sort_with_host_data(sorter, cq_exec, cq_comm, host, host, n, lws, &err);
			if (err) goto error;
			CCLEvent *m1 = ccl_enqueue_marker(cq_exec, NULL, &err);
			if (err) goto error;
			bench[N - 1][r] = cli_elapsed_ns(m0, m1);
			ccl_queue_finish(cq_comm, &err);
			if (err) goto error;
			sorted_ok = 1;
			for (size_t i = 0; i + 1 < n; ++i)
				if (cli_compare(t, host + bytes * i, host + bytes * (i + 1)) > 0) {
					sorted_ok = 0;
					break;
				}
			ccl_queue_gc(cq_exec);
		}
		unsigned long long total = 0;
		for (unsigned r = 0; r < runs; ++r) total += bench[N - 1][r];
		printf("       - 2^%d: %lf Mkeys/s %s\n", N,
			(1e-6 * (double)n * runs) / ((double)(total ? total : 1) * 1e-9),
			sorted_ok ? "" : "(sort did not work)");
	}
	if (out) {
		FILE *f = fopen(out, "w");
		if (!f) {
			fprintf(stderr, "Error: Unable to open output file '%s'\n", out);
			status = CLO_ERROR_OPENFILE;
			goto cleanup;
		}
		for (unsigned i = 0; i < maxpo2; ++i) {
			fprintf(f, "%d", i);
			for (unsigned j = 0; j < runs; ++j) fprintf(f, "\t%llu", bench[i][j]);
			fprintf(f, "\n");
		}
		fclose(f);
	}
	goto cleanup;
error:
	fprintf(stderr, "Error: %s\n", err->message);
	status = err->code ? err->code : CLO_ERROR_LIBRARY;
	clo_error_free(err);
cleanup:
	if (sorter) clo_sort_destroy(sorter);
	if (cq_exec) ccl_queue_destroy(cq_exec);
	if (cq_comm) ccl_queue_destroy(cq_comm);
	if (ctx) ccl_context_destroy(ctx);
	if (host) clo_host_free(host);
	if (bench) {
		for (unsigned i = 0; i < maxpo2; ++i) free(bench[i]);
		free(bench);
	}
	return status;
}
