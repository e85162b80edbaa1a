/*
 * clo_scan_bench: scan benchmark with the command line and output of the
 * reference's src/benchmarks/clo_scan_bench.c (options :120-170, loop and
 * check :200-280): sizes init_elems * 2^k, values in [0, 128), a blocking
 * host-data scan, device time between markers on the exec queue, and the
 * serial check ("[Overflow]" when the running sum leaves the sum type).
 */
#include "clo_cli.h"

static unsigned runs = 1;
static size_t lws = 0;
static int dev_idx = -1;
static unsigned rng_seed = 0;
static const char *type = "uint";
static const char *type_sum = "ulong";
static unsigned init_elems = 4;
static unsigned num_doub = 24;
static const char *compiler_opts = NULL;
static const char *algorithm = "blelloch";
static const char *alg_options = "";
static int no_check = 0;
static const char *out = NULL;

static const CliOpt opts[] = {
	{"runs", 'r', 1, "Number of runs (default is 1)"},
	{"localsize", 'l', 1, "Maximum local work size (default is auto-select)"},
	{"device", 'd', 1, "Device index"},
	{"rng-seed", 's', 1, "Seed for random number generator (default is 0)"},
	{"type", 't', 1, "Type of elements to scan (default uint)"},
	{"type-sum", 'y', 1, "Type of elements in scan result (default ulong)"},
	{"init-elems", 'i', 1, "The starting number of elements to scan (default is 4)"},
	{"num-doub", 'n', 1, "Number of times min-elems is doubled (default is 24)"},
	{"compiler", 'c', 1, "Compiler options"},
	{"algorithm", 'a', 1, "Scan algorithm to use (default is 'blelloch')"},
	{"alg-opts", 'p', 1, "Algorithm options"},
	{"no-check", 'u', 0, "Don't check scan with serial version"},
	{"out", 'o', 1, "File where to output scan benchmarks (default is no file output)"},
	{NULL, 0, 0, NULL}};

static void set(char c, const char *v) {
	switch (c) {
	case 'r': runs = (unsigned)strtoul(v, NULL, 0); break;
	case 'l': lws = (size_t)strtoull(v, NULL, 0); break;
	case 'd': dev_idx = atoi(v); break;
	case 's': rng_seed = (unsigned)strtoul(v, NULL, 0); break;
	case 't': type = v; break;
	case 'y': type_sum = v; break;
	case 'i': init_elems = (unsigned)strtoul(v, NULL, 0); break;
	case 'n': num_doub = (unsigned)strtoul(v, NULL, 0); break;
	case 'c': compiler_opts = v; break;
	case 'a': algorithm = v; break;
	case 'p': alg_options = v; break;
	case 'u': no_check = 1; break;
	case 'o': out = v; break;
	}
}

static uint64_t get_u(const unsigned char *p, size_t i, size_t bytes) {
	uint64_t v = 0;
	memcpy(&v, p + bytes * i, bytes);  /* little-endian hosts */
	return v;
}

int main(int argc, char **argv) {
	int pr = cli_parse(argc, argv, opts, "Test scan algorithms", set);
	if (pr) return pr > 0 ? CLO_SUCCESS : CLO_ERROR_ARGS;
	GError *err = NULL;
	int status = CLO_SUCCESS;
	CloScan *scanner = NULL;
	CCLQueue *cq_exec = NULL, *cq_comm = NULL;
	CCLContext *ctx = NULL;
	unsigned char *in = NULL, *res = NULL;
	double **bench = NULL;
	CliMt rng;
	CloType te = clo_type_by_name(type, &err);
	if (err) goto error;
	CloType ts = clo_type_by_name(type_sum, &err);
	if (err) goto error;
	if (runs == 0 || init_elems == 0 || num_doub == 0 || num_doub > 40) {
		fprintf(stderr, "Error: runs, init-elems and num-doub must be positive\n");
		return CLO_ERROR_ARGS;
	}
	size_t bytes = clo_type_sizeof(te), bytes_sum = clo_type_sizeof(ts);
	cli_mt_seed(&rng, rng_seed);
	if (dev_idx < 0) dev_idx = 0;
	ctx = ccl_context_new_from_menu_full(&dev_idx, &err);
	if (err) goto error;
	scanner = clo_scan_new(algorithm, alg_options, ctx, te, ts, compiler_opts, &err);
	if (err) goto error;
	cq_exec = ccl_queue_new(ctx, ccl_context_get_device(ctx, 0, NULL),
		CL_QUEUE_PROFILING_ENABLE, &err);
	if (err) goto error;
	cq_comm = ccl_queue_new(ctx, ccl_context_get_device(ctx, 0, NULL), 0, &err);
	if (err) goto error;

	printf("\n   =========================== Selected options ============================\n\n");
	printf("     Random number generator seed: %u\n", rng_seed);
	printf("     Maximum local worksize (0 = auto): %d\n", (int)lws);
	printf("     Type of elements to scan: %s\n", clo_type_get_name(te));
	printf("     Type of elements in scan result: %s\n", clo_type_get_name(ts));
	printf("     Starting number of elements: %d\n", init_elems);
	printf("     Number of times number of elements will be doubled: %d\n", num_doub);
	printf("     Number of runs: %d\n", runs);
	printf("     Compiler Options: %s\n", compiler_opts ? compiler_opts : "(null)");

	bench = calloc(num_doub, sizeof *bench);
	for (unsigned i = 0; i < num_doub; ++i) bench[i] = calloc(runs, sizeof **bench);
	size_t max_elems = (size_t)init_elems << num_doub;
	in = clo_host_alloc(bytes * max_elems, &err);
	if (err) goto error;
	res = clo_host_alloc(bytes_sum * max_elems, &err);
	if (err) goto error;
	size_t n = init_elems;
	for (unsigned N = 1; N <= num_doub; ++N, n *= 2) {
		const char *scan_ok = "";
		for (unsigned r = 0; r < runs; ++r) {
			for (size_t i = 0; i < n; ++i) {
				uint64_t v = (uint64_t)(cli_mt_double(&rng) * 128);
				memcpy(in + bytes * i, &v, bytes);
			}
			CCLEvent *m0 = ccl_enqueue_marker(cq_exec, NULL, &err);
			if (err) goto error;
			clo_scan_with_host_data(scanner, cq_exec, cq_comm, in, res, n, lws, &err);
			if (err) goto error;
			CCLEvent *m1 = ccl_enqueue_marker(cq_exec, NULL, &err);
			if (err) goto error;
			bench[N - 1][r] = (double)cli_elapsed_ns(m0, m1);
			ccl_queue_finish(cq_comm, &err);
			if (err) goto error;
			ccl_queue_gc(cq_exec);
			if (no_check) {
				scan_ok = "[Unverified]";
				continue;
			}
			scan_ok = "";
			const uint64_t maxu = bytes_sum >= 8 ? UINT64_MAX : ((1ull << (8 * bytes_sum)) - 1);
			uint64_t host = 0;
			for (size_t i = 0; i < n; ++i) {
				host = i == 0 ? 0 : host + get_u(in, i - 1, bytes);
				if (host > maxu) {
					scan_ok = "[Overflow]";
					break;
				}
				if (get_u(res, i, bytes_sum) != host) {
					scan_ok = "[Scan did not work]";
					break;
				}
			}
		}
		double total = 0;
		for (unsigned r = 0; r < runs; ++r) total += bench[N - 1][r];
		printf("       - %10d : %f MValues/s %s\n", (int)n,
			(1e-6 * (double)n * runs) / ((total ? total : 1) * 1e-9), scan_ok);
	}
	if (out) {
		FILE *f = fopen(out, "w");
		if (!f) {
			fprintf(stderr, "Error: Unable to open output file '%s'\n", out);
			status = CLO_ERROR_OPENFILE;
			goto cleanup;
		}
		for (unsigned i = 0; i < num_doub; ++i) {
			fprintf(f, "%d", i);
			for (unsigned j = 0; j < runs; ++j) fprintf(f, "\t%lf", bench[i][j]);
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
	if (scanner) clo_scan_destroy(scanner);
	if (cq_exec) ccl_queue_destroy(cq_exec);
	if (cq_comm) ccl_queue_destroy(cq_comm);
	if (ctx) ccl_context_destroy(ctx);
	if (in) clo_host_free(in);
	if (res) clo_host_free(res);
	if (bench) {
		for (unsigned i = 0; i < num_doub; ++i) free(bench[i]);
		free(bench);
	}
	return status;
}
