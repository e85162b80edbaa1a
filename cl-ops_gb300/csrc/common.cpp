// Common module: scalar type table, bit utilities and error plumbing.
// Reference behaviour: src/cl_ops/common/clo_common.c:54-223.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "clo_internal.h"

struct clo_type_info {
	const char *name;
	size_t size;
};

// Same order and sizes as the reference table (clo_common.c:54-68); the
// enum values index it directly.
static const clo_type_info kTypes[] = {
	{"char", 1}, {"uchar", 1}, {"short", 2}, {"ushort", 2},
	{"int", 4}, {"uint", 4}, {"long", 8}, {"ulong", 8},
	{"half", 2}, {"float", 4}, {"double", 8}, {nullptr, 0}};

static bool type_valid(int t) { return t >= CLO_CHAR && t <= CLO_DOUBLE; }

extern "C" {

const char *clo_type_get_name(CloType type) {
	if (!type_valid(type)) {
		fprintf(stderr, "cl_ops: clo_type_get_name: invalid type %d\n",
			(int)type);
		return nullptr;
	}
	return kTypes[type].name;
}

size_t clo_type_sizeof(CloType type) {
	if (!type_valid(type)) {
		fprintf(stderr, "cl_ops: clo_type_sizeof: invalid type %d\n",
			(int)type);
		return 0;
	}
	return kTypes[type].size;
}

CloType clo_type_by_name(const char *name, GError **err) {
	for (int i = 0; kTypes[i].name != nullptr; ++i)
		if (name && strcmp(name, kTypes[i].name) == 0) return (CloType)i;
	clo::set_error(err, CLO_ERROR_UNKNOWN_TYPE, "Unknown type '%s'",
		name ? name : "(null)");
	return (CloType)-1;
}

// Next power of two, x itself when it already is one (and 0 for 0), with
// 32-bit wrap-around like the reference's bit-smearing version.
unsigned int clo_nlpo2(unsigned int x) {
	if ((x & (x - 1)) == 0) return x;
	unsigned int p = 1u << (32 - __builtin_clz(x));
	return (32 - __builtin_clz(x)) >= 32 ? 0u : p;
}

unsigned int clo_ones32(unsigned int x) {
	return (unsigned int)__builtin_popcount(x);
}

// popcount((x & -x) - 1): the number of trailing zeros, 32 for x == 0.
unsigned int clo_tzc(int x) {
	unsigned int u = (unsigned int)x;
	return clo_ones32((u & (0u - u)) - 1u);
}

unsigned int clo_sum(unsigned int x) {
	// Closed form of the reference's recursion, same 32-bit wrap-around.
	unsigned long long s = (unsigned long long)x * (x + 1ull) / 2ull;
	return (unsigned int)s;
}

void clo_print_to_null(const char *string) { (void)string; }

GQuark clo_error_quark(void) {
	// Without GLib there is no quark table; a fixed non-zero id stands for
	// the "clo-error-quark" domain.
	return 0x434c4f31u;
}

void clo_error_free(GError *e) {
	if (!e) return;
	free(e->message);
	free(e);
}

void clo_clear_error(GError **err) {
	if (err && *err) {
		clo_error_free(*err);
		*err = nullptr;
	}
}

}  // extern "C"

namespace clo {

void set_error(GError **err, int code, const char *fmt, ...) {
	if (err == nullptr) return;
	if (*err != nullptr) {
		fprintf(stderr, "cl_ops: error set over a previous error\n");
		return;
	}
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	GError *e = (GError *)malloc(sizeof(GError));
	e->domain = clo_error_quark();
	e->code = code;
	e->message = strdup(buf);
	*err = e;
}

void propagate_error(GError **dest, GError *src) {
	if (!src) return;
	if (dest == nullptr || *dest != nullptr) {
		clo_error_free(src);
		return;
	}
	*dest = src;
}

bool cuda_ok(cudaError_t e, GError **err, const char *what) {
	if (e == cudaSuccess) return true;
	set_error(err, CLO_ERROR_LIBRARY, "%s: CUDA error %d (%s)", what, (int)e,
		cudaGetErrorString(e));
	// The error is reported here; clear the runtime's last-error state so a
	// later cudaGetLastError (after another call's launch) does not return
	// it again. A sticky error stays whatever is done here.
	cudaGetLastError();
	return false;
}

static std::atomic<long> g_live_wrappers{0};
void wrapper_created() { g_live_wrappers.fetch_add(1); }
void wrapper_destroyed() { g_live_wrappers.fetch_sub(1); }
long live_wrappers() { return g_live_wrappers.load(); }

static std::atomic<unsigned long long> g_launches{0};
void count_launches(unsigned n) { g_launches.fetch_add(n); }

bool check_offsets(const uint64_t *off, size_t S, size_t numel, GError **err) {
	if (S > 0 && off == nullptr) {
		set_error(err, CLO_ERROR_ARGS, "NULL segment offsets");
		return false;
	}
	for (size_t i = 0; i < S; ++i) {
		if (off[i] > off[i + 1] || off[i + 1] > numel ||
			off[i + 1] - off[i] >= (1ull << 30)) {
			set_error(err, CLO_ERROR_ARGS,
				"Segment %zu [%llu, %llu) is invalid: offsets must not decrease, "
				"must stay within %zu elements, and segments must be shorter "
				"than 2^30", i, (unsigned long long)off[i],
				(unsigned long long)off[i + 1], numel);
			return false;
		}
	}
	return true;
}

bool type_is_integer(CloType t) { return t >= CLO_CHAR && t <= CLO_ULONG; }
bool type_is_signed(CloType t) {
	return t == CLO_CHAR || t == CLO_SHORT || t == CLO_INT || t == CLO_LONG;
}

}  // namespace clo

extern "C" cl_ulong clo_gb300_launch_count(void) {
	return (cl_ulong)clo::g_launches.load();
}
