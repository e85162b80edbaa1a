/*
 * cl_ops on GB300 -- common types, error codes and bit utilities.
 *
 * Drop-in for the reference's common module:
 *   src/cl_ops/common/clo_common.in.h:31-165 (types, error codes, macros,
 *   utility prototypes) and src/cl_ops/common/clo_common.c:54-223.
 *
 * GLib is not required. When <glib.h> has not been included before this
 * header, a GError-layout-compatible struct is declared here
 * ({GQuark domain; int code; char *message}, the same field order and
 * types as GLib's GError) so code written against the reference compiles
 * unchanged. Errors created by this library are released with
 * clo_error_free().
 */
#ifndef CLO_COMMON_H
#define CLO_COMMON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- OpenCL scalar typedefs (only when no OpenCL header is present) ---- */
#if !defined(__OPENCL_CL_H) && !defined(CLO_HAVE_CL_TYPES)
#define CLO_HAVE_CL_TYPES 1
typedef int8_t cl_char;
typedef uint8_t cl_uchar;
typedef int16_t cl_short;
typedef uint16_t cl_ushort;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef int64_t cl_long;
typedef uint64_t cl_ulong;
typedef uint16_t cl_half;
typedef float cl_float;
typedef double cl_double;
typedef cl_uint cl_bool;
#define CL_FALSE 0
#define CL_TRUE 1
#endif

/* ---- GError-compatible error object (only when GLib is absent) ---- */
#if !defined(__G_LIB_H__) && !defined(CLO_HAVE_GERROR)
#define CLO_HAVE_GERROR 1
typedef uint32_t GQuark;
typedef struct _GError {
	GQuark domain;
	int code;
	char *message;
} GError;
#endif

/** Default RNG seed (clo_common.in.h:31). */
#define CLO_DEFAULT_SEED 0

/** Error domain of this library (clo_common.in.h:36). */
#define CLO_ERROR clo_error_quark()

/** Integer division rounding up (clo_common.in.h:53). */
#define CLO_DIV_CEIL(a, b) (((a) + (b) - 1) / (b))

/** Smallest multiple of lws that is >= gws (clo_common.in.h:63). */
#define CLO_GWS_MULT(gws, lws) ((lws) * CLO_DIV_CEIL(gws, lws))

/** True when x is a power of two (clo_common.in.h:70). */
#define CLO_IS_PO2(x) (((x) & ((x) - 1)) == 0)

/** Error codes (clo_common.in.h:80-95), same numeric values. */
enum clo_error_codes {
	CLO_SUCCESS = 0,
	CLO_ERROR_OPENFILE = 1,
	CLO_ERROR_ARGS = 2,
	CLO_ERROR_STREAM_WRITE = 3,
	CLO_ERROR_IMPL_NOT_FOUND = 5,
	CLO_ERROR_UNKNOWN_TYPE = 6,
	CLO_ERROR_LIBRARY = 7
};

/** Scalar element types (clo_common.in.h:108-120), same numeric values. */
typedef enum {
	CLO_CHAR = 0,
	CLO_UCHAR = 1,
	CLO_SHORT = 2,
	CLO_USHORT = 3,
	CLO_INT = 4,
	CLO_UINT = 5,
	CLO_LONG = 6,
	CLO_ULONG = 7,
	CLO_HALF = 8,
	CLO_FLOAT = 9,
	CLO_DOUBLE = 10
} CloType;

typedef struct clo_type_info CloTypeInfo;
typedef struct clo_sort CloSort;
typedef struct clo_scan CloScan;
typedef struct clo_rng CloRng;

/* clo_common.c:77 -- type name ("uint", ...) or NULL for a bad type. */
const char *clo_type_get_name(CloType type);

/* clo_common.c:91 -- size in bytes, 0 for a bad type. */
size_t clo_type_sizeof(CloType type);

/* clo_common.c:107 -- type by name; -1 and CLO_ERROR_UNKNOWN_TYPE when
 * the name is unknown. */
CloType clo_type_by_name(const char *name, GError **err);

/* clo_common.c:141 -- next power of two (x itself when already one). */
unsigned int clo_nlpo2(unsigned int x);

/* clo_common.c:162 -- population count of a 32-bit word. */
unsigned int clo_ones32(unsigned int x);

/* clo_common.c:183 -- trailing zero count (log2 of a power of two). */
unsigned int clo_tzc(int x);

/* clo_common.c:197 -- 0 + 1 + ... + x. */
unsigned int clo_sum(unsigned int x);

/* clo_common.c:208 -- print handler that discards its argument. */
void clo_print_to_null(const char *string);

/* clo_common.c:220 -- the CLO_ERROR domain. */
GQuark clo_error_quark(void);

/* Releases an error created by this library (replaces g_error_free for
 * errors this library sets when GLib is absent). Accepts NULL. */
void clo_error_free(GError *err);

/* Releases *err (if any) and sets *err to NULL, like g_clear_error. */
void clo_clear_error(GError **err);

#ifdef __cplusplus
}
#endif

#endif /* CLO_COMMON_H */
