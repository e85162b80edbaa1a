/*
 * TEST INFRASTRUCTURE -- OpenCL C on the host, just enough of it to run the
 * reference's own kernel text (cl_ops .cl files) on CPU cores and pin the
 * oracle against it. Used only by oracle/build_ref.py's generated units.
 *
 * Work-items of a work-group run as cooperative fibers (ucontext) on one
 * host thread; barrier() switches to the next work-item, so a work-group
 * advances barrier interval by barrier interval in local-id order -- one of
 * the schedules a conforming OpenCL device may choose. Kernels that hit
 * barriers in divergent ways are reported, not run.
 *
 * OpenCL types: char is signed char (schar below), long is 64-bit (LP64
 * hosts), vector types expose .x/.y/.z/.w and .s0-.s7.
 */
#ifndef CLC_HOST_H
#define CLC_HOST_H

#include <stdint.h>
#include <stddef.h>
#include <limits.h>
#include <string.h>

#include <functional>
#include <vector>

typedef unsigned char uchar;
typedef signed char schar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;
static_assert(sizeof(long) == 8, "OpenCL long is 64-bit");

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

struct uint2 {
	union { uint x; uint s0; };
	union { uint y; uint s1; };
	uint2() : x(0), y(0) {}
	uint2(uint a, uint b) : x(a), y(b) {}
};
struct uint4 {
	union { uint x; uint s0; };
	union { uint y; uint s1; };
	union { uint z; uint s2; };
	union { uint w; uint s3; };
	uint4() : x(0), y(0), z(0), w(0) {}
	uint4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};
struct uint8 {
	uint s0, s1, s2, s3, s4, s5, s6, s7;
	uint8(uint a, uint b, uint c, uint d, uint e, uint f, uint g, uint h)
		: s0(a), s1(b), s2(c), s3(d), s4(e), s5(f), s6(g), s7(h) {}
};
struct ulong2 {
	union { ulong x; ulong s0; };
	union { ulong y; ulong s1; };
	ulong2() : x(0), y(0) {}
	ulong2(ulong a, ulong b) : x(a), y(b) {}
};
static_assert(sizeof(uint2) == 8 && sizeof(uint4) == 16 && sizeof(ulong2) == 16,
	"vector layout");

template <typename D, typename S>
static inline D clc_as(S s) {
	static_assert(sizeof(D) == sizeof(S), "as_type needs equal sizes");
	D d;
	memcpy(&d, &s, sizeof d);
	return d;
}
static inline uint2 as_uint2(ulong v) { return clc_as<uint2>(v); }
static inline uint4 as_uint4(ulong2 v) { return clc_as<uint4>(v); }
static inline int as_int(uint v) { return clc_as<int>(v); }
static inline uint as_uint(int v) { return clc_as<uint>(v); }
static inline uint mul_hi(uint a, uint b) { return (uint)(((ulong)a * (ulong)b) >> 32); }
static inline uint convert_uint(ulong v) { return (uint)v; }

/* ---- work-item context (set by the runner) ------------------------- */
struct ClcWorkItem;
extern thread_local ClcWorkItem *clc_cur;
extern thread_local size_t clc_group, clc_lsize, clc_gsize, clc_ngroups;
size_t clc_local_id();
static inline size_t get_local_id(uint d) { return d == 0 ? clc_local_id() : 0; }
static inline size_t get_group_id(uint d) { return d == 0 ? clc_group : 0; }
static inline size_t get_local_size(uint d) { return d == 0 ? clc_lsize : 1; }
static inline size_t get_global_size(uint d) { return d == 0 ? clc_gsize : 1; }
static inline size_t get_num_groups(uint d) { return d == 0 ? clc_ngroups : 1; }
static inline size_t get_global_id(uint d) {
	return d == 0 ? clc_group * clc_lsize + clc_local_id() : 0;
}
void barrier(int flags);

/* Runs fn once per work-item of an NDRange of gws items in groups of lws
 * (gws a multiple of lws). local_init, when given, is called once per
 * group before its work-items start (to reset __local storage). Returns
 * false if the work-items of a group disagreed on barriers.
 *
 * Work-groups are independent (OpenCL gives them no order), so they are
 * spread over clc_workers() host threads, each running its groups one at a
 * time; __local buffers that a driver passes as kernel arguments must be
 * per worker (ClcLocal below). CLC_THREADS sets the worker count (default:
 * the hardware threads). */
bool clc_run(size_t gws, size_t lws, const std::function<void()> &fn,
	const std::function<void()> &local_init = nullptr);
size_t clc_workers();
size_t clc_worker(); /* index of the calling worker, 0 outside clc_run */

/* One __local buffer per worker: get() is the calling worker's copy. */
template <typename T>
struct ClcLocal {
	std::vector<std::vector<T>> bufs;
	explicit ClcLocal(size_t n) : bufs(clc_workers(), std::vector<T>(n)) {}
	T *get() { return bufs[clc_worker()].data(); }
};

#endif
