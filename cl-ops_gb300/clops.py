"""ctypes binding of libclops.so, the C-ABI drop-in for cl_ops.

Mirrors the reference API one to one (same function names and argument
order as src/cl_ops/*/clo_*.h and the cf4ocl2 calls the reference uses);
`Lib` exposes the raw functions, and the small classes below wrap them the
way the reference's tests and benchmarks use them (create a context and a
queue, create an object, run with device or host data, destroy).

Errors come back as GError* and are raised as CloError with the same
code. The library must be built (build_lib.py); importing this module
without it raises, there is no fallback path.
"""
import ctypes as C
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libclops.so"

# CloType values (clo_common.in.h:108-120).
CLO_CHAR, CLO_UCHAR, CLO_SHORT, CLO_USHORT, CLO_INT, CLO_UINT, CLO_LONG, \
    CLO_ULONG, CLO_HALF, CLO_FLOAT, CLO_DOUBLE = range(11)
# Error codes (clo_common.in.h:80-95).
CLO_SUCCESS, CLO_ERROR_OPENFILE, CLO_ERROR_ARGS, CLO_ERROR_STREAM_WRITE = 0, 1, 2, 3
CLO_ERROR_IMPL_NOT_FOUND, CLO_ERROR_UNKNOWN_TYPE, CLO_ERROR_LIBRARY = 5, 6, 7
# Seed types (clo_rng.in.h:78-92).
CLO_RNG_SEED_DEV_GID, CLO_RNG_SEED_HOST_MT, CLO_RNG_SEED_EXT_DEV, \
    CLO_RNG_SEED_EXT_HOST = range(4)
CL_QUEUE_PROFILING_ENABLE = 1 << 1
SEG_SORT_VARIANTS = 36  # CLO_SEG_SORT_VARIANTS
CL_MEM_READ_WRITE = 1 << 0

NP_OF_TYPE = {
    CLO_CHAR: np.int8, CLO_UCHAR: np.uint8, CLO_SHORT: np.int16,
    CLO_USHORT: np.uint16, CLO_INT: np.int32, CLO_UINT: np.uint32,
    CLO_LONG: np.int64, CLO_ULONG: np.uint64, CLO_HALF: np.float16,
    CLO_FLOAT: np.float32, CLO_DOUBLE: np.float64,
}

RNG_NAMES = ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller", "tauslcg"]
RNG_SEED_SIZE = {"lcg": 8, "xorshift64": 8, "xorshift128": 16, "mwc64x": 8,
                 "parkmiller": 4, "tauslcg": 16}


class GError(C.Structure):
    _fields_ = [("domain", C.c_uint32), ("code", C.c_int), ("message", C.c_char_p)]


class CloError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code
        self.message = message


class ServeRequest(C.Structure):
    """CloServeRequest (include/clo_serve.h)."""
    _fields_ = [("op", C.c_int), ("type", C.c_int), ("sum_type", C.c_int),
                ("n", C.c_size_t), ("draws", C.c_size_t), ("rng", C.c_int),
                ("in_", C.c_void_p), ("out", C.c_void_p), ("device_data", C.c_uint32)]


class ServeStats(C.Structure):
    """CloServeStats (include/clo_serve.h)."""
    _fields_ = [(f, C.c_uint64) for f in ("submitted", "admitted", "completed", "failed",
                                         "rejected", "batches", "max_queued")] + \
               [("budget_bytes", C.c_size_t), ("peak_bytes", C.c_size_t)] + \
               [(f, C.c_double) for f in ("p50_ms", "p99_ms", "max_ms", "mean_ms",
                                         "elements", "span_s")] + \
               [("max_concurrent_batches", C.c_uint64), ("device_busy_s", C.c_double),
                ("mean_concurrent_batches", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


SERVE_SORT, SERVE_SCAN, SERVE_RNG_FILL = 0, 1, 2

P = C.c_void_p
PERR = C.POINTER(C.POINTER(GError))
SZ = C.c_size_t
U32 = C.c_uint32
U64 = C.c_uint64

# name: (restype, [argtypes])
_SIGS = {
    # common
    "clo_type_get_name": (C.c_char_p, [C.c_int]),
    "clo_type_sizeof": (SZ, [C.c_int]),
    "clo_type_by_name": (C.c_int, [C.c_char_p, PERR]),
    "clo_nlpo2": (C.c_uint, [C.c_uint]),
    "clo_ones32": (C.c_uint, [C.c_uint]),
    "clo_tzc": (C.c_uint, [C.c_int]),
    "clo_sum": (C.c_uint, [C.c_uint]),
    "clo_print_to_null": (None, [C.c_char_p]),
    "clo_error_quark": (U32, []),
    "clo_error_free": (None, [C.POINTER(GError)]),
    "clo_clear_error": (None, [PERR]),
    # ccl shim
    "ccl_context_new_any": (P, [PERR]),
    "ccl_context_new_gpu": (P, [PERR]),
    "ccl_context_new_from_menu_full": (P, [P, PERR]),
    "ccl_context_new_from_device_index": (P, [C.c_int, PERR]),
    "ccl_context_destroy": (None, [P]),
    "ccl_context_ref": (None, [P]),
    "ccl_context_unref": (None, [P]),
    "ccl_context_get_num_devices": (U32, [P, PERR]),
    "ccl_context_get_device": (P, [P, U32, PERR]),
    "ccl_device_get_ordinal": (C.c_int, [P]),
    "ccl_queue_new": (P, [P, P, U64, PERR]),
    "ccl_queue_new_wrap": (P, [P, P, U64, PERR]),
    "ccl_queue_destroy": (None, [P]),
    "ccl_queue_finish": (U32, [P, PERR]),
    "ccl_queue_get_device": (P, [P, PERR]),
    "ccl_queue_get_context": (P, [P, PERR]),
    "ccl_queue_unwrap": (P, [P]),
    "ccl_queue_gc": (None, [P]),
    "ccl_buffer_new": (P, [P, U64, SZ, P, PERR]),
    "ccl_buffer_new_wrap": (P, [P, P, SZ, PERR]),
    "ccl_buffer_destroy": (None, [P]),
    "ccl_buffer_ref": (None, [P]),
    "ccl_buffer_unwrap": (P, [P]),
    "ccl_buffer_get_size": (SZ, [P]),
    "ccl_buffer_enqueue_read": (P, [P, P, U32, SZ, SZ, P, P, PERR]),
    "ccl_buffer_enqueue_write": (P, [P, P, U32, SZ, SZ, P, P, PERR]),
    "ccl_buffer_enqueue_copy": (P, [P, P, P, SZ, SZ, SZ, P, PERR]),
    "ccl_ewl": (P, None),
    "ccl_event_wait_list_add": (None, None),
    "ccl_event_wait_list_clear": (None, [P]),
    "ccl_event_wait": (U32, [P, PERR]),
    "ccl_event_set_name": (None, [P, C.c_char_p]),
    "ccl_event_get_name": (C.c_char_p, [P]),
    "ccl_event_get_duration": (U64, [P, PERR]),
    "ccl_enqueue_marker": (P, [P, P, PERR]),
    "ccl_event_elapsed_ns": (U64, [P, P, PERR]),
    "ccl_program_get_source": (C.c_char_p, [P]),
    "ccl_program_new_from_source": (P, [P, C.c_char_p, PERR]),
    "ccl_program_new_from_sources": (P, [P, U32, C.POINTER(C.c_char_p), C.POINTER(SZ), PERR]),
    "ccl_program_build": (U32, [P, C.c_char_p, PERR]),
    "ccl_program_get_build_log": (C.c_char_p, [P, PERR]),
    "ccl_program_get_kernel": (P, [P, C.c_char_p, PERR]),
    "ccl_program_destroy": (None, [P]),
    "ccl_arg_new": (P, [P, SZ]),
    "ccl_arg_destroy": (None, [P]),
    "ccl_kernel_suggest_worksizes": (U32, [P, P, U32, C.POINTER(SZ), C.POINTER(SZ),
                                            C.POINTER(SZ), PERR]),
    # variadic: the fixed part only (Program.enqueue passes the rest)
    "ccl_kernel_set_args_and_enqueue_ndrange": (P, None),
    "ccl_program_get_build_options": (C.c_char_p, [P]),
    "ccl_wrapper_memcheck": (U32, []),
    # sort
    "clo_sort_new": (P, [C.c_char_p, C.c_char_p, P, C.POINTER(C.c_int),
                         C.POINTER(C.c_int), C.c_char_p, C.c_char_p, C.c_char_p, PERR]),
    "clo_sort_destroy": (None, [P]),
    "clo_sort_with_device_data": (P, [P, P, P, P, P, SZ, SZ, PERR]),
    "clo_sort_with_host_data": (U32, [P, P, P, P, P, SZ, SZ, PERR]),
    "clo_sort_get_context": (P, [P]),
    "clo_sort_get_program": (P, [P]),
    "clo_sort_get_element_type": (C.c_int, [P]),
    "clo_sort_get_element_size": (SZ, [P]),
    "clo_sort_get_key_type": (C.c_int, [P]),
    "clo_sort_get_key_size": (SZ, [P]),
    "clo_sort_get_data": (P, [P]),
    "clo_sort_set_data": (None, [P, P]),
    "clo_sort_get_num_kernels": (U32, [P, PERR]),
    "clo_sort_get_kernel_name": (C.c_char_p, [P, U32, PERR]),
    "clo_sort_get_localmem_usage": (SZ, [P, U32, SZ, SZ, PERR]),
    # scan
    "clo_scan_new": (P, [C.c_char_p, C.c_char_p, P, C.c_int, C.c_int, C.c_char_p, PERR]),
    "clo_scan_destroy": (None, [P]),
    "clo_scan_with_device_data": (P, [P, P, P, P, P, SZ, SZ, PERR]),
    "clo_scan_with_host_data": (U32, [P, P, P, P, P, SZ, SZ, PERR]),
    "clo_scan_get_context": (P, [P]),
    "clo_scan_get_program": (P, [P]),
    "clo_scan_get_elem_type": (C.c_int, [P]),
    "clo_scan_get_element_size": (SZ, [P]),
    "clo_scan_get_sum_type": (C.c_int, [P]),
    "clo_scan_get_sum_size": (SZ, [P]),
    "clo_scan_get_data": (P, [P]),
    "clo_scan_set_data": (None, [P, P]),
    "clo_scan_get_num_kernels": (U32, [P, PERR]),
    "clo_scan_get_kernel_name": (C.c_char_p, [P, U32, PERR]),
    "clo_scan_get_localmem_usage": (SZ, [P, U32, SZ, SZ, PERR]),
    # rng
    "clo_rng_new": (P, [C.c_char_p, C.c_int, P, SZ, U64, C.c_char_p, P, P, PERR]),
    "clo_rng_destroy": (None, [P]),
    "clo_rng_get_source": (C.c_char_p, [P]),
    "clo_rng_get_device_seeds": (P, [P]),
    "clo_rng_get_size": (SZ, [P]),
    # additions
    "clo_sort_kv_with_device_data": (P, [P, P, P, P, C.c_int, SZ, PERR]),
    "clo_sort_kv_with_host_data": (U32, [P, P, P, P, C.c_int, SZ, PERR]),
    "clo_rng_fill": (P, [P, P, P, SZ, U32, U32, PERR]),
    "clo_host_alloc": (P, [SZ, PERR]),
    "clo_host_free": (None, [P]),
    "clo_gb300_launch_count": (U64, []),
    "clo_gb300_debug_scan_withhold": (None, [C.c_longlong]),
    "clo_sort_segmented_with_device_data": (P, [P, P, P, P, SZ, PERR]),
    "clo_sort_segmented_with_host_data": (U32, [P, P, P, SZ, P, SZ, PERR]),
    "clo_sort_segmented_tune": (C.c_int, [P, P, P, P, SZ, C.POINTER(C.c_double), PERR]),
    "clo_sort_segmented_get_variant": (C.c_int, [P]),
    "clo_scan_segmented_with_device_data": (P, [P, P, P, P, P, SZ, PERR]),
    "clo_scan_segmented_with_host_data": (U32, [P, P, P, P, SZ, P, SZ, PERR]),
    "clo_queue_begin_capture": (U32, [P, PERR]),
    "clo_queue_end_capture": (P, [P, PERR]),
    "clo_graph_launch": (U32, [P, P, PERR]),
    "clo_graph_get_num_nodes": (SZ, [P]),
    "clo_graph_destroy": (None, [P]),
    "clo_serve_new": (P, [P, SZ, C.c_int, PERR]),
    "clo_serve_submit": (U64, [P, C.POINTER(ServeRequest), PERR]),
    "clo_serve_wait": (U32, [P, U64, C.POINTER(C.c_double), PERR]),
    "clo_serve_drain": (U32, [P, PERR]),
    "clo_serve_replay": (U32, [P, C.POINTER(ServeRequest), C.POINTER(C.c_double), SZ,
                               C.POINTER(U64), PERR]),
    "clo_serve_configure": (U32, [P, SZ, SZ, SZ, PERR]),
    "clo_serve_get_stats": (None, [P, C.POINTER(ServeStats)]),
    "clo_serve_reset_stats": (None, [P]),
    "clo_serve_destroy": (None, [P]),
    "clo_serve_footprint": (SZ, [C.POINTER(ServeRequest)]),
    "clo_serve_select": (SZ, [C.POINTER(ServeRequest), SZ, SZ, SZ, SZ, SZ, C.POINTER(SZ)]),
    "clo_gb300_timing_enable": (None, [C.c_int]),
    "clo_gb300_timing_reset": (None, []),
    "clo_gb300_timing_get": (C.c_int, [C.c_char_p, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(U64)]),
}

# Data symbols exported by the library.
DATA_SYMBOLS = ["clo_rng_infos", "clo_sort_sbitonic_def", "clo_sort_abitonic_def",
                "clo_sort_gselect_def", "clo_sort_satradix_def", "clo_scan_blelloch_def"]


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built (run build_lib.py)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        if args is not None:
            f.argtypes = args
    return lib


lib = _load()


def err_ptr():
    return C.POINTER(GError)()


def check(e, what=""):
    """Raises CloError when the GError* holder is set (and frees it)."""
    if e:
        code, msg = e.contents.code, (e.contents.message or b"").decode()
        lib.clo_error_free(e)
        raise CloError(code, f"{what}: {msg}" if what else msg)


def call(fn, *args, what=None):
    """Calls fn(*args, &err) and raises on error."""
    e = err_ptr()
    r = fn(*args, C.byref(e))
    check(e, what or getattr(fn, "__name__", ""))
    return r


def np_ptr(a):
    return C.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- objects
class Context:
    def __init__(self, ordinal=0):
        self.h = call(lib.ccl_context_new_from_device_index, ordinal)

    def destroy(self):
        if self.h:
            lib.ccl_context_destroy(self.h)
            self.h = None


class Queue:
    def __init__(self, ctx, profiling=False, stream=None):
        props = CL_QUEUE_PROFILING_ENABLE if profiling else 0
        if stream is None:
            self.h = call(lib.ccl_queue_new, ctx.h, None, props)
        else:
            self.h = call(lib.ccl_queue_new_wrap, ctx.h, C.c_void_p(stream), props)

    def finish(self):
        call(lib.ccl_queue_finish, self.h)

    def gc(self):
        lib.ccl_queue_gc(self.h)

    def marker(self):
        return call(lib.ccl_enqueue_marker, self.h, None)

    @staticmethod
    def elapsed_ms(m0, m1):
        return call(lib.ccl_event_elapsed_ns, C.c_void_p(m0), C.c_void_p(m1)) / 1e6

    def destroy(self):
        if self.h:
            lib.ccl_queue_destroy(self.h)
            self.h = None


class Buffer:
    """Device buffer; `from_array` uploads, `read` downloads."""

    def __init__(self, ctx, nbytes, host=None):
        self.ctx = ctx
        self.nbytes = nbytes
        self.h = call(lib.ccl_buffer_new, ctx.h, CL_MEM_READ_WRITE, nbytes, None)
        self._host = host

    @classmethod
    def from_array(cls, ctx, q, a):
        a = np.ascontiguousarray(a)
        b = cls(ctx, a.nbytes)
        if a.nbytes:
            call(lib.ccl_buffer_enqueue_write, b.h, q.h, 1, 0, a.nbytes, np_ptr(a), None)
        return b

    def read(self, q, dtype, count):
        out = np.empty(count, dtype=dtype)
        if out.nbytes:
            call(lib.ccl_buffer_enqueue_read, self.h, q.h, 1, 0, out.nbytes, np_ptr(out), None)
        return out

    def write(self, q, a):
        a = np.ascontiguousarray(a)
        call(lib.ccl_buffer_enqueue_write, self.h, q.h, 1, 0, a.nbytes, np_ptr(a), None)

    @property
    def ptr(self):
        return lib.ccl_buffer_unwrap(self.h)

    def destroy(self):
        if self.h:
            lib.ccl_buffer_destroy(self.h)
            self.h = None


def wait(evt):
    """Blocks on one event (ccl_event_wait over a one-element list)."""
    ewl = C.c_void_p(None)
    lib.ccl_ewl(C.byref(ewl), C.c_void_p(evt), C.c_void_p(None))
    call(lib.ccl_event_wait, C.byref(ewl))


class Sorter:
    def __init__(self, ctx, algo, elem_type, key_type=None, options=None,
                 compare=None, get_key=None, compiler_opts=None):
        et = C.c_int(elem_type)
        kt = C.c_int(key_type) if key_type is not None else None
        self.h = call(lib.clo_sort_new, algo.encode(),
                      options.encode() if options else None, ctx.h, C.byref(et),
                      C.byref(kt) if kt is not None else None,
                      compare.encode() if compare else None,
                      get_key.encode() if get_key else None,
                      compiler_opts.encode() if compiler_opts else None)
        self.elem_type = elem_type

    def sort_device(self, q, buf_in, numel, buf_out=None, lws_max=0, q_comm=None):
        return call(lib.clo_sort_with_device_data, self.h, q.h,
                    q_comm.h if q_comm else None, buf_in.h,
                    buf_out.h if buf_out else None, numel, lws_max)

    def sort_host(self, q, a, out=None, lws_max=0, q_comm=None):
        a = np.ascontiguousarray(a)
        o = a if out is None else out
        call(lib.clo_sort_with_host_data, self.h, q.h if q else None,
             q_comm.h if q_comm else None, np_ptr(a), np_ptr(o), a.size, lws_max)
        return o

    def sort_kv_device(self, q, kbuf, vbuf, value_type, numel):
        return call(lib.clo_sort_kv_with_device_data, self.h, q.h, kbuf.h, vbuf.h,
                    value_type, numel)

    def sort_kv_host(self, q, keys, vals, value_type):
        call(lib.clo_sort_kv_with_host_data, self.h, q.h if q else None,
             np_ptr(keys), np_ptr(vals), value_type, keys.size)

    def sort_segmented_device(self, q, buf, off_buf, nseg):
        return call(lib.clo_sort_segmented_with_device_data, self.h, q.h, buf.h,
                    off_buf.h if off_buf else None, nseg)

    def sort_segmented_host(self, q, a, offsets):
        a = np.ascontiguousarray(a)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        call(lib.clo_sort_segmented_with_host_data, self.h, q.h if q else None,
             np_ptr(a), a.size, np_ptr(off), off.size - 1)
        return a

    def tune_segmented(self, q, buf, off_buf, nseg):
        """(chosen variant, per-variant ms)."""
        times = (C.c_double * SEG_SORT_VARIANTS)()
        v = call(lib.clo_sort_segmented_tune, self.h, q.h, buf.h, off_buf.h, nseg, times)
        return v, list(times)

    @property
    def seg_variant(self):
        return lib.clo_sort_segmented_get_variant(self.h)

    def destroy(self):
        if self.h:
            lib.clo_sort_destroy(self.h)
            self.h = None


class Scanner:
    def __init__(self, ctx, elem_type, sum_type, algo="blelloch", options=None):
        self.h = call(lib.clo_scan_new, algo.encode(),
                      options.encode() if options else None, ctx.h, elem_type,
                      sum_type, None)

    def scan_device(self, q, buf_in, buf_out, numel, lws_max=0):
        return call(lib.clo_scan_with_device_data, self.h, q.h, None, buf_in.h,
                    buf_out.h, numel, lws_max)

    def scan_host(self, q, a, out, lws_max=0):
        call(lib.clo_scan_with_host_data, self.h, q.h if q else None, None,
             np_ptr(a), np_ptr(out), a.size, lws_max)
        return out

    def scan_segmented_device(self, q, buf_in, buf_out, off_buf, nseg):
        return call(lib.clo_scan_segmented_with_device_data, self.h, q.h, buf_in.h,
                    buf_out.h, off_buf.h if off_buf else None, nseg)

    def scan_segmented_host(self, q, a, out, offsets):
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        call(lib.clo_scan_segmented_with_host_data, self.h, q.h if q else None,
             np_ptr(a), np_ptr(out), a.size, np_ptr(off), off.size - 1)
        return out

    def destroy(self):
        if self.h:
            lib.clo_scan_destroy(self.h)
            self.h = None


class Graph:
    """Work enqueued on a queue between begin() and end(), replayed by
    launch()."""

    def __init__(self, q):
        self.q = q
        self.h = None

    def begin(self):
        call(lib.clo_queue_begin_capture, self.q.h)

    def end(self):
        self.h = call(lib.clo_queue_end_capture, self.q.h)
        return self

    def launch(self, q=None):
        call(lib.clo_graph_launch, self.h, (q or self.q).h)

    @property
    def num_nodes(self):
        return int(lib.clo_graph_get_num_nodes(self.h))

    def destroy(self):
        if self.h:
            lib.clo_graph_destroy(self.h)
            self.h = None


class Program:
    """A client program built from CUDA source (ccl_program_new_from_source
    + ccl_program_build), e.g. around the text of Rng.source()."""

    def __init__(self, ctx, src, options=None):
        self.h = call(lib.ccl_program_new_from_source, ctx.h, src.encode())
        try:
            call(lib.ccl_program_build, self.h, options.encode() if options else None)
        except CloError:
            self.destroy()
            raise

    def kernel(self, name):
        return call(lib.ccl_program_get_kernel, self.h, name.encode())

    @staticmethod
    def suggest(kernel, real, want_gws=False):
        """(gws or None, lws) as ccl_kernel_suggest_worksizes gives them."""
        r, g, l_ = SZ(real), SZ(0), SZ(0)
        call(lib.ccl_kernel_suggest_worksizes, kernel, None, 1, C.byref(r),
             C.byref(g) if want_gws else None, C.byref(l_))
        return (g.value if want_gws else None), l_.value

    @staticmethod
    def enqueue(kernel, q, gws, lws, *args):
        """Launches kernel over gws work-items in groups of lws; args are
        Buffers or raw CCLBuffer handles (their device pointers) or
        (ctypes type, value) pairs."""
        items = []
        for a in args:
            if isinstance(a, Buffer):
                items.append(C.c_void_p(a.h))
            elif isinstance(a, int):  # a raw CCLBuffer handle
                items.append(C.c_void_p(a))
            else:
                ct, v = a
                val = ct(v)
                items.append(C.c_void_p(lib.ccl_arg_new(C.byref(val), C.sizeof(val))))
        g = SZ(gws)
        l_ = SZ(lws) if lws else None
        e = err_ptr()
        evt = lib.ccl_kernel_set_args_and_enqueue_ndrange(
            C.c_void_p(kernel), C.c_void_p(q.h), C.c_uint(1), None, C.byref(g),
            C.byref(l_) if l_ is not None else None, None, C.byref(e), *items, None)
        check(e, "ccl_kernel_set_args_and_enqueue_ndrange")
        return evt

    def destroy(self):
        if self.h:
            lib.ccl_program_destroy(self.h)
            self.h = None


class Rng:
    def __init__(self, ctx, q, name, seed_type, count, main_seed=0, hash=None,
                 seeds=None):
        self.count = count
        self.name = name
        if seed_type == CLO_RNG_SEED_EXT_HOST and seeds is not None:
            arr = np.ascontiguousarray(seeds)
            sp = np_ptr(arr)
        elif seed_type == CLO_RNG_SEED_EXT_DEV and seeds is not None:
            sp = C.c_void_p(seeds.h)
        else:
            sp = None
        self.h = call(lib.clo_rng_new, name.encode(), seed_type, sp, count,
                      main_seed, hash.encode() if hash is not None else None,
                      ctx.h, q.h)

    @property
    def seeds_buffer(self):
        return lib.clo_rng_get_device_seeds(self.h)

    def source(self):
        """The CUDA text for client kernels (clo_rng_get_source)."""
        return lib.clo_rng_get_source(self.h).decode()

    def states(self, q):
        size = lib.clo_rng_get_size(self.h)
        out = np.empty(size, dtype=np.uint8)
        if size:
            call(lib.ccl_buffer_enqueue_read, self.seeds_buffer, q.h, 1, 0, size,
                 np_ptr(out), None)
        return out

    def fill(self, q, out_buf, draws, bits=32, maxint=0):
        return call(lib.clo_rng_fill, self.h, q.h, out_buf.h, draws, bits, maxint)

    def destroy(self):
        if self.h:
            lib.clo_rng_destroy(self.h)
            self.h = None


def launch_count():
    return int(lib.clo_gb300_launch_count())


def kernel_timing(name):
    """(total_ms, total_algorithmic_bytes, launches) of one kernel."""
    ms, by, n = C.c_double(), C.c_double(), U64()
    if not lib.clo_gb300_timing_get(name.encode(), C.byref(ms), C.byref(by), C.byref(n)):
        return 0.0, 0.0, 0
    return ms.value, by.value, int(n.value)


class Server:
    """CloServer: continuous batching of host-data requests on one GPU."""

    def __init__(self, ctx, budget_bytes, streams=4):
        self.h = call(lib.clo_serve_new, ctx.h, budget_bytes, streams)

    @staticmethod
    def request(op, type_=0, sum_type=0, n=0, draws=0, rng=0, inp=None, out=None,
                device=False):
        """inp / out: numpy arrays or raw addresses (host memory), or, with
        device=True, device addresses on the server's GPU (Buffer.ptr)."""
        def addr(x):
            if x is None:
                return None
            return x.ctypes.data if isinstance(x, np.ndarray) else int(x)
        return ServeRequest(op, type_, sum_type, n, draws, rng, addr(inp), addr(out),
                            1 if device else 0)

    def submit(self, req):
        return call(lib.clo_serve_submit, self.h, C.byref(req))

    def wait(self, ticket):
        ms = C.c_double()
        call(lib.clo_serve_wait, self.h, ticket, C.byref(ms))
        return ms.value

    def drain(self):
        call(lib.clo_serve_drain, self.h)

    def replay(self, reqs, arrival_s):
        n = len(reqs)
        arr = (ServeRequest * n)(*reqs)
        ts = (C.c_double * n)(*arrival_s)
        tickets = (U64 * n)()
        call(lib.clo_serve_replay, self.h, arr, ts, n, tickets)
        return list(tickets)

    def configure(self, small_n=1 << 20, batch_elems=1 << 26, max_batch=4096):
        """Batching policy (clo_serve_configure); max_batch=1 turns it off."""
        call(lib.clo_serve_configure, self.h, small_n, batch_elems, max_batch)

    def stats(self):
        st = ServeStats()
        lib.clo_serve_get_stats(self.h, C.byref(st))
        return st.as_dict()

    def reset_stats(self):
        lib.clo_serve_reset_stats(self.h)

    def destroy(self):
        if self.h:
            lib.clo_serve_destroy(self.h)
            self.h = None
