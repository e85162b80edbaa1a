"""The no-allocation scan entry point (clo_scan_blelloch_noalloc).

For callers that cannot allocate device memory when they scan (inside
another thread's global-mode graph capture, under a fixed device budget,
or in loops that cannot afford an allocation that may synchronise). It
keeps its scratch in a static device array of the library, so two calls
in a row must both match the allocating entry point
(clo_scan_with_device_data) exactly: the second call must not see the
first call's tile statuses. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from inputs import splitmix64

pytestmark = pytest.mark.gpu


def _noalloc(clops):
    f = clops.lib.clo_scan_blelloch_noalloc
    f.restype = C.c_uint32
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t,
                  C.POINTER(C.POINTER(clops.GError))]
    return f


@pytest.mark.parametrize("in_type,in_dt,sum_type,sum_dt,first_n", [
    (5, np.uint32, 7, np.uint64, 1 << 28),        # uint -> ulong, every scratch slot
    (0, np.int8, 5, np.uint32, (1 << 20) + 7),    # char -> uint
])
def test_noalloc_scan_matches_allocating_scan_twice(clops, in_type, in_dt, sum_type, sum_dt,
                                                    first_n):
    f = _noalloc(clops)
    ctx = clops.Context(0)
    q = clops.Queue(ctx)
    try:
        # Two calls in a row: the first uses more tiles than the second (at
        # 2^28 elements, all 2^15 tile slots of the scratch, the last one
        # beside the tile counter). Each result must equal the allocating
        # entry point's and the oracle's serial scan.
        for n, seed in ((first_n, 45), (123457, 46)):
            raw = splitmix64(seed, n) >> np.uint64(40)
            a = raw.astype(np.uint64).astype(in_dt) if in_dt != np.int8 else \
                (raw & np.uint64(0xFF)).astype(np.uint8).view(np.int8)
            bi = clops.Buffer.from_array(ctx, q, a)
            ref = clops.Buffer(ctx, n * np.dtype(sum_dt).itemsize)
            got = clops.Buffer(ctx, n * np.dtype(sum_dt).itemsize)
            sc = clops.Scanner(ctx, in_type, sum_type)
            clops.wait(sc.scan_device(q, bi, ref, n))
            ok = clops.call(f, q.h, in_type, sum_type, bi.ptr, got.ptr, n)
            assert ok == 1
            q.finish()
            out = got.read(q, sum_dt, n)
            np.testing.assert_array_equal(out, ref.read(q, sum_dt, n))
            np.testing.assert_array_equal(out, oracle.scan(a, in_type, sum_dt))
            for x in (bi, ref, got, sc):
                x.destroy()
        # Beyond the static scratch: rejected before any device work.
        with pytest.raises(clops.CloError) as ei:
            clops.call(f, q.h, in_type, sum_type, C.c_void_p(16), C.c_void_p(16),
                       (1 << 28) + 1)
        assert ei.value.code == clops.CLO_ERROR_ARGS
    finally:
        q.destroy()
        ctx.destroy()
