"""Admission and batching policy of the serving layer (clo_serve_select,
clo_serve_footprint): pure host logic, no device work."""
import ctypes as C

import pytest

SORT, SCAN, RNG = 0, 1, 2
UINT, ULONG, INT = 5, 7, 4


@pytest.fixture(scope="module")
def lib(clops):
    return clops


def req(clops, op, n, type_=UINT, sum_type=ULONG, draws=0, rng=0, device=False):
    return clops.Server.request(op, type_, sum_type, n, draws, rng, inp=16, out=16,
                                device=device)


def select(clops, reqs, free, small_n=1 << 20, batch_elems=1 << 26, max_batch=64):
    arr = (clops.ServeRequest * len(reqs))(*reqs)
    out = (C.c_size_t * max_batch)()
    k = clops.lib.clo_serve_select(arr, len(reqs), free, small_n, batch_elems, max_batch, out)
    return list(out[:k])


def fp(clops, r):
    return clops.lib.clo_serve_footprint(C.byref(r))


def test_footprints(lib):
    s = req(lib, SORT, 1000)
    assert fp(lib, s) >= 2 * 1000 * 4
    assert fp(lib, req(lib, SORT, 1000, type_=ULONG)) > fp(lib, s)
    assert fp(lib, req(lib, SCAN, 1000)) >= 1000 * 12
    assert fp(lib, req(lib, RNG, 1000, draws=16, rng=3)) >= 1000 * 8 + 1000 * 16 * 4
    # malformed: no buffers, float types, unknown generator, zero draws
    bad = lib.Server.request(SORT, UINT, 0, 10)
    assert fp(lib, bad) == 0
    assert fp(lib, req(lib, SORT, 10, type_=9)) == 0
    assert fp(lib, req(lib, RNG, 10, draws=4, rng=9)) == 0
    assert fp(lib, req(lib, RNG, 10, draws=0, rng=1)) == 0


def test_fifo_head_blocks_when_it_does_not_fit(lib):
    big, small = req(lib, SORT, 1 << 24), req(lib, SORT, 100)
    assert select(lib, [big, small], fp(lib, big) - 1) == []
    assert select(lib, [big, small], fp(lib, big)) == [0]  # big is not batched


def test_small_same_kind_requests_batch_in_order(lib):
    reqs = [req(lib, SORT, 100), req(lib, SCAN, 50), req(lib, SORT, 200),
            req(lib, SORT, 300, type_=ULONG), req(lib, SORT, 1 << 21), req(lib, SORT, 400)]
    assert select(lib, reqs, 1 << 40) == [0, 2, 5]
    assert select(lib, reqs[1:], 1 << 40) == [0]          # the scan alone
    scans = [req(lib, SCAN, 10), req(lib, SCAN, 10, sum_type=UINT), req(lib, SCAN, 10)]
    assert select(lib, scans, 1 << 40) == [0, 2]           # sum types must match


def test_batch_limits(lib):
    reqs = [req(lib, SORT, 1000) for _ in range(10)]
    assert len(select(lib, reqs, 1 << 40, max_batch=4)) == 4
    assert len(select(lib, reqs, 1 << 40, batch_elems=3500)) == 3
    one = fp(lib, reqs[0])
    assert len(select(lib, reqs, 2 * one + one // 2)) == 2
    assert select(lib, [req(lib, RNG, 100, draws=2, rng=1)] * 3, 1 << 40) == [0]


def test_device_and_host_requests_batch_apart(lib):
    reqs = [req(lib, SORT, 100), req(lib, SORT, 100, device=True), req(lib, SORT, 100),
            req(lib, SORT, 100, device=True)]
    assert select(lib, reqs, 1 << 40) == [0, 2]
    assert select(lib, reqs[1:], 1 << 40) == [0, 2]
    # the same footprint either way (the device-resident form is charged
    # as much as the host one)
    assert fp(lib, reqs[0]) == fp(lib, reqs[1])
