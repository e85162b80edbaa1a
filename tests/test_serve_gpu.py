"""Serving layer on the GPU: every request of a concurrent mix (batched
sorts and scans of many sizes and types, random fills) gives the oracle's
result -- the result it gets when served alone -- and admission keeps the
held bytes within the budget."""
import numpy as np
import pytest

import oracle
from inputs import keys_of_type, splitmix64

pytestmark = pytest.mark.gpu

NAMES = ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller", "tauslcg"]
TYPES = [(5, np.uint32), (7, np.uint64), (4, np.int32), (1, np.uint8), (3, np.uint16)]


def make_requests(clops, count, seed, max_log2=18):
    """(request, expected output, output array) triples."""
    u = splitmix64(seed, 4 * count)
    out = []
    for i in range(count):
        kind = int(u[4 * i] % np.uint64(10))
        n = int(1 << int(u[4 * i + 1] % np.uint64(max_log2 + 1)))
        n = max(1, n - int(u[4 * i + 2] % np.uint64(max(n // 2, 1))))
        code, dt = TYPES[int(u[4 * i + 3] % np.uint64(len(TYPES)))]
        if kind < 6:
            a = keys_of_type(1000 + i, n, dt)
            dst = np.empty_like(a)
            r = clops.Server.request(clops.SERVE_SORT, code, 0, n, inp=a, out=dst)
            out.append((r, oracle.radix_sort(a), dst, a))
        elif kind < 9:
            a = keys_of_type(2000 + i, n, dt)
            sum_code, sum_dt = (7, np.uint64) if i % 2 else (5, np.uint32)
            dst = np.zeros(n, sum_dt)
            r = clops.Server.request(clops.SERVE_SCAN, code, sum_code, n, inp=a, out=dst)
            out.append((r, oracle.scan(a, code, sum_dt), dst, a))
        else:
            name = NAMES[i % len(NAMES)]
            states = max(1, n // 16)
            draws = 1 + i % 7
            seeds = splitmix64(3000 + i, states * oracle.SEED_SIZE[name] // 4 + 2)
            seeds = seeds.view(np.uint8)[:states * oracle.SEED_SIZE[name]].copy()
            if name == "parkmiller":
                w = seeds.view(np.uint32)
                w[:] = (w % np.uint32(2147483646)) + np.uint32(1)
            dst = np.zeros(states * draws, np.uint32)
            r = clops.Server.request(clops.SERVE_RNG_FILL, 0, 0, states, draws,
                                     oracle.GEN[name], inp=seeds, out=dst)
            exp, _ = oracle.rng_fill(name, seeds, states, draws)
            out.append((r, exp, dst, seeds))
    return out


def test_serve_mix_matches_oracle_and_alone(clops, ctx):
    reqs = make_requests(clops, 240, seed=70)
    srv = clops.Server(ctx, 8 << 30, streams=4)
    tickets = [srv.submit(r) for r, _, _, _ in reqs]
    lat = [srv.wait(t) for t in tickets]
    srv.drain()
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] < len(reqs)          # small requests were batched
    assert min(lat) > 0 and st["p99_ms"] >= st["p50_ms"] > 0
    mixed = []
    for r, exp, dst, _ in reqs:
        np.testing.assert_array_equal(dst, exp)
        mixed.append(dst.copy())
        dst[:] = 0
    # The same requests one at a time: identical results.
    for (r, _, dst, _), m in zip(reqs, mixed):
        srv.wait(srv.submit(r))
        np.testing.assert_array_equal(dst, m)
    srv.destroy()


def test_serve_admission_small_budget_and_rejection(clops, ctx):
    budget = 24 << 20
    srv = clops.Server(ctx, budget, streams=2)
    arrs = [keys_of_type(80 + i, 1 << 20, np.uint32) for i in range(24)]
    outs = [np.empty_like(a) for a in arrs]
    reqs = [clops.Server.request(clops.SERVE_SORT, 5, 0, a.size, inp=a, out=o)
            for a, o in zip(arrs, outs)]
    tickets = srv.replay(reqs, [0.0] * len(reqs))
    assert all(t > 0 for t in tickets)
    srv.drain()
    st = srv.stats()
    assert st["completed"] == 24 and st["peak_bytes"] <= budget
    assert st["max_queued"] > 1
    for a, o in zip(arrs, outs):
        np.testing.assert_array_equal(o, np.sort(a))
    big = np.zeros(1 << 23, np.uint32)
    with pytest.raises(clops.CloError) as ei:
        srv.submit(clops.Server.request(clops.SERVE_SORT, 5, 0, big.size, inp=big, out=big))
    assert ei.value.code == clops.CLO_ERROR_ARGS
    assert srv.stats()["rejected"] == 1
    srv.destroy()


def test_serve_open_loop_replay_latency(clops, ctx):
    reqs = make_requests(clops, 120, seed=71, max_log2=16)
    srv = clops.Server(ctx, 4 << 30, streams=4)
    arrivals = list(np.cumsum(np.full(len(reqs), 2e-4)))
    tickets = srv.replay([r for r, _, _, _ in reqs], arrivals)
    srv.drain()
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["span_s"] >= arrivals[-1] * 0.9
    for r, exp, dst, _ in reqs:
        np.testing.assert_array_equal(dst, exp)
    assert all(t > 0 for t in tickets)
    srv.destroy()


def to_device(clops, ctx, q, reqs):
    """The same requests with device-resident buffers: (request, expected,
    input buffer, output buffer, output dtype, count, input array)."""
    out = []
    for r, exp, dst, a in reqs:
        bi = clops.Buffer.from_array(ctx, q, a)
        bo = clops.Buffer(ctx, max(dst.nbytes, 1))
        rd = clops.Server.request(r.op, r.type, r.sum_type, r.n, r.draws, r.rng,
                                  inp=bi.ptr, out=bo.ptr, device=True)
        out.append((rd, exp, bi, bo, dst.dtype, dst.size, a))
    return out


def test_serve_device_resident_mix_matches_oracle_and_alone(clops, ctx, queue):
    reqs = to_device(clops, ctx, queue, make_requests(clops, 200, seed=72))
    srv = clops.Server(ctx, 8 << 30, streams=4)
    tickets = [srv.submit(r[0]) for r in reqs]
    for t in tickets:
        srv.wait(t)
    srv.drain()
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] < len(reqs)          # small requests were batched
    mixed = []
    for rd, exp, bi, bo, dt, cnt, a in reqs:
        got = bo.read(queue, dt, cnt)
        np.testing.assert_array_equal(got, exp)
        np.testing.assert_array_equal(bi.read(queue, a.dtype, a.size), a)  # input only read
        mixed.append(got)
    for (rd, _, _, bo, dt, cnt, _), m in zip(reqs, mixed):
        bo.write(queue, np.zeros(cnt, dt))
        srv.wait(srv.submit(rd))
        np.testing.assert_array_equal(bo.read(queue, dt, cnt), m)
    srv.destroy()
    for r in reqs:
        r[2].destroy()
        r[3].destroy()


def test_serve_host_and_device_requests_together(clops, ctx, queue):
    host = make_requests(clops, 60, seed=73, max_log2=14)
    dev = to_device(clops, ctx, queue, make_requests(clops, 60, seed=74, max_log2=14))
    srv = clops.Server(ctx, 2 << 30, streams=3)
    order = []
    for h, d in zip(host, dev):
        order.append(srv.submit(h[0]))
        order.append(srv.submit(d[0]))
    srv.drain()
    assert srv.stats()["completed"] == 120 and srv.stats()["failed"] == 0
    for _, exp, dst, _ in host:
        np.testing.assert_array_equal(dst, exp)
    for rd, exp, bi, bo, dt, cnt, _ in dev:
        np.testing.assert_array_equal(bo.read(queue, dt, cnt), exp)
        bi.destroy()
        bo.destroy()
    srv.destroy()


def test_batches_overlap_on_the_device_with_four_streams(clops, ctx):
    """Requests that arrive together run as batches on the server's 4
    streams at the same time: the device intervals of at least two batches
    overlap (each interval runs from an event recorded before the batch's
    first operation to one after its last, on its stream). Each result
    still equals the oracle's."""
    n = 1 << 22  # above the batching limit: one request per batch
    a = [keys_of_type(4000 + i, n, np.uint32) for i in range(16)]
    dst = [np.empty_like(x) for x in a]
    pinned = []
    for x in a + dst:  # page-locked, so the copies are asynchronous
        addr = clops.lib.clo_host_alloc(x.nbytes, None)
        pinned.append((addr, np.ctypeslib.as_array((clops.C.c_uint32 * n).from_address(addr))))
    for (addr, arr), x in zip(pinned[:16], a):
        arr[:] = x
    srv = clops.Server(ctx, 8 << 30, streams=4)
    try:
        tickets = [srv.submit(clops.Server.request(clops.SERVE_SORT, 5, 0, n, inp=pi[0],
                                                   out=po[0]))
                   for pi, po in zip(pinned[:16], pinned[16:])]
        for t in tickets:
            srv.wait(t)
        st = srv.stats()
        assert st["completed"] == 16 and st["batches"] == 16
        assert st["max_concurrent_batches"] >= 2, st
        assert st["mean_concurrent_batches"] > 1.0, st
        assert 0 < st["device_busy_s"] <= st["span_s"] + 1e-3
        for (_, arr), x in zip(pinned[16:], a):
            np.testing.assert_array_equal(arr, oracle.radix_sort(x))
    finally:
        srv.destroy()
        for addr, arr in pinned:
            del arr
        for addr, _ in pinned:
            clops.lib.clo_host_free(addr)


def test_batching_off_runs_every_request_alone(clops, ctx):
    """max_batch = 1: every request is its own batch (the plain kernels),
    with the same results as batched serving."""
    reqs = make_requests(clops, 60, seed=71, max_log2=14)
    srv = clops.Server(ctx, 8 << 30, streams=1)
    try:
        srv.configure(max_batch=1)
        for t in [srv.submit(r) for r, _, _, _ in reqs]:
            srv.wait(t)
        st = srv.stats()
        assert st["batches"] == 60 and st["max_concurrent_batches"] == 1
        for _, exp, dst, _ in reqs:
            np.testing.assert_array_equal(dst, exp)
        with pytest.raises(clops.CloError):
            srv.configure(max_batch=0)
    finally:
        srv.destroy()
