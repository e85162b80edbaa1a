#!/usr/bin/env python3
"""Benchmark of the cl_ops hot path on GB300.

Headline workload: "satradix" sort of 2^28 uint32 keys drawn uniformly
from splitmix64 (seed 42), keys only, through the C-ABI
(clo_sort_with_device_data). One step = one full sort of a resident
2^28-key array; every step sorts its own copy of the input (1 GiB each,
larger than L2), so the timed region is exactly K sorts back to back.

  value     Gkeys/s over the timed region (device events on the library
            queue), summed over ranks (replicas; no collective).
  e2e       the same metric through clo_sort_with_host_data from pinned
            host memory: host->device copy, sort and device->host copy in
            every step.
  roofline  live per-launch device time of the dominant kernel
            (satradix_onesweep) against its algorithmic bytes.
  suite     the other large-size primitives (abitonic 2^26 uint32,
            satradix 2^27 (uint64, uint32) pairs, blelloch scan 2^30
            uint32 -> uint64, the five RNGs 2^24 states x 64 draws),
            informational.
  cpu_baseline  the CPU restatement (LSD radix, radix 16 as the reference
            default, all host threads) on a 2^24-key sample.

`--impl reference` times the reference's algorithm on the host cores
instead (the reference itself needs an OpenCL runtime, GLib and cf4ocl2,
none of which exist here); only rank 0 works under torchrun.
"""
import argparse
import gc
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "cl-ops_gb300"))
sys.path.insert(0, str(ROOT / "tests"))

METRIC = "Gkeys/s (radix/bitonic), scan GB/s vs HBM peak; batched vs plain on 1 GB300"
WORKLOAD = "satradix sort, 2^28 uint32 keys, uniform splitmix64 seed 42, keys only"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Host-side barrier and max-reduction across ranks (gloo, CPU only)."""

    def __init__(self, rank, world):
        self.rank, self.world = rank, world
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist
            self.pg = True

    def barrier(self):
        if self.pg:
            self.dist.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.dist.destroy_process_group()


def keys_u32_chunked(seed, n, chunk=1 << 24):
    from inputs import splitmix64
    out = np.empty(n, dtype=np.uint32)
    for o in range(0, n, chunk):
        m = min(chunk, n - o)
        out[o:o + m] = (splitmix64(seed, m, offset=o) >> np.uint64(32)).astype(np.uint32)
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# HBM bandwidth of the GB300 specification, the secondary denominator.
SPEC_HBM_GBS = 8000.0


def ncu_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture, if committed."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        # Keep only samples taken once the timed region has begun: wait for
        # nvidia-smi's first line, then drop it.
        t0 = time.time()
        while not self.lines and time.time() - t0 < 5 and self.proc.poll() is None:
            time.sleep(0.01)
        self.lines.clear()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def timed_region(clops, q, steps_fn, k):
    """Runs steps_fn(i) for i in range(k) between two queue markers and
    returns the device milliseconds between them."""
    m0 = q.marker()
    for i in range(k):
        steps_fn(i)
    m1 = q.marker()
    return clops.Queue.elapsed_ms(m0, m1)


def run_ours(args):
    rank, world, local = dist_env()
    dist = Dist(rank, world)
    import clops
    ctx = clops.Context(local)
    q = clops.Queue(ctx, profiling=True)
    n = 1 << args.log2n
    K, W = args.steps, args.warmup

    keys = keys_u32_chunked(42, n)
    src = clops.Buffer.from_array(ctx, q, keys)
    bufs = [clops.Buffer(ctx, keys.nbytes) for _ in range(K + W)]
    for b in bufs:
        clops.call(clops.lib.ccl_buffer_enqueue_copy, src.h, b.h, q.h, 0, 0, keys.nbytes, None)
    q.finish()
    sorter = clops.Sorter(ctx, "satradix", clops.CLO_UINT)

    for i in range(W):
        sorter.sort_device(q, bufs[i], n)
    q.finish()
    q.gc()

    clops.lib.clo_gb300_timing_enable(1)
    clops.lib.clo_gb300_timing_reset()
    launches0 = clops.launch_count()
    dist.barrier()
    q.finish()
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_region(clops, q, lambda i: sorter.sort_device(q, bufs[W + i], n), K)
    q.finish()
    clk = clocks.stop()
    launches = clops.launch_count() - launches0
    dist.barrier()
    ms_max = dist.max(ms)
    one_ms, one_bytes, one_n = clops.kernel_timing("satradix_onesweep")
    up_ms, _, up_n = clops.kernel_timing("satradix_upsweep")
    clops.lib.clo_gb300_timing_enable(0)

    # Check the last step's output before reporting (sortedness + multiset).
    got = bufs[-1].read(q, np.uint32, n)
    ok = bool(np.all(got[1:] >= got[:-1])) and int(got.sum(dtype=np.uint64)) == \
        int(keys.sum(dtype=np.uint64))
    for b in bufs:
        b.destroy()
    src.destroy()
    q.gc()

    # ---- end to end: pinned host in/out, blocking host-data call ------------
    e2e_steps = K
    hin = clops.lib.clo_host_alloc(keys.nbytes, None)
    hout = clops.lib.clo_host_alloc(keys.nbytes, None)
    ain = np.ctypeslib.as_array((clops.C.c_uint32 * n).from_address(hin))
    aout = np.ctypeslib.as_array((clops.C.c_uint32 * n).from_address(hout))
    ain[:] = keys
    for _ in range(2):
        sorter.sort_host(q, ain, aout)
    gc.collect()
    dist.barrier()
    t0 = time.perf_counter()
    e2e_marks = []
    for _ in range(e2e_steps):
        sorter.sort_host(q, ain, aout)
        e2e_marks.append(time.perf_counter())
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_step_ms = np.diff(np.array([t0] + e2e_marks)) * 1e3
    ok = ok and bool(np.all(aout[1:] >= aout[:-1]))
    del ain, aout
    clops.lib.clo_host_free(hin)
    clops.lib.clo_host_free(hout)

    suite = run_suite(clops, ctx, q, args) if (args.suite and rank == 0) else None

    peak, peak_kind = measured_peaks()
    achieved = (one_bytes / one_n) / (one_ms / one_n * 1e-3) / 1e9 if one_n else None
    traffic = ncu_traffic("satradix_onesweep_2pow28_u32.txt")
    out = {
        "metric": METRIC,
        "value": round(world * n * K / (ms_max * 1e-3) / 1e9, 3),
        "unit": "Gkeys/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(ms_max / K, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u32",
        "data": "synthetic (splitmix64 seed 42, uniform over [0, 2^32))",
        "config": bench_config(n, world, ok),
        "e2e": {"value": round(world * n * e2e_steps / e2e_s / 1e9, 3), "unit": "Gkeys/s",
                "step_ms": {"min": round(float(e2e_step_ms.min()), 3),
                            "median": round(float(np.median(e2e_step_ms)), 3),
                            "max": round(float(e2e_step_ms.max()), 3)},
                "h2d_bytes_per_step": n * 4, "d2h_bytes_per_step": n * 4,
                "api": "clo_sort_with_host_data, pinned host buffers"},
        "gpu_launches": int(launches),
        "roofline": {
            "kernel": "satradix_onesweep",
            "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None,
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4) if achieved else None,
            "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
            "traffic": traffic,
            "algorithmic_bytes_per_launch": one_bytes / one_n if one_n else None,
            "launches": one_n,
            "avg_launch_ms": round(one_ms / one_n, 4) if one_n else None,
            "upsweep_avg_ms": round(up_ms / up_n, 4) if up_n else None,
            "whole_sort_model": "36 B/key (4 B upsweep + 4 passes x 8 B)",
            "whole_sort_frac": round((36.0 * n * K / (ms / 1e3) / 1e9) / peak, 4),
            # The same fractions against the 8 TB/s specification, and the
            # whole sort against its n x 8 B lower bound (one read and one
            # write of the keys).
            "spec_peak": SPEC_HBM_GBS,
            "frac_of_spec": round(achieved / SPEC_HBM_GBS, 4) if achieved else None,
            "whole_sort_frac_of_spec": round((36.0 * n * K / (ms / 1e3) / 1e9) / SPEC_HBM_GBS, 4),
            "lower_bound_8B_per_key_frac": round((8.0 * n * K / (ms / 1e3) / 1e9) / peak, 4),
        },
        "clocks": clk,
    }
    if suite is not None:
        out["suite"] = suite
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(out), flush=True)
    sorter.destroy()
    q.destroy()
    ctx.destroy()
    dist.close()


def run_suite(clops, ctx, q, args, only=None):
    """The other large-size primitives, 2 warm-up + 3 timed calls each
    (`only` selects one of them)."""
    from inputs import splitmix64, keys_u64
    res = {}
    peak, _ = measured_peaks()

    def timed(fn, reps=3, warm=2):
        for _ in range(warm):
            fn()
        q.finish()
        return timed_region(clops, q, lambda i: fn(), reps) / reps

    def copy(src, dst, nbytes):
        clops.call(clops.lib.ccl_buffer_enqueue_copy, src.h, dst.h, q.h, 0, 0, nbytes, None)

    def abitonic():
        n = 1 << 26
        a = keys_u32_chunked(44, n)
        b = clops.Buffer.from_array(ctx, q, a)
        pristine = clops.Buffer.from_array(ctx, q, a)
        s = clops.Sorter(ctx, "abitonic", clops.CLO_UINT)
        ms_copy = timed(lambda: copy(pristine, b, a.nbytes))
        ms = timed(lambda: (copy(pristine, b, a.nbytes), s.sort_device(q, b, n))) - ms_copy
        # For uint32 keys the network's output is the ascending order.
        ok = bool(np.array_equal(b.read(q, np.uint32, n), np.sort(a)))
        res["abitonic_2pow26_u32"] = {
            "Gkeys/s": round(n / (ms * 1e-3) / 1e9, 3), "ms": round(ms, 3),
            "canonical_bytes_GB": 17.7,
            "frac_of_peak_canonical": round(17.7e9 / (ms * 1e-3) / 1e9 / peak, 4),
            "result_check": "equal to np.sort" if ok else "FAILED"}
        for x in (s, b, pristine):
            x.destroy()

    def kv():
        n = 1 << (27 if only is None else min(args.log2n, 27))
        k = keys_u64(43, n)
        v = np.arange(n, dtype=np.uint32)
        kp, vp = clops.Buffer.from_array(ctx, q, k), clops.Buffer.from_array(ctx, q, v)
        kb, vb = clops.Buffer(ctx, k.nbytes), clops.Buffer(ctx, v.nbytes)
        s = clops.Sorter(ctx, "satradix", clops.CLO_ULONG)

        def restore():
            copy(kp, kb, k.nbytes)
            copy(vp, vb, v.nbytes)
        ms_copy = timed(restore)
        ms = timed(lambda: (restore(), s.sort_kv_device(q, kb, vb, clops.CLO_UINT, n))) - ms_copy
        # Values are the original indices. Keys ascending, values a
        # permutation carrying each key, and ties in index order: together
        # the stable sort's output exactly.
        gk, gv = kb.read(q, np.uint64, n), vb.read(q, np.uint32, n)
        same = gk[1:] == gk[:-1]
        ok = bool(np.all(gk[1:] >= gk[:-1]) and np.array_equal(k[gv], gk)
                  and np.all(np.bincount(gv, minlength=n) == 1)
                  and np.all(gv[1:][same] > gv[:-1][same]))
        res[f"satradix_kv_2pow{n.bit_length() - 1}_u64_u32"] = {
            "Gpairs/s": round(n / (ms * 1e-3) / 1e9, 3), "ms": round(ms, 3),
            "model_bytes_per_pair": 200,
            "frac_of_peak": round(200.0 * n / (ms * 1e-3) / 1e9 / peak, 4),
            "result_check": "stable sort of the pairs" if ok else "FAILED"}
        for x in (kp, vp, kb, vb, s):
            x.destroy()

    def scan():
        n = 1 << (30 if only is None else min(args.log2n, 30))
        a = np.empty(n, dtype=np.uint32)
        for o in range(0, n, 1 << 24):
            m = min(1 << 24, n - o)
            a[o:o + m] = (splitmix64(45, m, offset=o) >> np.uint64(56)).astype(np.uint32)
        bi = clops.Buffer.from_array(ctx, q, a)
        bo = clops.Buffer(ctx, n * 8)
        sc = clops.Scanner(ctx, clops.CLO_UINT, clops.CLO_ULONG)
        ms = timed(lambda: sc.scan_device(q, bi, bo, n))
        entry = {"GB/s": round(12.0 * n / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 3),
                 "frac_of_peak": round(12.0 * n / (ms * 1e-3) / 1e9 / peak, 4)}
        for x in (bi, bo):
            x.destroy()
        # End to end from page-locked host memory (clo_scan_with_host_data):
        # 4 B in and 8 B out per element over the host link.
        ne = min(n, 1 << 28)
        hin = clops.lib.clo_host_alloc(ne * 4, None)
        hout = clops.lib.clo_host_alloc(ne * 8, None)
        ain = np.ctypeslib.as_array((clops.C.c_uint32 * ne).from_address(hin))
        ain[:] = a[:ne]
        sc.scan_host(q, ain, np.ctypeslib.as_array((clops.C.c_uint64 * ne).from_address(hout)))
        t0 = time.perf_counter()
        for _ in range(3):
            clops.call(clops.lib.clo_scan_with_host_data, sc.h, q.h, None, hin, hout, ne, 0)
        dt = (time.perf_counter() - t0) / 3
        entry["e2e_host_data"] = {"n": ne, "ms": round(dt * 1e3, 2),
                                  "Gelem/s": round(ne / dt / 1e9, 2),
                                  "h2d_bytes": ne * 4, "d2h_bytes": ne * 8}
        del ain
        clops.lib.clo_host_free(hin)
        clops.lib.clo_host_free(hout)
        sc.destroy()
        res[f"blelloch_2pow{n.bit_length() - 1}_u32_u64"] = entry

    def rngs():
        # 2^24 states (with --only rng, 2^(log2n - 4) up to that: a small
        # case for profiling).
        count = 1 << (24 if only is None else min(24, max(args.log2n - 4, 10)))
        draws = 64
        out = clops.Buffer(ctx, count * draws * 4)
        for name in ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller"]:
            size = clops.RNG_SEED_SIZE[name]
            seeds = splitmix64(46, count * size // 8 + 1).view(np.uint8)[:count * size].copy()
            if name == "parkmiller":  # nonzero 31-bit states
                w = seeds.view(np.uint32)
                w[:] = (w % 2147483646) + 1
            rng = clops.Rng(ctx, q, name, clops.CLO_RNG_SEED_EXT_HOST, count, seeds=seeds)
            ms = timed(lambda: rng.fill(q, out, draws))
            byts = count * draws * 4 + 2 * count * size
            res[f"rng_{name}"] = {"Gdraws/s": round(count * draws / (ms * 1e-3) / 1e9, 2),
                                  "GB/s": round(byts / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 4),
                                  "frac_of_peak": round(byts / (ms * 1e-3) / 1e9 / peak, 4)}
            rng.destroy()
        out.destroy()

    def segmented():
        """50,000 segments, lognormal(7, 2) lengths clipped to [1, 2^22]
        (splitmix64 seed 48): the batched segmented sort and scan (a plain
        call and its CUDA-graph replay) against one plain call per segment."""
        from inputs import lognormal_lengths, offsets_of
        nseg = 50000 if only is None else min(50000, 1 << max(args.log2n - 13, 4))
        lens = lognormal_lengths(nseg, 7.0, 2.0, 1, 1 << 22, seed=48)
        off = offsets_of(lens)
        n = int(off[-1])
        keys = keys_u32_chunked(148, n)
        vals = np.empty(n, dtype=np.uint32)
        for o in range(0, n, 1 << 24):
            m = min(1 << 24, n - o)
            vals[o:o + m] = (splitmix64(248, m, offset=o) >> np.uint64(56)).astype(np.uint32)
        pristine = clops.Buffer.from_array(ctx, q, keys)
        b = clops.Buffer(ctx, keys.nbytes)
        ob = clops.Buffer.from_array(ctx, q, off)
        vi = clops.Buffer.from_array(ctx, q, vals)
        vo = clops.Buffer(ctx, n * 8)
        s = clops.Sorter(ctx, "satradix", clops.CLO_UINT)
        sc = clops.Scanner(ctx, clops.CLO_UINT, clops.CLO_ULONG)
        copy(pristine, b, keys.nbytes)
        variant, vtimes = s.tune_segmented(q, b, ob, nseg)
        ms_copy = timed(lambda: copy(pristine, b, keys.nbytes))
        ms_sort = timed(lambda: (copy(pristine, b, keys.nbytes),
                                 s.sort_segmented_device(q, b, ob, nseg))) - ms_copy
        g = clops.Graph(q)
        g.begin()
        s.sort_segmented_device(q, b, ob, nseg)
        g.end()
        ms_graph = timed(lambda: (copy(pristine, b, keys.nbytes), g.launch())) - ms_copy
        got = b.read(q, np.uint32, n)
        big = lens > 8192
        ok = True
        for i in range(0, nseg, max(1, nseg // 64)):  # sampled segment checks
            lo, hi = int(off[i]), int(off[i + 1])
            ok = ok and bool(np.array_equal(got[lo:hi], np.sort(keys[lo:hi])))
        ms_scan = timed(lambda: sc.scan_segmented_device(q, vi, vo, ob, nseg))
        gs = clops.Graph(q)
        gs.begin()
        sc.scan_segmented_device(q, vi, vo, ob, nseg)
        gs.end()
        ms_scan_graph = timed(lambda: gs.launch())
        # One plain call per segment on wrapped sub-buffers (what a caller
        # without the segmented entry points does).
        copy(pristine, b, keys.nbytes)
        q.finish()
        subs = []
        for i in range(nseg):
            lo, ln = int(off[i]), int(lens[i])
            kb = clops.call(clops.lib.ccl_buffer_new_wrap, ctx.h, b.ptr + 4 * lo, 4 * ln)
            vb = clops.call(clops.lib.ccl_buffer_new_wrap, ctx.h, vi.ptr + 4 * lo, 4 * ln)
            ob_ = clops.call(clops.lib.ccl_buffer_new_wrap, ctx.h, vo.ptr + 8 * lo, 8 * ln)
            subs.append((kb, vb, ob_, ln))
        t0 = time.perf_counter()
        for kb, _, _, ln in subs:
            clops.call(clops.lib.clo_sort_with_device_data, s.h, q.h, None, kb, None, ln, 0)
        q.finish()
        ms_plain_sort = (time.perf_counter() - t0) * 1e3
        q.gc()
        t0 = time.perf_counter()
        for _, vb, ob_, ln in subs:
            clops.call(clops.lib.clo_scan_with_device_data, sc.h, q.h, None, vb, ob_, ln, 0)
        q.finish()
        ms_plain_scan = (time.perf_counter() - t0) * 1e3
        q.gc()
        for kb, vb, ob_, _ in subs:
            for h in (kb, vb, ob_):
                clops.lib.ccl_buffer_destroy(h)
        model = 36.0 * float(lens[big].sum()) + 8.0 * float(lens[~big].sum())
        best = min(ms_sort, ms_graph)
        res["segmented_lognormal_50k"] = {
            "segments": nseg, "elements": n,
            "sort_ms": round(ms_sort, 3), "sort_graph_ms": round(ms_graph, 3),
            "sort_Gkeys/s": round(n / (best * 1e-3) / 1e9, 3),
            "sort_plain_per_segment_ms": round(ms_plain_sort, 1),
            "sort_speedup_vs_plain": round(ms_plain_sort / best, 1),
            "sort_model_bytes": "36 B/key in segments > 8192, 8 B/key in the others",
            "sort_frac_of_peak": round(model / (best * 1e-3) / 1e9 / peak, 4),
            "autotuner": {"chosen": variant, "chosen_shape": seg_shape(variant),
                          "chosen_ms": round(vtimes[variant], 3),
                          "default_ms": round(vtimes[0], 3),
                          "slowest_ms": round(max(vtimes), 3),
                          "variants_timed": len(vtimes),
                          "variant_ms": [round(t, 3) for t in vtimes]},
            "scan_ms": round(ms_scan, 3), "scan_graph_ms": round(ms_scan_graph, 3),
            "scan_GB/s": round(12.0 * n / (min(ms_scan, ms_scan_graph) * 1e-3) / 1e9, 1),
            "scan_frac_of_peak": round(12.0 * n / (min(ms_scan, ms_scan_graph) * 1e-3)
                                       / 1e9 / peak, 4),
            "scan_plain_per_segment_ms": round(ms_plain_scan, 1),
            "scan_speedup_vs_plain": round(ms_plain_scan / min(ms_scan, ms_scan_graph), 1),
            "result_check": "sampled segments sorted" if ok else "FAILED"}
        for x in (g, gs, pristine, b, ob, vi, vo, s, sc):
            x.destroy()

    def serve():
        """Open-loop serving: Poisson arrivals (seed 49), 60 % sort / 30 %
        scan / 10 % random fill, n log-uniform in [2^10, 2^26], uint / ulong
        50/50, 120 GB admission budget, --serve-seconds of arrivals (10 s by
        default). Device-resident buffers (requests read slices of a 4 GiB
        device pool and write their own slices of a 48 GiB device output
        ring):
          * at 20k requests/s (offered far above capacity: the aggregate
            is the server's capacity), against the same requests as serial
            plain device-data calls;
          * at a load the server sustains (the same request sequence with
            arrivals stretched to offer about 25 Gelem/s), so p50/p99 are
            service latency, against the same arrivals served one request
            at a time on one stream with batching off (serial plain calls
            behind the same queue).
        Host buffers (page-locked pools): at a sustainable load (about
        8 Gelem/s) for the same duration, and at 20k requests/s for 2 s
        against serial plain host-data calls. Each run reports how many
        batches were in flight on the device at once."""
        dur = args.serve_seconds
        base_rate = 20000.0
        u = splitmix64(49, 1 << 22)
        with np.errstate(divide="ignore"):
            gaps = -np.log(np.maximum((u[0::8] >> np.uint64(11)).astype(np.float64)
                                      / float(1 << 53), 1e-300)) / base_rate
        base_arrivals = np.cumsum(gaps)
        kind = (u[1::8] % np.uint64(10)).astype(np.int64)
        logn = 10.0 + 16.0 * (u[2::8] >> np.uint64(11)).astype(np.float64) / float(1 << 53)
        nreq = np.minimum(np.exp2(logn).astype(np.int64), 1 << 26)
        wide = (u[3::8] & np.uint64(1)).astype(bool)
        pos_in = u[4::8]
        pos_out = u[5::8]
        # (op, type / generator, sum type, n or states, draws, in bytes, out bytes)
        specs, elems_of = [], []
        for i in range(base_arrivals.size):
            n = int(nreq[i])
            if kind[i] < 6:
                code, eb = (clops.CLO_ULONG, 8) if wide[i] else (clops.CLO_UINT, 4)
                specs.append((clops.SERVE_SORT, code, 0, n, 0, n * eb, n * eb))
                elems_of.append(n)
            elif kind[i] < 9:
                code, eb = (clops.CLO_ULONG, 8) if wide[i] else (clops.CLO_UINT, 4)
                specs.append((clops.SERVE_SCAN, code, clops.CLO_ULONG, n, 0, n * eb, n * 8))
                elems_of.append(n)
            else:
                g, st, dr = i % 5, max(1, n // 16), 16
                specs.append((clops.SERVE_RNG_FILL, g, 0, st, dr,
                              st * clops.RNG_SEED_SIZE[clops.RNG_NAMES[g]], st * dr * 4))
                elems_of.append(st * dr)
        elems_of = np.array(elems_of, dtype=np.float64)
        mean_rate_elems = elems_of.mean() * base_rate  # offered elem/s at 20k req/s

        def window(offered_gelem, seconds):
            """Arrivals offering about offered_gelem Gelem/s (None: 20k
            requests/s) over `seconds`: (arrival times, request count)."""
            scale = 1.0 if offered_gelem is None else mean_rate_elems / (offered_gelem * 1e9)
            arr = base_arrivals * scale
            count = int(np.searchsorted(arr, seconds))
            return arr[:count], count

        block = splitmix64(149, 1 << 26).view(np.uint8)  # 512 MiB of random bytes

        def make(count, pool_in, pool_bytes, out_addr, device):
            reqs = []
            for i in range(count):
                op, code, sc, n, dr, span_in, span_out = specs[i]
                a = pool_in + int(pos_in[i] % np.uint64((pool_bytes - span_in) // 16)) * 16
                bo = out_addr(i, span_out)
                if op == clops.SERVE_RNG_FILL:
                    reqs.append(clops.Server.request(op, 0, 0, n, dr, code, inp=a, out=bo,
                                                     device=device))
                else:
                    reqs.append(clops.Server.request(op, code, sc, n, inp=a, out=bo,
                                                     device=device))
            return reqs

        def served(reqs, arrivals, streams=4, max_batch=4096):
            srv = clops.Server(ctx, 120 << 30, streams=streams)
            srv.configure(max_batch=max_batch)
            for r in reqs[:64]:  # warm-up: a few requests of each kind
                srv.submit(r)
            srv.drain()
            srv.reset_stats()
            srv.replay(reqs, list(arrivals))
            srv.drain()
            st_ = srv.stats()
            srv.destroy()
            return st_

        sorters = {clops.CLO_UINT: clops.Sorter(ctx, "satradix", clops.CLO_UINT),
                   clops.CLO_ULONG: clops.Sorter(ctx, "satradix", clops.CLO_ULONG)}
        scanners = {clops.CLO_UINT: clops.Scanner(ctx, clops.CLO_UINT, clops.CLO_ULONG),
                    clops.CLO_ULONG: clops.Scanner(ctx, clops.CLO_ULONG, clops.CLO_ULONG)}

        class Wrapped:
            def __init__(self, addr, nbytes):
                self.h = clops.call(clops.lib.ccl_buffer_new_wrap, ctx.h, clops.C.c_void_p(addr),
                                    nbytes)

            def destroy(self):
                clops.lib.ccl_buffer_destroy(self.h)

        def serial_device(reqs):
            """The requests one at a time as plain device-data calls (about
            2 s of work)."""
            done_el, t0 = 0.0, time.perf_counter()
            for r, sp in zip(reqs, specs):
                bi, bo_ = Wrapped(r.in_, max(sp[5], 1)), Wrapped(r.out, max(sp[6], 1))
                if r.op == clops.SERVE_SORT:
                    clops.wait(clops.call(clops.lib.clo_sort_with_device_data, sorters[r.type].h,
                                          q.h, None, bi.h, bo_.h, r.n, 0))
                    done_el += r.n
                elif r.op == clops.SERVE_SCAN:
                    clops.wait(clops.call(clops.lib.clo_scan_with_device_data, scanners[r.type].h,
                                          q.h, None, bi.h, bo_.h, r.n, 0))
                    done_el += r.n
                else:
                    rng = clops.Rng(ctx, q, clops.RNG_NAMES[r.rng], clops.CLO_RNG_SEED_EXT_DEV,
                                    r.n, seeds=bi)
                    clops.wait(rng.fill(q, bo_, r.draws))
                    rng.destroy()
                    done_el += r.n * r.draws
                bi.destroy()
                bo_.destroy()
                if time.perf_counter() - t0 > 2.0:
                    break
            return done_el / (time.perf_counter() - t0)

        def serial_host(reqs):
            """The requests one at a time as plain host-data calls (about 2 s
            of work)."""
            done_el, t0 = 0.0, time.perf_counter()
            for r in reqs:
                if r.op == clops.SERVE_SORT:
                    clops.call(clops.lib.clo_sort_with_host_data, sorters[r.type].h, q.h, None,
                               r.in_, r.out, r.n, 0)
                    done_el += r.n
                elif r.op == clops.SERVE_SCAN:
                    clops.call(clops.lib.clo_scan_with_host_data, scanners[r.type].h, q.h, None,
                               r.in_, r.out, r.n, 0)
                    done_el += r.n
                else:
                    name = clops.RNG_NAMES[r.rng]
                    seeds = np.ctypeslib.as_array(
                        (clops.C.c_uint8 * (r.n * clops.RNG_SEED_SIZE[name])).from_address(r.in_))
                    rng = clops.Rng(ctx, q, name, clops.CLO_RNG_SEED_EXT_HOST, r.n, seeds=seeds)
                    ob_ = clops.Buffer(ctx, r.n * r.draws * 4)
                    clops.wait(rng.fill(q, ob_, r.draws))
                    clops.call(clops.lib.ccl_buffer_enqueue_read, ob_.h, q.h, 1, 0,
                               r.n * r.draws * 4, r.out, None)
                    ob_.destroy()
                    rng.destroy()
                    done_el += r.n * r.draws
                if time.perf_counter() - t0 > 2.0:
                    break
            return done_el / (time.perf_counter() - t0)

        def report(st_, count, seconds, buffers, serial=None):
            agg = st_["elements"] / st_["span_s"] if st_["span_s"] else 0.0
            offered = float(elems_of[:count].sum())
            out = {
                "buffers": buffers, "open_loop_s": seconds,
                "offered_req_per_s": round(count / seconds, 1), "requests": count,
                "offered_Gelem_per_s": round(offered / seconds / 1e9, 2),
                "submitted": st_["submitted"], "admitted": st_["admitted"],
                "completed": st_["completed"], "rejected": st_["rejected"],
                "batches": st_["batches"], "max_queued": st_["max_queued"],
                "peak_budget_GB": round(st_["peak_bytes"] / 1e9, 2),
                "budget_GB": round(120 * 1.073741824, 2),
                "p50_ms": round(st_["p50_ms"], 2), "p99_ms": round(st_["p99_ms"], 2),
                "mean_ms": round(st_["mean_ms"], 2), "span_s": round(st_["span_s"], 3),
                "aggregate_Gelem_per_s": round(agg / 1e9, 3),
                "batches_in_flight_max": int(st_["max_concurrent_batches"]),
                "batches_in_flight_mean": round(st_["mean_concurrent_batches"], 2),
                "device_busy_s": round(st_["device_busy_s"], 3)}
            if serial is not None:
                out["serial_plain_Gelem_per_s"] = round(serial / 1e9, 3)
                out["speedup_vs_serial_plain"] = round(agg / serial, 2) if serial else None
            return out

        # Device-resident buffers.
        dpool = 4 << 30
        din = clops.Buffer(ctx, dpool)
        for o in range(0, dpool, block.size):
            clops.call(clops.lib.ccl_buffer_enqueue_write, din.h, q.h, 1, o, block.size,
                       clops.np_ptr(block), None)
        ring = 48 << 30
        dout = clops.Buffer(ctx, ring)
        cursor = [0]

        def ring_slot(i, span):
            span = (span + 255) // 256 * 256
            if cursor[0] + span > ring:
                cursor[0] = 0
            at = dout.ptr + cursor[0]
            cursor[0] += span
            return at
        arr, count = window(None, dur)
        dreqs = make(count, din.ptr, dpool, ring_slot, True)
        dev_res = report(served(dreqs, arr), count, dur, "device-resident",
                         serial_device(dreqs))
        arr, count = window(25.0, dur)
        dreqs = dreqs[:count] if count <= len(dreqs) else \
            make(count, din.ptr, dpool, ring_slot, True)
        sus = report(served(dreqs, arr), count, dur, "device-resident")
        one = report(served(dreqs, arr, streams=1, max_batch=1), count, dur,
                     "device-resident, one stream, batching off")
        sus["serial_plain_same_arrivals"] = {
            k: one[k] for k in ("p50_ms", "p99_ms", "mean_ms", "aggregate_Gelem_per_s",
                                "max_queued", "span_s", "batches_in_flight_max")}
        sus["p50_speedup_vs_serial_plain"] = round(one["p50_ms"] / sus["p50_ms"], 2) \
            if sus["p50_ms"] else None
        sus["p99_speedup_vs_serial_plain"] = round(one["p99_ms"] / sus["p99_ms"], 2) \
            if sus["p99_ms"] else None
        din.destroy()
        dout.destroy()

        # Host buffers (page-locked pools; outputs at random slices).
        pool_bytes = 4 << 30
        hin = clops.lib.clo_host_alloc(pool_bytes, None)
        hout = clops.lib.clo_host_alloc(pool_bytes, None)
        pin = np.ctypeslib.as_array((clops.C.c_uint8 * pool_bytes).from_address(hin))
        for o in range(0, pool_bytes, block.size):
            pin[o:o + block.size] = block

        def host_out(i, span):
            return hout + int(pos_out[i] % np.uint64((pool_bytes - span) // 16)) * 16
        arr, count = window(8.0, dur)
        hreqs = make(count, hin, pool_bytes, host_out, False)
        host_sus = report(served(hreqs, arr), count, dur, "host (page-locked)")
        hsec = min(dur, 2.0)
        arr, count = window(None, hsec)
        hreqs = make(count, hin, pool_bytes, host_out, False)
        host_res = report(served(hreqs, arr), count, hsec, "host (page-locked)",
                          serial_host(hreqs))
        for x in list(sorters.values()) + list(scanners.values()):
            x.destroy()
        del pin
        clops.lib.clo_host_free(hin)
        clops.lib.clo_host_free(hout)
        res["serve_poisson_20k"] = dev_res
        res["serve_sustained_25Gelem"] = sus
        res["serve_poisson_20k_host_buffers"] = host_res
        res["serve_sustained_8Gelem_host_buffers"] = host_sus

    def c1_c3():
        """C1: 2^20 uint32 keys with the reference's radix=16 option
        (latency-bound, informational). C3: 2^28 uint32 keys sorted,
        reverse-sorted, all equal, 16 distinct values, Zipf(1.1) over 2^20
        ranks, and 2^27 uint64 keys with only the low 20 bits random; each
        with the passes the digit histograms leave (constant digits are
        skipped)."""
        from inputs import adversarial_u32, low20_u64
        s32 = clops.Sorter(ctx, "satradix", clops.CLO_UINT, options="radix=16")
        a = keys_u32_chunked(42, 1 << 20)
        pr = clops.Buffer.from_array(ctx, q, a)
        b = clops.Buffer(ctx, a.nbytes)
        t_copy = timed(lambda: copy(pr, b, a.nbytes), reps=20)
        ms = timed(lambda: (copy(pr, b, a.nbytes), s32.sort_device(q, b, a.size)),
                   reps=20) - t_copy
        res["c1_satradix_2pow20_u32_radix16"] = {"Gkeys/s": round(a.size / (ms * 1e-3) / 1e9, 3),
                                                  "ms": round(ms, 4)}
        for x in (pr, b):
            x.destroy()
        n = 1 << 28 if only is None else 1 << min(args.log2n, 28)
        out = {}
        # Sorted and reverse-sorted inputs come from sorting uniform keys on
        # the device (a host sort of 2^28 keys would dominate the run).
        base = keys_u32_chunked(47, n)
        bb = clops.Buffer.from_array(ctx, q, base)
        clops.wait(s32.sort_device(q, bb, n))
        srt = bb.read(q, np.uint32, n)
        bb.destroy()
        cases = [("sorted", lambda: srt), ("reverse", lambda: srt[::-1].copy())]
        cases += [(k, lambda k=k: adversarial_u32(k, n)) for k in ("equal", "distinct16", "zipf")]
        cases.append(("u64_low20", lambda: low20_u64(n // 2)))
        for name, gen in cases:
            a = gen()
            s = s32 if a.dtype == np.uint32 else clops.Sorter(ctx, "satradix", clops.CLO_ULONG)
            pr = clops.Buffer.from_array(ctx, q, a)
            b = clops.Buffer(ctx, a.nbytes)
            t_copy = timed(lambda: copy(pr, b, a.nbytes))
            before = clops.launch_count()
            ms = timed(lambda: (copy(pr, b, a.nbytes), s.sort_device(q, b, a.size))) - t_copy
            launches = (clops.launch_count() - before) / 5.0  # 2 warm-up + 3 timed
            got = b.read(q, a.dtype, a.size)
            ok = bool(np.all(got[1:] >= got[:-1]))
            out[name] = {"n": int(a.size), "Gkeys/s": round(a.size / (ms * 1e-3) / 1e9, 3),
                         "ms": round(ms, 3), "kernels_per_sort": launches,
                         "sorted": ok}
            for x in (pr, b):
                x.destroy()
            if s is not s32:
                s.destroy()
        res["c3_satradix_adversarial"] = out
        s32.destroy()

    parts = {"abitonic": abitonic, "kv": kv, "scan": scan, "rng": rngs,
             "segmented": segmented, "serve": serve, "c1c3": c1_c3}
    for name, fn in parts.items():
        if only is None or only == name:
            fn()
    q.gc()
    return res


def bench_config(n, world, ok):
    """The headline workload's config, the same in both arms."""
    return {"workload": WORKLOAD, "n": n, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2: a distinct 1 GiB copy per step",
            "result_check": "sorted+multiset ok" if ok else "FAILED"}


def seg_shape(v):
    """The segmented sort's shape for variant v (include/clo_gb300.h)."""
    d, v = v % 2, v // 2
    l_, v = v % 3, v // 3
    b, a = v % 3, v // 3
    return {"class_a": ["128x8", "256x8"][a], "class_b": ["512x16", "256x16", "1024x16"][b],
            "long_keys_per_thread": [56, 48, 40][l_], "cta_digit_bits": [8, 4][d]}


def cpu_port_sorts(keys, steps, warmup, cores):
    """The reference's algorithm (LSD radix sort, 4-bit digits as its default
    radix 16) restated in C, on all host threads: `steps` timed sorts of a
    fresh copy of `keys` (the copy is made outside the timed part). Returns
    (total seconds, last output ok)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    work = np.empty_like(keys)
    for _ in range(warmup):
        work[:] = keys
        oracle.radix_sort_u32_threaded(work, cores, 4)
    total = 0.0
    for _ in range(steps):
        work[:] = keys
        t0 = time.perf_counter()
        oracle.radix_sort_u32_threaded(work, cores, 4)
        total += time.perf_counter() - t0
    ok = bool(np.all(work[1:] >= work[:-1])) and \
        int(work.sum(dtype=np.uint64)) == int(keys.sum(dtype=np.uint64))
    return total, ok


def reference_kernels_c1():
    """The reference's own satradix kernels (its OpenCL C, compiled for the
    host by oracle/build_ref.py) on 2^20 uint32 keys from seed 42 with radix
    16, one timed sort. Work-groups run in parallel on all host threads;
    each work-group's work-items are fibers switched at every barrier, so
    the time includes that emulation's overhead. Checked against the
    committed digest of the same run. None where the library is absent."""
    sys.path.insert(0, str(ROOT / "oracle"))
    try:
        import ref
        if not ref.available():
            return None
    except Exception:
        return None
    import hashlib
    n = 1 << 20
    keys = keys_u32_chunked(42, n)
    t0 = time.perf_counter()
    out = ref.sort(keys, 5, "satradix", 256)
    dt = time.perf_counter() - t0
    want = None
    kats = json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())["kats"]
    for k in kats:
        if k["op"] == "sort" and k["algo"] == "satradix" and k["n"] == n and k["seed"] == 42:
            want = k["sha256"]
    got = hashlib.sha256(out.tobytes()).hexdigest()
    return {"value": round(n / dt / 1e9, 6), "unit": "Gkeys/s", "seconds": round(dt, 2),
            "cores": int(os.environ.get("CLC_THREADS", os.cpu_count() or 1)),
            "kind": "reference",
            "sample": "2^20 uint32 keys, seed 42, radix 16, lws 256: the reference's own "
                      "satradix kernels through a host OpenCL-C emulation (work-groups on "
                      "threads, work-items as fibers switched at barriers)",
            "result_check": "reference digest ok" if got == want else "FAILED"}


def cpu_baseline(args):
    """The reference's algorithm on the host cores, on the full headline
    workload (3 timed sorts of 2^28 keys), plus the reference's own kernels
    at 2^20 keys."""
    n = 1 << args.log2n
    cores = os.cpu_count() or 1
    reps = 3
    total, ok = cpu_port_sorts(keys_u32_chunked(42, n), reps, 1, cores)
    out = {"value": round(n * reps / total / 1e9, 4), "unit": "Gkeys/s", "cores": cores,
           "kind": "port",
           "sample": f"the full workload: {reps} sorts of all 2^{args.log2n} uint32 keys, "
                     "LSD radix 16, all host threads",
           "result_check": "sorted+multiset ok" if ok else "FAILED"}
    rk = reference_kernels_c1() if args.ref_kernels else None
    if rk is not None:
        out["reference_kernels"] = rk
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n = 1 << args.log2n
    cores = os.cpu_count() or 1
    total, ok = cpu_port_sorts(keys_u32_chunked(42, n), args.steps, args.warmup, cores)
    val = n * args.steps / total / 1e9
    out = {
        "impl": "reference",
        "metric": METRIC, "value": round(val, 4), "unit": "Gkeys/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (splitmix64 seed 42, uniform over [0, 2^32))",
        "config": bench_config(n, world, ok),
        "cpu_baseline": {"value": round(val, 4), "unit": "Gkeys/s", "cores": cores, "kind": "port",
                         "sample": f"each step sorts all 2^{args.log2n} keys with the reference's "
                                   "LSD radix-16 scheme (restated in C) on all host threads"},
        "e2e": {"value": round(val, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--log2n", type=int, default=28)
    ap.add_argument("--no-suite", dest="suite", action="store_false")
    ap.add_argument("--no-ref-kernels", dest="ref_kernels", action="store_false",
                    help="skip timing the reference's own kernels at 2^20 keys")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="open-loop duration of the serving workload")
    ap.add_argument("--only", choices=["abitonic", "kv", "scan", "rng", "segmented", "serve",
                                       "c1c3"],
                    help="run one suite primitive alone (profiling cases)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.only:
        import clops
        ctx = clops.Context(dist_env()[2])
        q = clops.Queue(ctx, profiling=True)
        print(json.dumps(run_suite(clops, ctx, q, args, only=args.only)), flush=True)
        q.destroy()
        ctx.destroy()
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
