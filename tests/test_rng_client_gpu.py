"""The CloRng client model: a caller's own kernel, built from the text
clo_rng_get_source() returns plus the caller's source, draws from the
RNG's device states through the device API (clo_rng_next_int, _int2,
_int4, _int8). Modelled on the reference's only RNG test
(src/tests/test_rng.c:32-38, 79-115: DEV_GID seeds, 10000 states, main
seed 1234, hash "(x * 3 + 1)", a kernel writing clo_rng_next_int(seeds,
UINT_MAX) per work-item), for every generator, with the outputs and the
final states compared to the oracle.

The vector forms draw lane k from state k * global_size + gid, so a launch
over count / w work-items draws each of the count states once: its output
is the oracle's one-draw fill in the same state order."""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

COUNT, MAIN_SEED, HASH = 10000, 1234, "(x * 3 + 1)"
GENERATORS = ["lcg", "xorshift64", "xorshift128", "mwc64x", "parkmiller", "tauslcg"]

CLIENT = r'''
extern "C" __global__ void clo_rng_test(clo_statetype *seeds, unsigned long long *output) {
	uint32_t gid = clo_rng_gid();
	uint32_t x = clo_rng_next_int(seeds, 0xFFFFFFFFu);
	output[gid] = (unsigned long long)x;
}
extern "C" __global__ void draw2(clo_statetype *s, uint32_t *out, uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	uint2 v = clo_rng_next_int2(s, n);
	out[g] = v.x; out[w + g] = v.y;
}
extern "C" __global__ void draw4(clo_statetype *s, uint32_t *out, uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	uint4 v = clo_rng_next_int4(s, n);
	out[g] = v.x; out[w + g] = v.y; out[2 * w + g] = v.z; out[3 * w + g] = v.w;
}
extern "C" __global__ void draw8(clo_statetype *s, uint32_t *out, uint32_t n) {
	uint32_t g = clo_rng_gid(), w = clo_rng_global_size();
	clo_uint8 v = clo_rng_next_int8(s, n);
	out[g] = v.s0; out[w + g] = v.s1; out[2 * w + g] = v.s2; out[3 * w + g] = v.s3;
	out[4 * w + g] = v.s4; out[5 * w + g] = v.s5; out[6 * w + g] = v.s6; out[7 * w + g] = v.s7;
}
'''


@pytest.mark.parametrize("name", GENERATORS)
def test_client_kernel_draws_match_oracle(clops, ctx, queue, name):
    rng = clops.Rng(ctx, queue, name, clops.CLO_RNG_SEED_DEV_GID, COUNT, MAIN_SEED, HASH)
    prg = clops.Program(ctx, rng.source() + CLIENT)
    try:
        st = oracle.rng_init_gid(name, COUNT, MAIN_SEED, 0)
        assert np.array_equal(rng.states(queue), st)
        # The reference test: next_int(UINT_MAX) into 64-bit outputs, with
        # the work sizes ccl_kernel_suggest_worksizes picks for 10000 items.
        k = prg.kernel("clo_rng_test")
        _, lws = clops.Program.suggest(k, COUNT)
        assert COUNT % lws == 0
        out = clops.Buffer(ctx, COUNT * 8)
        clops.wait(clops.Program.enqueue(k, queue, COUNT, lws, rng.seeds_buffer, out))
        ref, st = oracle.rng_fill(name, st, COUNT, 1, 32, 0xFFFFFFFF)
        np.testing.assert_array_equal(out.read(queue, np.uint64, COUNT), ref.astype(np.uint64))
        np.testing.assert_array_equal(rng.states(queue), st)
        out.destroy()
        # The vector forms, each continuing the streams.
        out = clops.Buffer(ctx, COUNT * 4)
        for w, kname, n in ((2, "draw2", 1000), (4, "draw4", 77777), (8, "draw8", 3)):
            k = prg.kernel(kname)
            gws = COUNT // w
            _, lws = clops.Program.suggest(k, gws)
            clops.wait(clops.Program.enqueue(k, queue, gws, lws, rng.seeds_buffer, out,
                                             (C.c_uint32, n)))
            ref, st = oracle.rng_fill(name, st, COUNT, 1, 32, n)
            np.testing.assert_array_equal(out.read(queue, np.uint32, COUNT), ref, kname)
            np.testing.assert_array_equal(rng.states(queue), st)
        out.destroy()
    finally:
        prg.destroy()
        rng.destroy()


def test_client_program_errors(clops, ctx, queue):
    # A compile error carries NVRTC's log; a missing kernel, a global size
    # that is not a multiple of the local one and a bad dimension count
    # are argument errors.
    with pytest.raises(clops.CloError) as ei:
        clops.Program(ctx, "extern \"C\" __global__ void k() { undeclared(); }")
    assert ei.value.code == clops.CLO_ERROR_LIBRARY and "undeclared" in str(ei.value)
    prg = clops.Program(ctx, "extern \"C\" __global__ void k(unsigned *o) "
                             "{ o[blockIdx.x * blockDim.x + threadIdx.x] = 7u; }")
    try:
        with pytest.raises(clops.CloError):
            prg.kernel("missing")
        # A reported error does not resurface in the next call.
        sc = clops.Scanner(ctx, 0, 1)
        a = np.arange(100, dtype=np.int8)
        bi, bo = clops.Buffer.from_array(ctx, queue, a), clops.Buffer(ctx, 100)
        clops.wait(sc.scan_device(queue, bi, bo, 100))
        np.testing.assert_array_equal(bo.read(queue, np.uint8, 100), oracle.scan(a, 0, np.uint8))
        for x in (bi, bo, sc):
            x.destroy()
        k = prg.kernel("k")
        out = clops.Buffer(ctx, 4 * 1000)
        with pytest.raises(clops.CloError) as ei:
            clops.Program.enqueue(k, queue, 1000, 64, out)
        assert ei.value.code == clops.CLO_ERROR_ARGS
        gws, lws = clops.Program.suggest(k, 1000, want_gws=True)
        assert (gws, lws) == (1024, 256)
        _, lws = clops.Program.suggest(k, 1000)
        assert lws == 250
        clops.wait(clops.Program.enqueue(k, queue, 1000, lws, out))
        assert np.all(out.read(queue, np.uint32, 1000) == 7)
        out.destroy()
    finally:
        prg.destroy()
