"""The replica path of bench.py on CPU (gloo, two ranks): the host-side
barrier and max-reduction every rank's timing goes through, and the
reference arm launched under torchrun, where rank 0 alone measures and
prints and the other rank exits without work."""
import json
import multiprocessing as mp
import os
import pathlib
import socket
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    r, w, lr = bench.dist_env()
    d = bench.Dist(r, w)
    d.barrier()
    m = d.max(1.5 + r)     # each rank's "time"; every rank gets the max
    d.barrier()
    d.close()
    q.put((r, w, lr, m))


def test_dist_barrier_and_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(i, 2, port, q)) for i in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(180)
    assert [p.exitcode for p in ps] == [0, 0]
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_single_rank_dist_is_a_no_op():
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(0, 1)
    d.barrier()
    assert d.max(3.25) == 3.25
    d.close()


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--log2n", "20"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-3000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")
