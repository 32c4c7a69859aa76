"""The N > 1 path of bench.py on CPU: ranks are independent replicas, and
the only collectives are the timing barrier and the max over ranks.
world_size 2 over gloo on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), GB_BENCH_BACKEND="gloo")
    sys.path.insert(0, REPO)
    import torch.distributed as dist

    import bench
    r, w, _ = bench.dist_setup()
    bench.barrier(w)
    q.put((r, w, bench.max_over_ranks(1.5 * (r + 1), w)))
    bench.barrier(w)
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=180) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 3.0), (1, 2, 3.0)]


def test_reference_arm_two_ranks_gloo():
    """torchrun with 2 ranks: rank 0 alone runs the bounded CPU sample and
    prints one JSON line; the other rank exits 0 without work."""
    env = dict(os.environ, GB_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _free_port(), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--log-n", "12"]
    out = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
