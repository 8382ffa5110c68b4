"""The multi-process path of bench.py on the CPU: two ranks over gloo.

bench.py runs N independent replicas (one process per GPU, no data-path
collective); what the ranks share is the barrier around the timed region, the
maximum of the per-rank times and the rule that rank 0 alone runs the CPU
reference arm (here on a small tank) while the other ranks return at once.
Those host-side pieces are exercised here with world size 2."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class _Args:
    impl = "reference"
    n = 300      # a small tank, so that the oracle runs in about a second
    steps = 2
    warmup = 1
    gpus = 2


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w, _ = bench.dist_init(_Args)
    bench.barrier(w)
    t_max = bench.allmax(w, 0.5 * (r + 1))
    # only rank 0 runs (and prints) the reference arm; the others return at once
    line = bench.run_reference(_Args, r, w)
    bench.barrier(w)
    ran = None if line is None else (line["impl"], line["steps"], line["value"] > 0,
                                     line["measured"]["gmres_iterations"] > 0)
    q.put((r, w, dist.get_backend(), t_max, ran))
    dist.destroy_process_group()


def test_two_ranks_share_barrier_and_max_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in procs)
    assert got == [(0, 2, "gloo", 1.0, ("reference", 2, True, True)), (1, 2, "gloo", 1.0, None)]
