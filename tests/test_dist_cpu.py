"""Host-side multi-rank logic of bench.py on CPU: world size 2 over the gloo backend.

bench.py runs one replica per GPU (torchrun, one process each); every rank times the
same work and the job reports the slowest rank's time with the bytes of all ranks.
Here two CPU processes check that reduction and the aggregate formula; the GPU path
calls the same helpers over NCCL."""
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


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank)
        env = bench.dist_env()
        value = bench.aggregate_gbs(env[0], 2e9, slowest)
        q.put((rank, slowest, env, value))
    finally:
        dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_with_all_ranks_bytes():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, slowest, env, value in out:
        assert slowest == 15.0                # the max over both ranks
        assert env == (2, rank, rank)         # WORLD_SIZE, RANK, LOCAL_RANK
        assert value == pytest.approx(2 * 2e9 / 15e-3 / 1e9)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.aggregate_gbs(1, 1e9, 1000.0) == pytest.approx(1.0)
