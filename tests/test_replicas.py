"""The multi-GPU path of bench.py is replicas only: N independent simulations, one per rank,
no data-path collective; the job's time is the slowest replica's and the job's rate is
N x steps over it. The host logic runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        env = bench.dist_env()
        slowest = bench.max_over_ranks(1.0 + rank, ws, device="cpu")
        rate = bench.replica_rate(ws, 10, slowest)

        class A:  # the reference arm on a rank other than 0 does no work
            steps, warmup = 2, 1
        ref = bench.reference_arm(A, ws, rank) if rank != 0 else "rank0"
        q.put((rank, env, slowest, rate, ref))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_sum_the_work():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, env, slowest, rate, ref in out:
        assert env == (ws, rank, rank)
        assert slowest == 2.0                       # rank 1's 2 s
        assert rate == pytest.approx(2 * 10 / 2.0)  # both replicas' steps over the slowest
    assert out[1][4] is None                        # rank 1 prints no reference line
