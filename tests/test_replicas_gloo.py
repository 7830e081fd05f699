"""Replica aggregation across ranks with the gloo backend (world size 2, CPU)."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from tinyfluids_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = 10.0 + 5.0 * rank  # rank 1 is slower
        value, ms = replicas.job_throughput(1000, 4, ms_local, world)
        q.put((rank, value, ms))
    finally:
        dist.destroy_process_group()


def test_job_throughput_uses_slowest_rank_and_all_ranks_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, value, ms in res:
        assert ms == 15.0
        assert abs(value - 2 * 1000 * 4 / 15e-3 / 1e9) < 1e-12


def test_single_process_is_identity():
    from tinyfluids_gb300 import replicas
    v, ms = replicas.job_throughput(10, 2, 4.0, 1)
    assert ms == 4.0 and abs(v - 10 * 2 / 4e-3 / 1e9) < 1e-15
