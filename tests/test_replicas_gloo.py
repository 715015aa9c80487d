"""Multi-GPU is replicas only (independent poses, no data-path collective):
the host-side aggregation of bench.py runs on gloo with two CPU ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_local = 0.10 if rank == 0 else 0.25  # the slower rank sets the job time
    t, v = bench.replica_throughput(t_local, 1000, world, "cpu")
    q.put((rank, t, v))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, t, v in res:
        assert t == pytest.approx(0.25)
        assert v == pytest.approx(2 * 1000 / 0.25)


def test_single_rank_is_identity():
    import bench
    assert bench.replica_throughput(0.5, 100, 1) == (0.5, 200.0)
