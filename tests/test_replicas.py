"""The N-GPU form of the benchmark runs N independent replicas (one process
per GPU, no collective on the data path); the job's time is its slowest
rank's.  This checks that aggregation with two gloo ranks on the CPU."""
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


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    value, ms = bench.replica_throughput(10.0 * (rank + 1), 100.0, device="cpu")
    out.put((rank, value, ms))
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, value, ms in res:
        assert ms == 20.0                       # the slower rank
        assert value == pytest.approx(2 * 100 / 0.020)
