"""Replicas on several ranks (CPU, gloo, world size 2): the bench's
max-over-ranks time and whole-job rate, exercised without a GPU."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 10.0 + 5.0 * rank          # rank 1 is the slow replica
    m = bench.max_over_ranks(ms, device="cpu")
    out.put((rank, m, bench.whole_job_rate(1_000_000, ws, m)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_rate_gloo():
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
    assert [m for _, m, _ in res] == [15.0, 15.0]
    assert all(abs(rate - 2_000_000 / 0.015) < 1e-3 for _, _, rate in res)
