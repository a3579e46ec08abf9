"""The multi-rank path of bench.py on CPU (gloo, world size 2): the path
shards as independent replicas, so the job's throughput is the sum of the
ranks' bytes over the slowest rank's time, with no data-path collective."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    import torch.distributed as td

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    td.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    # rank r took (r+1) * 10 ms for 1 GB of algorithmic traffic
    ms, gbs = bench.job_throughput(10.0 * (rank + 1), 10 ** 9, ws, device="cpu")
    q.put((rank, ms, gbs, bench.dist()))
    td.barrier()
    td.destroy_process_group()


def test_replicas_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, gbs, d in out:
        assert ms == pytest.approx(20.0)  # slowest rank
        assert gbs == pytest.approx(2e9 / 20e-3 / 1e9)  # both ranks' bytes over that time
        assert d == (2, rank, rank)


def test_single_rank_is_local():
    import bench

    ms, gbs = bench.job_throughput(4.0, 8 * 10 ** 9, 1)
    assert ms == 4.0 and gbs == pytest.approx(2000.0)
