"""The multi-GPU form of the bench is replicas only: every rank solves its own
copy and the job's time is the slowest rank's. This checks the cross-rank
reduction and the reference arm's rank rule with two gloo ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path
from types import SimpleNamespace

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    args = SimpleNamespace(impl="reference", gpus=ws)
    if rank == 0:
        bench.dist_init(args)  # the reference arm runs on gloo
        out = None
    else:
        out = bench.run_reference(args)  # ranks other than 0 do no work
    t, n = bench.reduce_replicas(1.5 + rank, 10.0 * (rank + 1), "cpu")
    q.put((rank, t, n, out, dist.get_backend()))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, n, out, backend in res:
        assert backend == "gloo"
        assert t == pytest.approx(2.5)   # the slowest rank's time
        assert n == pytest.approx(30.0)  # launches summed over ranks
    assert res[1][3] == 0


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.reduce_replicas(3.0, 7.0, "cpu") == (3.0, 7.0)
