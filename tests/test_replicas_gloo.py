"""The multi-GPU path is replicas only (no collective on the data path):
units spread over the ranks, a barrier and the maximum of the step time over
the ranks.  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from at3d_gb300 import replicas
    import torch.distributed as dist
    r, n = replicas.init("gloo")
    replicas.barrier()
    m = replicas.max_over_ranks(10.0 * (r + 1))
    mine = replicas.shard(11, r, n)
    out.put((r, n, m, mine))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2, 2]
    assert [r[2] for r in res] == [20.0, 20.0]          # max of the two ranks' values
    units = sorted(u for r in res for u in r[3])
    assert units == list(range(11))                     # every unit on exactly one rank
    assert abs(len(res[0][3]) - len(res[1][3])) <= 1


def test_single_rank_is_identity(monkeypatch):
    from at3d_gb300 import replicas
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.init() == (0, 1)
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.shard(5, 0, 1) == [0, 1, 2, 3, 4]
