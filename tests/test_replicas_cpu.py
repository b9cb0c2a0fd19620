"""Replica bookkeeping across ranks (sad_gb300/replicas.py) with two gloo processes on the
CPU: the shares of a work list partition it, the barrier holds, and the maximum over ranks
reaches every rank, which is all the multi-GPU benchmark does between its replicas."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    from sad_gb300 import replicas
    env = replicas.rank_env()
    replicas.init(env, "gloo")
    try:
        mine = replicas.shard(list(range(11)), env)
        replicas.barrier(env)
        m = replicas.max_over_ranks(env, 10.0 * (rank + 1))
        out.put((rank, mine, m))
    finally:
        replicas.finish(env)


@pytest.mark.timeout(120)
def test_two_rank_replicas_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    shares = [r[1] for r in res]
    assert sorted(shares[0] + shares[1]) == list(range(11))
    assert abs(len(shares[0]) - len(shares[1])) <= 1
    assert [r[2] for r in res] == [20.0, 20.0]


def test_single_rank_defaults(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from sad_gb300 import replicas
    env = replicas.rank_env()
    assert (env.world_size, env.rank, env.local_rank) == (1, 0, 0)
    replicas.init(env)  # no process group for one rank
    assert replicas.max_over_ranks(env, 3.5) == 3.5
    assert replicas.shard([1, 2, 3], env) == [1, 2, 3]
