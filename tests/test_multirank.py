"""Host plumbing of multi-GPU runs (tfm_gb300/replicas.py), on CPU ranks over
gloo, world size 2: each rank gets its own disjoint replica seeds, the
timing reduction returns the slowest rank's time on every rank, and the
whole-job rate counts every rank's units against that time. The replicas
never exchange data, so these are the only collectives on the path."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from tfm_gb300 import replicas

    w, r, local = replicas.init("gloo")
    assert (w, r, local) == (ws, rank, rank)
    seeds = torch.tensor(replicas.replica_seeds(512, rank).astype(np.int64))
    gathered = [torch.zeros_like(seeds) for _ in range(ws)]
    dist.all_gather(gathered, seeds)
    replicas.barrier(ws)
    t = replicas.max_over_ranks(1.5 + rank, ws)  # rank 1 is the slow one
    rate = replicas.whole_job_rate(1000, ws, t)
    out.put((rank, [g.tolist() for g in gathered], t, rate))
    replicas.finalize(ws)


def test_two_gloo_ranks():
    ws = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, t, rate in res:
        a, b = set(gathered[0]), set(gathered[1])
        assert len(a) == len(b) == 512 and not (a & b)  # disjoint ensembles
        assert t == 2.5  # max over ranks, on every rank
        assert rate == pytest.approx(2 * 1000 / 2.5)


def test_single_rank_needs_no_group():
    from tfm_gb300 import replicas

    assert replicas.max_over_ranks(3.0, 1) == 3.0
    replicas.barrier(1)
    with pytest.raises(ValueError):
        replicas.replica_seeds(200000, 0)
