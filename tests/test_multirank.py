"""Host plumbing of multi-GPU runs (tfm_gb300/replicas.py), on CPU ranks over
gloo, world size 2: each rank gets its own disjoint replica seeds, the
timing reduction returns the slowest rank's time on every rank, the
whole-job rate counts every rank's units against that time, and a fixed
ensemble split by bead count puts every replica on exactly one rank. The replicas
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


def _ensemble_sizes(n=512, seed=2026):
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(np.log(1024), np.log(16384), n))).astype(np.int32)


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
    # a fixed ensemble split by bead count: each rank derives its share alone
    sizes = _ensemble_sizes()
    idx, sz, sd = replicas.local_replicas(sizes, np.arange(len(sizes)) + 1, ws, rank)
    share = torch.tensor([len(idx), int(sz.sum())], dtype=torch.int64)
    shares = [torch.zeros_like(share) for _ in range(ws)]
    dist.all_gather(shares, share)
    mine = torch.zeros(len(sizes), dtype=torch.int64)
    mine[torch.tensor(idx)] = 1
    dist.all_reduce(mine)  # replicas held by each index, summed over ranks
    out.put((rank, [g.tolist() for g in gathered], t, rate, [x.tolist() for x in shares],
             mine.tolist(), bool((sd == idx + 1).all())))
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
    total = int(_ensemble_sizes().sum())
    for rank, gathered, t, rate, shares, held, seeds_kept in res:
        a, b = set(gathered[0]), set(gathered[1])
        assert len(a) == len(b) == 512 and not (a & b)  # disjoint ensembles
        assert t == 2.5  # max over ranks, on every rank
        assert rate == pytest.approx(2 * 1000 / 2.5)
        assert held == [1] * 512  # every replica on exactly one rank
        assert sum(n for n, _ in shares) == 512 and sum(b for _, b in shares) == total
        assert max(b for _, b in shares) <= total / ws + 16384  # within one replica of even
        assert seeds_kept  # replicas keep their global seeds


def test_single_rank_needs_no_group():
    from tfm_gb300 import replicas

    assert replicas.max_over_ranks(3.0, 1) == 3.0
    replicas.barrier(1)
    with pytest.raises(ValueError):
        replicas.replica_seeds(200000, 0)


def test_split_replicas_balance_and_cover():
    from tfm_gb300 import replicas

    sizes = _ensemble_sizes()
    for ws in (1, 2, 3, 4, 8):
        parts = replicas.split_replicas(sizes, ws)
        assert len(parts) == ws
        assert sorted(np.concatenate(parts).tolist()) == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) for p in parts]
        # longest-processing-time-first: no rank exceeds the mean by more than
        # one replica, nor 4/3 of the optimum (itself at least the mean)
        assert max(loads) <= sizes.sum() / ws + sizes.max()
        assert max(loads) <= 4 / 3 * max(sizes.sum() / ws, sizes.max())
        again = replicas.split_replicas(sizes.tolist(), ws)
        assert all(np.array_equal(p, q) for p, q in zip(parts, again))  # deterministic
    # more ranks than replicas: the extra ranks get nothing
    parts = replicas.split_replicas([5, 3], 4)
    assert [p.tolist() for p in parts] == [[0], [1], [], []]
    # the largest replica alone bounds the load
    parts = replicas.split_replicas([100, 1, 1, 1], 2)
    assert [p.tolist() for p in parts] == [[0], [1, 2, 3]]
    for bad in ([0, 3], [[1, 2]]):
        with pytest.raises(ValueError):
            replicas.split_replicas(bad, 2)
    with pytest.raises(ValueError):
        replicas.split_replicas([1, 2], 0)


def test_local_replicas_checks_its_arguments():
    from tfm_gb300 import replicas

    with pytest.raises(ValueError, match="one seed per replica"):
        replicas.local_replicas([10, 20, 30], [1, 2], 2, 0)
    with pytest.raises(ValueError, match="outside a world"):
        replicas.local_replicas([10, 20], [1, 2], 2, 2)
    idx, sz, sd = replicas.local_replicas([10, 20, 30], [7, 8, 9], 2, 1)
    assert idx.tolist() == [0, 1] and sz.tolist() == [10, 20] and sd.tolist() == [7, 8]
