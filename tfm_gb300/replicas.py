"""Several GPUs of one node: one process per GPU, each advancing its own batch
of replicas. The replicas are independent simulations, so no data crosses
ranks; the only collectives are a barrier around a timed region and the
maximum of the ranks' timings (the whole job is as slow as its slowest rank).

Each rank draws its replicas' seeds from its own disjoint range, so an N-rank
job simulates N distinct ensembles (weak scaling: the work per GPU is fixed).
A fixed ensemble is instead split over the ranks by bead count
(split_replicas / local_replicas: strong scaling), each replica keeping its
seed.
"""
import os

import numpy as np

SEED_STRIDE = 100000  # seeds of rank r: r * SEED_STRIDE + 1 ... r * SEED_STRIDE + n


def world():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None):
    """Joins the process group when the job has more than one rank: NCCL on
    GPUs (one device per local rank), gloo otherwise. Returns world()."""
    ws, rank, local = world()
    if ws > 1:
        import torch
        import torch.distributed as dist

        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return ws, rank, local


def finalize(ws):
    if ws > 1:
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()


def replica_seeds(n_replicas, rank):
    """Seeds of one rank's replicas; disjoint between ranks."""
    if not 0 < n_replicas < SEED_STRIDE:
        raise ValueError("replicas per rank must be in [1, %d)" % SEED_STRIDE)
    return np.arange(n_replicas, dtype=np.uint64) + 1 + SEED_STRIDE * rank


def split_replicas(sizes, ws):
    """Partition of a fixed ensemble over ws ranks, balanced by bead count:
    replicas in decreasing size (ties by index) each go to the rank with the
    fewest beads so far (ties to the lowest rank), the longest-processing-
    time-first rule, whose largest load is at most 4/3 of the optimum. Returns
    one sorted index array per rank. Every rank computes the same partition
    from the same sizes, so no collective is needed."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if ws < 1:
        raise ValueError("world size must be at least 1")
    if sizes.ndim != 1 or (sizes < 1).any():
        raise ValueError("replica sizes must be a list of positive bead counts")
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load = [0] * ws
    parts = [[] for _ in range(ws)]
    for k in order:
        r = min(range(ws), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += int(sizes[k])
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def local_replicas(sizes, seeds, ws, rank):
    """This rank's share of a fixed ensemble (strong scaling): the global
    indices from split_replicas and their sizes and seeds. A replica keeps its
    global seed, so its trajectory does not depend on the number of ranks."""
    if not 0 <= rank < ws:
        raise ValueError("rank %d outside a world of %d" % (rank, ws))
    sizes = np.asarray(sizes)
    seeds = np.asarray(seeds, dtype=np.uint64)
    if seeds.shape != sizes.shape:
        raise ValueError("one seed per replica is needed")
    idx = split_replicas(sizes, ws)[rank]
    return idx, sizes.astype(np.int32)[idx], seeds[idx]


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(v, ws):
    """The largest v over all ranks (every rank receives it)."""
    if ws == 1:
        return float(v)
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, ws, seconds):
    """Units processed by all ranks per second of the slowest rank's time."""
    return ws * float(units_per_rank) / float(seconds)
