"""Host logic of the multi-GPU runs: one process per GPU, each advancing its own
independent systems (the path partitions into systems; there is no data-path
collective). Used by bench.py, ensemble.py and serving.py under torchrun; the
collectives here only aggregate timings and results (NCCL on GPUs, gloo on CPU
in the tests)."""
import os

import numpy as np


def dist_env():
    """(rank, world, local_rank) from torchrun's environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value, device=None):
    """Largest value over ranks (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, steps, seconds, world):
    """Units processed by all ranks per second of the slowest rank (weak scaling)."""
    return world * units_per_rank * steps / seconds


def shard(items, rank, world):
    """This rank's share of independent work items: every world-th item from rank,
    so each item runs on exactly one rank and the shares differ by at most one."""
    return items[rank::world]


def gather_values(values, device=None):
    """All ranks' 1-D float arrays concatenated in rank order (e.g. per-request
    latencies, for whole-job percentiles)."""
    import torch
    import torch.distributed as dist

    values = np.asarray(values, np.float64)
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return values
    world = dist.get_world_size()
    n = torch.tensor([len(values)], dtype=torch.int64, device=device)
    sizes = [torch.zeros(1, dtype=torch.int64, device=device) for _ in range(world)]
    dist.all_gather(sizes, n)
    m = int(max(int(x.item()) for x in sizes))
    buf = torch.zeros(max(m, 1), dtype=torch.float64, device=device)
    buf[: len(values)] = torch.as_tensor(values, dtype=torch.float64)
    parts = [torch.zeros(max(m, 1), dtype=torch.float64, device=device) for _ in range(world)]
    dist.all_gather(parts, buf)
    return np.concatenate([p[: int(sz.item())].cpu().numpy() for p, sz in zip(parts, sizes)])
