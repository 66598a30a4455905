"""Multi-GPU runs of the path: replicas only.

Images, batch items and requests are independent, and a vertical sweep is a
chain along a whole column, so the path does not shard: every rank runs an
independent replica on its own GPU.  The only collectives are the timing
barrier and a max over ranks of the timed duration; the whole-job rate is
the units all ranks processed divided by that slowest rank's time.
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def env_ranks():
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over the ranks of the default process group
    (the value itself without one)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_step: float, steps: int, world: int, ms_max: float) -> float:
    """Units per second of the whole job: every rank processed
    units_per_step * steps units; the job took the slowest rank's time."""
    return units_per_step * steps * world / (ms_max / 1e3)


def replica_seed(base: int, rank: int) -> int:
    """Each replica synthesises its own inputs."""
    return base + rank
