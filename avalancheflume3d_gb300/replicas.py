"""Independent replicas across ranks (one process per GPU).

The clump-DEM step has no exchange between flumes, so N GPUs run N independent flumes (weak
scaling) with no collective on the data path.  The only collectives are the timing ones: a
barrier on both sides of the timed region and a max over ranks of the elapsed time, so that the
reported throughput is all ranks' clump-steps divided by the slowest rank's time.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Ranks:
    rank: int
    world: int
    local: int

    @property
    def distributed(self) -> bool:
        return self.world > 1


def from_env() -> Ranks:
    """RANK / WORLD_SIZE / LOCAL_RANK as torch.distributed.run sets them (defaults: one rank)."""
    return Ranks(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                 int(os.environ.get("LOCAL_RANK", "0")))


def init(r: Ranks, backend: str = "nccl", device=None) -> None:
    if not r.distributed:
        return
    import torch.distributed as dist
    kw = {}
    if device is not None:
        kw["device_id"] = device
    dist.init_process_group(backend, **kw)


def barrier(r: Ranks) -> None:
    if r.distributed:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(r: Ranks, value: float, device=None) -> float:
    """The largest `value` over all ranks (the slowest rank's elapsed time)."""
    if not r.distributed:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(r: Ranks, units_per_rank: float, seconds_local: float, device=None) -> float:
    """Whole-job units per second: every rank's units over the slowest rank's time."""
    slowest = max_over_ranks(r, seconds_local, device)
    return r.world * units_per_rank / slowest if slowest > 0 else 0.0


def finalize(r: Ranks) -> None:
    if r.distributed:
        import torch.distributed as dist
        dist.destroy_process_group()
