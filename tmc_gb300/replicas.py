"""Replicas across GPUs for bench.py: one process per GPU, launched by torch.distributed.run.

Extraction does not shard: each rank extracts its own volume (seeded by its rank) with no
collective on the data path, so the work per GPU stays fixed as ranks are added (weak scaling).
The only collectives are the timing ones: a barrier on both sides of the timed region and the
maximum of the ranks' times, from which the whole-job throughput is computed.  The backend is NCCL
on GPUs and gloo on CPUs (the multi-rank tests).
"""
import os


def dist_env():
    """(rank, world size, local rank) from the torch.distributed.run environment (1 rank without it)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def replica_seed(base: int, rank: int) -> int:
    """The seed of rank `rank`'s volume: every replica extracts a different volume of the same kind."""
    return base + rank


def reports(rank: int) -> bool:
    """Rank 0 alone prints the JSON line (and runs the CPU baselines)."""
    return rank == 0


def throughput(world: int, cells_per_rank: int, steps: int, seconds: float) -> float:
    """Whole-job Gcells/s: the cells all ranks processed over the slowest rank's time."""
    return world * cells_per_rank * steps / seconds / 1e9


class Replicas:
    """The process group of a multi-rank run (nothing to do for one rank)."""

    def __init__(self, world: int, backend: str = "nccl", local: int = 0):
        self.world = world
        self.backend = backend
        self.local = local
        if world > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", local))
            else:
                dist.init_process_group(backend)

    def _device(self):
        return f"cuda:{self.local}" if self.backend == "nccl" else "cpu"

    def barrier(self):
        """All ranks reach this point (after the caller synchronised its own device work)."""
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_over_ranks(self, x: float) -> float:
        """The largest value of x over the ranks (the slowest rank's time)."""
        if self.world == 1:
            return x
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], device=self._device(), dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
