"""Replica bookkeeping for multi-GPU runs of the (non-sharded) path.

The assembly path does not shard: every rank runs the same workload on its
own GPU (replicas), with no collective on the data path.  Ranks meet only to
start the timed region together and to agree on its duration (the maximum
over ranks); the job's throughput is the units of all ranks over that time.
torch.distributed (gloo) carries these two host-side exchanges.
"""
import os


def dist_env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Replicas:
    """Barrier and max-over-ranks on a gloo process group (no-ops for one rank)."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, value):
        """The maximum of `value` over all ranks (every rank gets it)."""
        if not self.dist:
            return float(value)
        import torch
        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank, ms_per_step_this_rank):
        """(job throughput in units/s, max ms per step): all ranks' units over
        the slowest rank's time."""
        ms = self.max(ms_per_step_this_rank)
        return self.world * units_per_rank / (ms * 1e-3), ms

    def close(self):
        if self.dist and self.dist.is_initialized():
            self.dist.destroy_process_group()
