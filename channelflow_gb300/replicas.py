"""Replica runs under torchrun: one independent DNS per rank (the DNS of one field does not shard), no
collective in the data path; the ranks only meet to bracket the timed region with barriers and to take the
slowest rank's time.

The aggregate throughput counts the steps of all ranks over the slowest rank's time (weak scaling: per-rank
work fixed).  NCCL on GPUs, gloo on the host (the CPU tests run two gloo ranks).
"""

from __future__ import annotations

import os


class Replicas:
    def __init__(self, rank: int = 0, world: int = 1):
        self.rank, self.world = int(rank), int(world)
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            use_nccl = torch.cuda.is_available()
            if use_nccl:
                torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", self.rank)))
                self.device = "cuda"
            if not dist.is_initialized():
                dist.init_process_group("nccl" if use_nccl else "gloo", rank=self.rank, world_size=self.world)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max_over_ranks(self, x: float) -> float:
        if not self.dist:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds_max: float) -> float:
        """Whole-job rate: the units every rank processed over the slowest rank's time."""
        return self.world * float(units_per_rank) / float(seconds_max)

    def close(self):
        if self.dist and self.dist.is_initialized():
            self.dist.destroy_process_group()
        self.dist = None
