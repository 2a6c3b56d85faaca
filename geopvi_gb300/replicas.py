"""Replica runs over ranks, for the bench and for drivers that spread VI work.

The (sample, shot) solves are independent and a sample's shots are summed on
the GPU that ran them, so the multi-GPU form is replicas: every rank (one
process per GPU, launched by torch.distributed.run) solves its own batch and
no tensor of the data path crosses ranks.  Only the host bookkeeping is
collective: a barrier around timed regions, the maximum of the ranks' times
(the job ends when the slowest rank does), and one reporting rank.  Throughput
is the units all ranks processed over that maximum (weak scaling).
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


class ReplicaGroup:
    """RANK / WORLD_SIZE / LOCAL_RANK from the environment; a process group
    only when there is more than one rank (NCCL with a device, gloo without)."""

    def __init__(self, device: torch.device | None = None, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device
        self._own = False
        if self.world > 1 and not dist.is_initialized():
            if backend is None:
                backend = "nccl" if device is not None and device.type == "cuda" else "gloo"
            kw = {"device_id": device} if backend == "nccl" and device is not None else {}
            dist.init_process_group(backend, **kw)
            self._own = True

    @property
    def reporter(self) -> bool:
        return self.rank == 0

    def barrier(self) -> None:
        if self.world > 1:
            dist.barrier()

    def max_seconds(self, seconds: float) -> float:
        """The slowest rank's time."""
        if self.world == 1:
            return float(seconds)
        dev = self.device if self.device is not None and dist.get_backend() == "nccl" else torch.device("cpu")
        t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds_max: float) -> float:
        """Whole-job rate: every rank's units over the slowest rank's time."""
        return units_per_rank * self.world / seconds_max

    def close(self) -> None:
        if self._own and dist.is_initialized():
            dist.destroy_process_group()
            self._own = False
