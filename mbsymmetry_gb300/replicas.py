"""Host side of an N-GPU run: independent replicas, one process per GPU.

The GW iteration is timed per replica (every rank runs the whole iteration on
its own GPU; the contractions are not sharded, no data-path collective), so
the time of one iteration is the maximum over ranks; the job completes
``world`` independent iterations in that time, reported separately as a
throughput.  This module holds that logic for ``bench.py`` so that it
runs, and is tested, the same way on CPU ranks (``gloo``) as on GPUs
(``nccl``)."""
import os

import torch
import torch.distributed as dist


def rank_info():
    """(rank, world size, local rank) from the torchrun environment (1 process: 0, 1, 0)."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Replicas:
    def __init__(self, backend: str = None, device: str = "cpu"):
        self.rank, self.world, self.local = rank_info()
        self.device = device
        if self.world > 1 and not dist.is_initialized():
            dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))

    def barrier(self):
        if self.device.startswith("cuda"):
            torch.cuda.synchronize()
        if self.world > 1:
            dist.barrier()

    def max_over_ranks(self, x: float) -> float:
        """The largest of the ranks' values (every rank gets it)."""
        if self.world == 1:
            return float(x)
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def seconds_per_iteration(self, ms_max: float) -> float:
        """Seconds per GW iteration of one crystal: the slowest replica's time.
        Replicas do not shard an iteration, so adding ranks does not shorten it."""
        return ms_max / 1e3

    def replica_throughput(self, ms_max: float) -> float:
        """Independent iterations the whole job completes per second (`world` in
        the slowest replica's time): throughput of copies, not a faster iteration."""
        return self.world / (ms_max / 1e3)

    @property
    def reports(self) -> bool:
        """Rank 0 prints the JSON line (and alone runs the reference arm)."""
        return self.rank == 0

    def close(self):
        if self.world > 1 and dist.is_initialized():
            dist.destroy_process_group()
