"""Independent replicas of a workload, one process per GPU (torchrun ranks).

HydroGPU runs one problem on one device and its update does not shard; N GPUs run N
independent replicas (weak scaling) with no data-path communication.  The process
group (gloo, host side only) carries the two things the measurement needs: a barrier
on both sides of the timed region and the maximum of the ranks' times.  The
whole-job rate is the units all ranks processed over that maximum."""
import os


class Replicas:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", 0))
        self.local_rank = int(os.environ.get("LOCAL_RANK", 0))
        self.world = int(os.environ.get("WORLD_SIZE", 1))
        self._dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self._dist = dist

    def barrier(self):
        if self._dist:
            self._dist.barrier()

    def max(self, x):
        """Maximum of x over the ranks (x itself on one rank)."""
        if not self._dist:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def rate(self, units_per_rank, seconds):
        """Whole-job rate: every rank's units over the slowest rank's time."""
        return units_per_rank * self.world / self.max(seconds)

    def close(self):
        if self._dist:
            self._dist.destroy_process_group()
            self._dist = None
