"""Host-side logic of the multi-GPU path: replicas only.

Each rank (one process per GPU, launched by torchrun) advances its own
ensemble member, seeded by its rank, with no exchange of model data.  The
only collectives are the ones the measurement needs: a barrier before and
after the timed region and a MAX over ranks of the elapsed time.  The
whole-job rate is then the sum over ranks of the simulated time advanced,
divided by that slowest rank's wall time (weak scaling: each rank does the
same fixed work).

The class is written against ``torch.distributed`` so the same code runs
with NCCL on GPUs (reductions on a CUDA tensor) and with gloo on CPU
(reductions on a host tensor), which is how the tests exercise it.
"""
import os


class ReplicaGroup:
    def __init__(self, backend=None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend
        self.dist = None
        if self.world > 1:
            import torch.distributed as tdist

            if not tdist.is_initialized():
                tdist.init_process_group(backend)
            self.dist = tdist
            self.backend = tdist.get_backend()

    @property
    def is_root(self):
        return self.rank == 0

    def member_seed(self, base=0):
        """Seed of this rank's ensemble member (members differ, no exchange)."""
        return base + self.rank

    def _device(self):
        return "cuda" if self.backend == "nccl" else "cpu"

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, x):
        """MAX of a per-rank float over all ranks (the slowest rank's time)."""
        if self.dist is None:
            return float(x)
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64, device=self._device())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def job_rate(self, units_per_rank, max_seconds):
        """Whole-job throughput: every rank processed ``units_per_rank`` units
        (e.g. simulated days) in at most ``max_seconds`` of wall time."""
        return units_per_rank * self.world / max_seconds

    def close(self):
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()
        self.dist = None
