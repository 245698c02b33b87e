"""Independent replicas of a workload, one process per GPU.

The path has no exchange between plates, so N GPUs run N independent replicas (one plate,
or one batch of plates, per rank) with no data-path collective; the only collectives are
the timing barrier and the max over ranks of a measured time. Launched by torchrun
(RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* from the environment); NCCL when CUDA is
available, gloo otherwise.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", str(self.rank)))
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = "cuda"
            dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist

            dist.barrier()

    def max(self, v: float) -> float:
        """The largest value over the ranks (a per-rank time: the job's time)."""
        if self.world == 1:
            return float(v)
        import torch
        import torch.distributed as dist

        t = torch.tensor([float(v)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            import torch.distributed as dist

            if dist.is_initialized():
                dist.destroy_process_group()
