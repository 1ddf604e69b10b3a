"""Process-per-GPU replicas for benchmarks.

Worlds are independent, so a multi-GPU run is N replicas with no data-path collective:
each rank advances its own world(s); the only communication is a barrier around the timed
region and a max/sum of the per-rank results.  Launched by torch.distributed.run (RANK,
LOCAL_RANK, WORLD_SIZE, MASTER_ADDR/PORT from the environment).

With NCCL each rank is pinned to its GPU through CUDA_VISIBLE_DEVICES before any CUDA
call, so the library's kernels (its own CUDA runtime state) and torch both see that GPU as
device 0.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str = "nccl"):
        self.world_size = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world_size > 1:
            if backend == "nccl":
                visible = [d for d in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if d.strip()]
                os.environ["CUDA_VISIBLE_DEVICES"] = (visible[self.local_rank] if self.local_rank < len(visible)
                                                      else str(self.local_rank))
                import torch
                torch.cuda.set_device(0)
            import torch.distributed as dist
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self) -> None:
        if self.pg:
            self.pg.barrier()

    def _reduce(self, value: float, op: str) -> float:
        if not self.pg:
            return value
        import torch
        dev = "cuda:0" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=getattr(self.pg.ReduceOp, op))
        return float(t.item())

    def max(self, value: float) -> float:
        return self._reduce(value, "MAX")

    def sum(self, value: float) -> float:
        return self._reduce(value, "SUM")

    def close(self) -> None:
        if self.pg:
            self.pg.destroy_process_group()
            self.pg = None
