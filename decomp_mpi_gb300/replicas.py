"""Independent replicas of the reshape + split-FFT path, one per GPU.

The reference spreads one global array over MPI ranks.  Here every rank of
that processor grid is a virtual rank inside one GPU's memory, so the whole
path runs on one GPU and nothing in it exchanges data between GPUs.  Several
GPUs therefore run several independent replicas, each on its own array.  This
module is the host-side coordination of such a run, launched one process per
GPU by ``torch.distributed.run``: rank discovery from the launcher's
environment, the barrier that brackets a timed region and the maximum of the
timed durations over the replicas.  There is no collective on the data path.
"""
from __future__ import annotations

import os


class Replicas:
    """One process's view of an N-replica run (N = 1 without a launcher)."""

    def __init__(self, env=None):
        env = os.environ if env is None else env
        self.world = int(env.get("WORLD_SIZE", "1"))
        self.rank = int(env.get("RANK", "0"))
        self.local_rank = int(env.get("LOCAL_RANK", "0"))
        self._dist = None
        self._device = "cpu"

    @property
    def leader(self) -> bool:
        return self.rank == 0

    def gpu_index(self, env=None) -> str:
        """The nvidia-smi index of this replica's GPU."""
        env = os.environ if env is None else env
        vis = env.get("CUDA_VISIBLE_DEVICES")
        if vis:
            ids = [x.strip() for x in vis.split(",") if x.strip()]
            if self.local_rank < len(ids):
                return ids[self.local_rank]
        return str(self.local_rank)

    def init(self, backend: str) -> None:
        """Join the process group (``nccl`` for GPU replicas, ``gloo`` on CPU); no-op for one replica."""
        if self.world <= 1:
            return
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend=backend)
        self._dist = dist
        self._device = "cuda:%d" % torch.cuda.current_device() if backend == "nccl" else "cpu"

    def barrier(self) -> None:
        if self._dist is not None:
            import torch
            # an all-reduce of one element, on the backend's own device: a barrier that works on
            # gloo and nccl alike without naming device ids
            t = torch.zeros(1, dtype=torch.float64, device=self._device)
            self._dist.all_reduce(t)
            if self._device != "cpu":
                torch.cuda.synchronize()

    def max(self, values):
        """Element-wise maximum of a list of floats over all replicas."""
        return self._reduce(values, "max")

    def sum(self, values):
        """Element-wise sum of a list of floats over all replicas."""
        return self._reduce(values, "sum")

    def _reduce(self, values, how):
        vals = [float(v) for v in values]
        if self._dist is None:
            return vals
        import torch
        t = torch.tensor(vals, dtype=torch.float64, device=self._device)
        op = self._dist.ReduceOp.MAX if how == "max" else self._dist.ReduceOp.SUM
        self._dist.all_reduce(t, op=op)
        return [float(x) for x in t.cpu().tolist()]

    def close(self) -> None:
        if self._dist is not None and self._dist.is_initialized():
            self._dist.destroy_process_group()
        self._dist = None
