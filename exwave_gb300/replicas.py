"""Replica runs: one process per GPU, each advancing its own independent
solves.  The solves do not exchange data, so there is no collective on the
data path; the ranks only meet at the barriers around a timed region and in
the reduction of its duration (the slowest rank decides the whole job's
time).  Launched by torchrun (RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR /
MASTER_PORT from the environment)."""
import os


def dist_info():
    """(world size, rank, local rank) from the torchrun environment."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Replicas:
    """Process group of the replicas (none for a single process).  backend
    "nccl" for GPU runs, "gloo" for host-only runs and tests."""

    def __init__(self, backend="nccl"):
        self.world_size, self.rank, self.local_rank = dist_info()
        self.backend = backend
        self._dist = None
        if self.world_size > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend)
            self._dist = dist

    def barrier(self):
        if self._dist is not None:
            self._dist.barrier()

    def max(self, value):
        """The largest of the ranks' values (every rank gets it)."""
        if self._dist is None:
            return float(value)
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self._dist is not None:
            self._dist.destroy_process_group()
            self._dist = None
