"""Replica plumbing for several GPUs of one node.

The stencil path does not shard: one grid would need a halo exchange along
i that the reference never defines (its MPI scaffold exchanges nothing,
main.cpp:210-220).  Several GPUs therefore run independent replicas -- one
grid per GPU, or, in the batching form, a disjoint share of the grids -- and
only the timing meets: a barrier before and after the timed region and the
maximum of the per-rank times.  The process group is gloo on the host, so no
collective touches the device data path.
"""
import os


class Replicas:
    """Rank/world from the torchrun environment; gloo barrier and reductions."""

    def __init__(self, backend="gloo"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self._td = None
        if self.world > 1:
            import torch.distributed as td
            if not td.is_initialized():
                td.init_process_group(backend)
            self._td = td

    def barrier(self):
        if self._td is not None:
            self._td.barrier()

    def _reduce(self, x, op):
        if self._td is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, None if self._td is None else self._td.ReduceOp.MAX)

    def sum(self, x):
        return self._reduce(x, None if self._td is None else self._td.ReduceOp.SUM)

    def close(self):
        if self._td is not None and self._td.is_initialized():
            self._td.destroy_process_group()
        self._td = None


def shard(n_items, rank, world):
    """Indices of a disjoint, balanced share of n_items for one rank
    (round robin, so uneven item sizes spread across ranks)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return list(range(rank, n_items, world))
