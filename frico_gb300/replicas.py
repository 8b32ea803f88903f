"""Multi-GPU layout of the hot path: independent replicas, one process per GPU.

FRICO's solver (src/emw_solver.h:92-167, src/emw_ana_antenna.cpp,
src/emw_ana_bistatic_rcs.cpp) has no exchange step between frequencies,
excitations or geometries: each solve owns its Z, its factors and its fields.
Several GPUs therefore run independent solves (a frequency sweep is split
into contiguous blocks of frequencies, one block per rank) and only the
bookkeeping crosses ranks: a barrier around the timed region, the maximum of
the per-rank times, and the gather of per-frequency results to rank 0. The
data path has no collective.

The process group is whatever torch.distributed offers (gloo on the host,
which is enough for these small host-side exchanges; the tensors involved are
a handful of floats per frequency).
"""
from __future__ import annotations

import os
from typing import Any, Sequence


def shard_bounds(n_items: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of the contiguous block of `n_items` owned by `rank` of `world`.
    The first n_items % world ranks take one extra item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    if n_items < 0:
        raise ValueError("n_items must be >= 0")
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard(items: Sequence[Any], rank: int, world: int) -> list:
    lo, hi = shard_bounds(len(items), rank, world)
    return list(items[lo:hi])


class ReplicaGroup:
    """Host-side coordination of `world` replicas (rank from the environment
    when not given). With world == 1 every method is a no-op."""

    def __init__(self, world: int | None = None, rank: int | None = None, backend: str = "gloo"):
        self.world = int(os.environ.get("WORLD_SIZE", "1")) if world is None else world
        self.rank = int(os.environ.get("RANK", "0")) if rank is None else rank
        self._td = None
        if self.world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if not td.is_initialized():
                td.init_process_group(backend, rank=self.rank, world_size=self.world)
            self._td = td

    def barrier(self) -> None:
        if self._td is not None:
            self._td.barrier()

    def max(self, x: float) -> float:
        if self._td is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._td.all_reduce(t, op=self._td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self._td is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self._td.all_reduce(t, op=self._td.ReduceOp.SUM)
        return float(t.item())

    def gather_rows(self, rows, n_total: int):
        """Concatenate each rank's block of result rows (numpy, same trailing
        shape and dtype on every rank, block sizes from shard_bounds) on every
        rank, in global order."""
        import numpy as np
        rows = np.ascontiguousarray(rows)
        if self._td is None:
            return rows
        import torch
        lo, hi = shard_bounds(n_total, self.rank, self.world)
        if rows.shape[0] != hi - lo:
            raise ValueError(f"rank {self.rank} holds {rows.shape[0]} rows, its shard is {hi - lo}")
        real = rows.view(np.float64) if rows.dtype == np.complex128 else rows.astype(np.float64, copy=False)
        width = int(np.prod(real.shape[1:])) if real.ndim > 1 else 1
        full = torch.zeros((n_total, width), dtype=torch.float64)
        if hi > lo:
            full[lo:hi] = torch.from_numpy(real.reshape(hi - lo, width))
        self._td.all_reduce(full, op=self._td.ReduceOp.SUM)   # disjoint blocks: a concatenation
        out = full.numpy().reshape((n_total,) + real.shape[1:])
        return out.view(np.complex128) if rows.dtype == np.complex128 else out.astype(rows.dtype, copy=False)

    def close(self) -> None:
        if self._td is not None and self._td.is_initialized():
            self._td.destroy_process_group()
        self._td = None
