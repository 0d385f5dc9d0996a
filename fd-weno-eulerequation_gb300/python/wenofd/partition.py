"""x-slab decomposition of one solve over ranks, on torch.distributed.

The reference's only parallel strategy is MPI over x-slabs: near-equal slabs
with the remainder on the low ranks, y never split (src/WENOFD.cpp:36-70); a
4-column ghost exchange with the x neighbours, periodic in rank order, before
every right-hand side (exchangeGhostCellsValue, src/WENOFD.cpp:850-929); and
the minimum of the ranks' time steps (src/WENOFD.cpp:444-449).

On GB300 one whole-domain solve lives on one GPU, so the GPU path runs
replicas; this module is the host-side partition logic of a sharded run,
exercised among CPU ranks (gloo).  Handed device tensors under NCCL, the same
calls move the halos between GPUs.

A slab array is [4][count + 8][ny + 8] (float64, ej fastest): the rank's
nodes [start, start + count) of the x interior at columns 4 .. 4 + count,
4 ghost columns on each side, all y nodes with their 4 ghost rows.
"""
from __future__ import annotations

import numpy as np

GHOST = 4


def slab_partition(nx: int, world: int) -> list[tuple[int, int]]:
    """(first interior node, node count) of every rank's slab
    (src/WENOFD.cpp:47-61: nx // world each, one more on the first
    nx % world ranks)."""
    if world < 1 or nx < 1:
        raise ValueError("nx and world must be positive")
    base, rem = divmod(nx, world)
    out, start = [], 0
    for r in range(world):
        n = base + (1 if r < rem else 0)
        out.append((start, n))
        start += n
    return out


class SlabExchange:
    """Ghost-column exchange and time-step reduction of one rank's slab."""

    def __init__(self, nx: int, ny: int, rank: int | None = None, world: int | None = None, group=None):
        import torch.distributed as dist

        self._dist = dist
        self.group = group
        self.rank = dist.get_rank(group) if rank is None else rank
        self.world = dist.get_world_size(group) if world is None else world
        self.nx, self.ny = nx, ny
        self.parts = slab_partition(nx, self.world)
        self.start, self.count = self.parts[self.rank]
        # rank 0 and the last rank skip the duplicated periodic end node, so
        # every slab sends 4 columns from at least 5 nodes
        if min(n for _, n in self.parts) < GHOST + 1:
            raise ValueError(f"{nx} x nodes over {self.world} ranks leaves a slab with fewer than {GHOST + 1} nodes")
        self.left = (self.rank - 1) % self.world
        self.right = (self.rank + 1) % self.world

    @property
    def left_edge(self) -> bool:
        """This slab holds the domain's left boundary (rank 0)."""
        return self.rank == 0

    @property
    def right_edge(self) -> bool:
        return self.rank == self.world - 1

    def _tensor(self, U):
        import torch

        if isinstance(U, np.ndarray):
            if U.dtype != np.float64 or not U.flags.c_contiguous:
                raise ValueError("expected a C-contiguous float64 slab")
            return torch.from_numpy(U)
        return U

    def exchange(self, U) -> None:
        """Fill the 4 ghost columns on each side of the interior rows from
        the x neighbours (src/WENOFD.cpp:850-929): the left neighbour's last
        4 columns into the left ghosts, the right neighbour's first 4 into the
        right ghosts, periodic in rank order; rank 0 sends its columns 2..5
        and the last rank its columns n-5..n-2, skipping the periodic
        duplicate node.  Edge ranks of a non-periodic domain overwrite their
        outer ghosts with the boundary condition afterwards (setBoundary)."""
        import torch

        T = self._tensor(U)
        if tuple(T.shape) != (4, self.count + 2 * GHOST, self.ny + 2 * GHOST):
            raise ValueError(f"slab shape {tuple(T.shape)} != (4, {self.count + 2 * GHOST}, {self.ny + 2 * GHOST})")
        sx, ex, sy, ey = GHOST, GHOST + self.count, GHOST, GHOST + self.ny
        lo = 1 if self.rank == 0 else 0
        hi = 1 if self.rank == self.world - 1 else 0
        send_left = T[:, sx + lo:sx + lo + GHOST, sy:ey].contiguous()
        send_right = T[:, ex - GHOST - hi:ex - hi, sy:ey].contiguous()
        if self.world == 1:
            recv_left, recv_right = send_right, send_left
        else:
            d = self._dist
            recv_left, recv_right = torch.empty_like(send_left), torch.empty_like(send_right)
            reqs = [d.irecv(recv_left, src=self.left, tag=1, group=self.group),
                    d.irecv(recv_right, src=self.right, tag=2, group=self.group),
                    d.isend(send_right, dst=self.right, tag=1, group=self.group),
                    d.isend(send_left, dst=self.left, tag=2, group=self.group)]
            for r in reqs:
                r.wait()
        T[:, sx - GHOST:sx, sy:ey] = recv_left
        T[:, ex:ex + GHOST, sy:ey] = recv_right

    def min_dt(self, local_dt: float, device=None) -> float:
        """The step all ranks take: the minimum of the ranks' clipped local
        steps (src/WENOFD.cpp:444-449).  NaN propagates (each rank checks
        its own before, as the reference does)."""
        import torch

        if self.world == 1:
            return float(local_dt)
        t = torch.tensor([local_dt], dtype=torch.float64, device=device)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MIN, group=self.group)
        return float(t.item())

    def gather_interior(self, interior, device=None):
        """The whole [4][nx][ny] interior on every rank from the slabs'
        [4][count][ny] interiors (GatherAllUhToRank0's result, on all ranks)."""
        import torch

        T = self._tensor(interior)
        if self.world == 1:
            return T.clone()
        width = max(n for _, n in self.parts)
        pad = torch.zeros((4, width, self.ny), dtype=T.dtype, device=T.device if device is None else device)
        pad[:, :self.count] = T
        bufs = [torch.empty_like(pad) for _ in range(self.world)]
        self._dist.all_gather(bufs, pad, group=self.group)
        return torch.cat([b[:, :n] for b, (_, n) in zip(bufs, self.parts)], dim=1)
