"""x-slab decomposition among CPU ranks (gloo, world sizes 2 and 3).

Each rank holds its slab of the oracle's state, exchanges ghost columns with
the product's wenofd.partition.SlabExchange, applies the boundary conditions
its slab owns, and computes its RHS with the oracle.  The ghosted slabs, the
RHS and several SSP-RK3 steps (dt from the ranks' minimum) must equal the
whole-domain oracle bit for bit: the reference's multi-rank decomposition
(src/WENOFD.cpp:36-70, 850-929, 444-449) changes no arithmetic."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle as orc
from wenofd.partition import GHOST, SlabExchange, slab_partition

CASES = [  # (testcase, nx, ny, seed): periodic, symmetric, SPECIAL x + SLIP y + gravity, SPECIAL x
    (orc.SHEAR, 40, 24, 7),
    (orc.RIEMANN_SEEDED, 37, 29, 11),
    (orc.RTI, 23, 48, 0),
    (orc.RIEMANN1, 31, 26, 0),
]
STEPS = 3


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, case: tuple) -> None:
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tc, nx, ny, seed = case
        whole = orc.Problem(tc, nx, ny, orc.WENOZ, 2, 0.6, seed=seed)
        ex = SlabExchange(nx, ny)
        assert (ex.start, ex.count) == slab_partition(nx, world)[rank]
        slab = orc.Slab(whole, ex.start, ex.count)
        cols = slice(ex.start, ex.start + ex.count + 2 * GHOST)

        # ghosts: exchange + the slab's own conditions == whole-domain fill
        slab.U[:, :GHOST] = np.nan
        slab.U[:, -GHOST:] = np.nan
        slab.U[:, :, :GHOST] = np.nan
        slab.U[:, :, -GHOST:] = np.nan
        ex.exchange(slab.U)
        slab.fill_boundary(ex.left_edge, ex.right_edge)
        whole.fill_boundary()
        assert np.array_equal(slab.U, whole.U[:, cols, :], equal_nan=True), "ghosted slab"

        # the slab's RHS == its part of the whole-domain RHS
        rhs = slab.assemble_rhs()
        ref_rhs = whole.assemble_rhs()[:, ex.start:ex.start + ex.count]
        assert np.array_equal(rhs, ref_rhs), "slab RHS"

        # SSP-RK3 steps (RunRK3, src/WENOFD.cpp:352-396) with the ranks' dt
        ref = orc.Problem(tc, nx, ny, orc.WENOZ, 2, 0.6, seed=seed)
        now = 0.0
        for _ in range(STEPS):
            dt = ex.min_dt(slab.local_dt(0.6, now, ref.t_end))
            assert dt == ref.calc_dt(), "time step"
            ref.rk_step(dt)
            Un = slab.U.copy()
            for a, b, c in ((1.0, 0.0, 1.0), (3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0), (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0)):
                ex.exchange(slab.U)
                slab.fill_boundary(ex.left_edge, ex.right_edge)
                slab.assemble_rhs()
                i = (slice(None), slice(GHOST, GHOST + ex.count), slice(GHOST, GHOST + ny))
                slab.U[i] = a * Un[i] + b * slab.U[i] + c * dt * slab.rhs[i]
            now += dt
            ref.now = now
        full = ex.gather_interior(np.ascontiguousarray(slab.interior())).numpy()
        assert np.array_equal(full, ref.interior()), "state after steps"
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"tc{c[0]}_{c[1]}x{c[2]}")
def test_slab_ranks_equal_whole_domain(world, case):
    mp.spawn(_worker, args=(world, _free_port(), case), nprocs=world, join=True)


@pytest.mark.parametrize("nx,world", [(37, 3), (40, 2), (4096, 6), (101, 7), (9, 1), (64, 64)])
def test_slab_partition_matches_reference_rule(nx, world):
    parts = slab_partition(nx, world)
    base, rem = nx // world, nx % world
    assert [n for _, n in parts] == [base + (r < rem) for r in range(world)]
    assert parts[0][0] == 0 and all(parts[r][0] == parts[r - 1][0] + parts[r - 1][1] for r in range(1, world))
    assert sum(n for _, n in parts) == nx


def test_slab_too_thin_is_rejected():
    with pytest.raises(ValueError):
        SlabExchange(9, 10, rank=0, world=2)  # 5 + 4 nodes


def test_single_rank_exchange_is_the_periodic_fill():
    p = orc.Problem(orc.SHEAR, 20, 12, orc.WENOZ, 2, 0.6, seed=2)
    ex = SlabExchange(20, 12, rank=0, world=1)
    slab = orc.Slab(p, 0, 20)
    ex.exchange(slab.U)
    slab.fill_boundary(True, True)
    p.fill_boundary()
    assert np.array_equal(slab.U, p.U)
