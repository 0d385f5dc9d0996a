"""Initial states of the seeded shear layer (TESTCASE 5) on a 2x finer node
grid, for accuracy studies against a finer solution.

The shear layer's perturbation is N(0, 1e-3) noise drawn per node from one
seeded stream, so two grids initialised from the same seed start from
different random fields: a finer solution of its own initial condition is
not a finer solution of the coarse problem, and the difference between the
two fields dominates any error measured against it.  ``shear_layer_refined``
builds the fine grid's initial state from the coarse one instead: the
layer's analytic base state (rho = 2 for |y - 0.5| < 0.25 else 1, u = +-0.5,
p = 2.5, v = 0.01 sin(4 pi x)) at the fine nodes, plus the coarse grid's own
perturbation of v prolonged bilinearly (fine node 2k = coarse node k).  Both
grids then solve the same problem up to the prolongation of the noise.
"""
from __future__ import annotations

import numpy as np


def prolong_nodes(c: np.ndarray) -> np.ndarray:
    """Bilinear prolongation of node values (n, m) to the 2x finer node grid
    (2n - 1, 2m - 1): even nodes are the coarse nodes, odd nodes the means of
    their two (or four) coarse neighbours."""
    n, m = c.shape
    f = np.empty((2 * n - 1, 2 * m - 1))
    f[::2, ::2] = c
    f[1::2, ::2] = 0.5 * (c[:-1, :] + c[1:, :])
    f[::2, 1::2] = 0.5 * (c[:, :-1] + c[:, 1:])
    f[1::2, 1::2] = 0.25 * (c[:-1, :-1] + c[1:, :-1] + c[:-1, 1:] + c[1:, 1:])
    return f


def _nodes(n: int) -> np.ndarray:
    # node coordinates of [0, 1] with n nodes, formed as the solver forms
    # them: (xl - 4 dx) + (i + 4) dx
    d = 1.0 / (n - 1)
    return (0.0 - d * 4) + (np.arange(n) + 4) * d


def shear_layer_refined(coarse: np.ndarray, gamma: float = 1.4) -> np.ndarray:
    """The fine grid's initial state [4][2n-1][2m-1] (conserved variables)
    for the coarse shear-layer state [4][n][m] at t = 0 (see the module
    docstring).  The periodic duplicate row and column copy the first ones,
    as the solver's own initial state does."""
    n, m = coarse.shape[1:]
    xc, yc = _nodes(n), _nodes(m)
    noise = coarse[2] / coarse[0] - 0.01 * np.sin(4 * np.pi * xc)[:, None]
    xf, yf = _nodes(2 * n - 1), _nodes(2 * m - 1)
    inside = np.abs(yf - 0.5) < 0.25
    rho = np.broadcast_to(np.where(inside, 2.0, 1.0)[None, :], (xf.size, yf.size))
    u = np.broadcast_to(np.where(inside, 0.5, -0.5)[None, :], (xf.size, yf.size))
    v = 0.01 * np.sin(4 * np.pi * xf)[:, None] + prolong_nodes(noise)
    E = 2.5 / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    fine = np.stack([rho, rho * u, rho * v, E])
    fine[:, -1, :] = fine[:, 0, :]
    fine[:, :, -1] = fine[:, :, 0]
    return np.ascontiguousarray(fine)
