"""wenofd.refine: the shear layer's initial state on the 2x finer node grid
from the coarse one (same perturbation), for accuracy studies against a
finer solution.  Checked against the oracle's initial state on the CPU."""
import numpy as np

import oracle as orc
from wenofd.refine import prolong_nodes, shear_layer_refined


def test_prolongation_keeps_coarse_nodes_and_linear_fields():
    rng = np.random.default_rng(3)
    c = rng.standard_normal((5, 7))
    f = prolong_nodes(c)
    assert f.shape == (9, 13)
    assert np.array_equal(f[::2, ::2], c)
    x, y = np.meshgrid(np.arange(5.0), np.arange(7.0), indexing="ij")
    xf, yf = np.meshgrid(np.arange(9.0) / 2, np.arange(13.0) / 2, indexing="ij")
    assert np.allclose(prolong_nodes(2 * x - 3 * y + 1), 2 * xf - 3 * yf + 1, rtol=0, atol=1e-14)


def test_refined_shear_layer_matches_the_coarse_state_at_coarse_nodes():
    n = 17
    coarse = orc.Problem(orc.SHEAR, n, n, orc.WENOZ, 2, 0.7, seed=2024).interior()
    fine = shear_layer_refined(coarse)
    assert fine.shape == (4, 2 * n - 1, 2 * n - 1)
    assert np.allclose(fine[:, ::2, ::2], coarse, rtol=1e-13, atol=1e-15)
    # periodic duplicates agree; the base state is the layer's
    assert np.array_equal(fine[:, -1, :], fine[:, 0, :]) and np.array_equal(fine[:, :, -1], fine[:, :, 0])
    assert set(np.unique(fine[0])) == {1.0, 2.0}
    p = 0.4 * (fine[3] - 0.5 * (fine[1] ** 2 + fine[2] ** 2) / fine[0])
    assert np.allclose(p, 2.5, rtol=1e-12)
    # the fine grid's own seeded initial state draws other noise
    own = orc.Problem(orc.SHEAR, 2 * n - 1, 2 * n - 1, orc.WENOZ, 2, 0.7, seed=2024).interior()
    assert np.max(np.abs(own[2, ::2, ::2] - coarse[2])) > 1e-4
