"""The largest size of the specification (the 8192^2 shear layer) checked
through size-independent properties: on the doubly periodic shear layer the
flux-difference form conserves mass, both momenta and energy up to rounding
in every form, and the learned form's routing must not change that (a face
flux is shared by the two nodes it separates, whichever flux it takes).

The grid is node-based: the last row and column duplicate the first
(src/WENOFD.cpp:850-929 skips the duplicate when filling periodic ghosts), so
the conserved sums run over the unique nodes, without the last row and
column."""
import numpy as np
import pytest

import mlp_oracle
import wenofd

pytestmark = pytest.mark.gpu


def _sums_drift(n, precision, steps, params=None, interval=1):
    cfg = {"TESTCASE": 5, "ELEMNUMX": n, "ELEMNUMY": n, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1, "SEED": 2024,
           "PRECISION": precision, "INDICATOR_INTERVAL": interval}
    def sums(U):
        return np.array([U[r, :-1, :-1].sum() for r in range(4)]), np.array([np.abs(U[r, :-1, :-1]).sum()
                                                                             for r in range(4)])

    with wenofd.Solver(cfg) as s:
        s.initialize()
        if params is not None:
            s.set_indicator(params, 0.5)
        before, scale = sums(s.get_state())
        assert s.advance(max_steps=steps) == steps
        U = s.get_state()
        flagged = float(s.routing_flags().mean()) if params is not None else None
    assert np.all(np.isfinite(U))
    after, _ = sums(U)
    # relative to the sum of magnitudes (the momenta sum to about zero)
    drift = np.abs(after - before) / scale
    print(f"n={n} precision={precision} steps={steps}: drift {drift}")
    return drift, flagged


@pytest.mark.parametrize("precision,steps,bound", [(wenofd.FP64, 1, 1e-13), (wenofd.FP32, 3, 1e-11)])
def test_8192_shear_conserves(precision, steps, bound):
    drift, _ = _sums_drift(8192, precision, steps)
    assert np.all(drift <= bound), drift


def test_8192_learned_form_conserves():
    P = mlp_oracle.init_params(3)
    drift, flagged = _sums_drift(8192, wenofd.LEARNED, 3, P, interval=2)
    assert 0.0 < flagged < 1.0  # a mix of linear and WENO faces
    assert np.all(drift <= 1e-11), drift
