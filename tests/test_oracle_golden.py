"""The CPU restatement (oracle/) against the reference's own outputs.

The fixtures come from the reference's unmodified sources compiled with
-ffp-contract=off (tests/golden/make_golden.py).  The restatement must agree
with them bit for bit: same initial state, same ghost fill, same RHS, same
time steps, same state after N steps.  The published convergence rows
(README.md:67-74) pin it independently of any build.
"""
import numpy as np
import pytest

import oracle as orc
from conftest import assert_same, fixture_id, fixture_paths, load_fixture

NG = orc.NG


def _problem(meta):
    return orc.Problem(meta["testcase"], meta["nx"], meta["ny"], meta["scheme"], meta["rk"],
                       meta["cfl"], meta["seed"], meta["t_end"])


@pytest.mark.parametrize("path", fixture_paths("rhs_"), ids=fixture_id)
def test_rhs_matches_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    p = _problem(m)
    assert p.grid.dx == m["dx"] and p.grid.dy == m["dy"]
    # the oracle's own initial condition equals the reference's initializeAve
    assert_same(p.interior(), fx["init"], "initial state")
    p.set_interior(fx["init"])
    rhs = p.assemble_rhs()
    assert_same(rhs, fx["rhs"], "rhs")
    # the whole array after the boundary fill, every ghost node included
    assert_same(p.U, fx["ghosted"], "state with ghosts")
    assert p.calc_dt() == float(fx["dt"])


@pytest.mark.parametrize("path", fixture_paths("run_"), ids=fixture_id)
def test_run_matches_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    p = _problem(m)
    p.set_interior(fx["init"])
    steps, dts = p.run(max_steps=m["steps"])
    assert steps == m["steps"]
    assert_same(dts, fx["dts"], "time steps")
    assert_same(p.interior(), fx["state"], "state")


def test_wenoz_translation_and_symmetry():
    # WENO-Z reproduces constants and linear data exactly in exact arithmetic;
    # in FP64 to rounding.
    assert orc.weno5(orc.WENOZ, 2.0, 2.0, 2.0, 2.0, 2.0) == pytest.approx(2.0, abs=1e-15)
    assert orc.weno5(orc.WENOZ, 1.0, 2.0, 3.0, 4.0, 5.0) == pytest.approx(3.5, abs=1e-14)
    w = orc.wenoz_weights(1.0, 1.1, 1.2, 1.3, 1.4)
    assert w == pytest.approx([0.1, 0.6, 0.3], abs=1e-12)


def test_eigenvectors_are_inverse():
    rng = np.random.default_rng(0)
    for direction in (0, 1):
        for _ in range(20):
            rho = rng.uniform(0.1, 2.0)
            u, v = rng.uniform(-1, 1, 2)
            p = rng.uniform(0.05, 2.0)
            U = [rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)]
            L, R = orc.eigen_lr(direction, 1.4, U)
            assert np.allclose(L @ R, np.eye(4), atol=1e-12)


def test_flux_split_sums_to_physical_flux():
    U = np.array([1.2, 0.3, -0.2, 2.5])
    for d in (0, 1):
        fm, fp = orc.flux_split(d, 1.4, U)
        F = np.zeros(4)
        orc.lib().orc_phys_flux(d, 1.4, orc._p(U), orc._p(F))
        assert np.allclose(fm + fp, F, rtol=1e-15, atol=1e-15)


# README.md:67-74 (WENO-JS and WENO-Z, RK3, CFL 0.05, t=1, smooth case): the
# printed three digits of Linf and L1 at N=100.
README_N100 = {orc.WENOZ: (1.66e-07, 4.21e-08), orc.WENOJS: (6.42e-07, 1.92e-07)}


@pytest.mark.parametrize("scheme", [orc.WENOZ, orc.WENOJS], ids=["wenoz", "wenojs"])
def test_readme_convergence_row_n100(scheme):
    p = orc.Problem(orc.SMOOTH, 100, 100, scheme, rk=2, cfl=0.05)
    steps, _ = p.run()
    assert p.now == pytest.approx(1.0, abs=1e-9)
    linf, l1, _ = p.error_norms()
    want_inf, want_l1 = README_N100[scheme]
    assert f"{linf:.2e}" == f"{want_inf:.2e}"
    assert f"{l1:.2e}" == f"{want_l1:.2e}"
    # and the exact values of the reference built with -ffp-contract=off
    exact = {orc.WENOZ: (1.661938627828263e-07, 4.2102026724544218e-08),
             orc.WENOJS: (6.4235668695289405e-07, 1.9170672280854889e-07)}[scheme]
    assert linf == pytest.approx(exact[0], rel=1e-12)
    assert l1 == pytest.approx(exact[1], rel=1e-9)
