"""CUDA path (through the C ABI) against the reference's outputs and the oracle.

FP64 with WENO-JS / WENO-Z must equal the reference bit for bit (compared
with ==, so +0 and -0 agree): RHS, ghost fill, time step, and the state
after N steps.  WENO-ZP / WENO-ZPI evaluate the reference's pow(x, 2) as the
correctly rounded x*x while glibc's pow is off by one ulp on ~0.1% of inputs,
so those two schemes are held to a 1e-12 relative bound instead.  Whole runs
at the drop-in configuration's sizes (800^2 to t = 0.3, 4096^2 for 20 steps)
and against the reference built with its own flags are in
test_gpu_parity_long.py.
"""
import numpy as np
import pytest

import oracle as orc
import wenofd
from conftest import assert_same, fixture_id, fixture_paths, load_fixture

pytestmark = pytest.mark.gpu

NG = 4
REL_TOL_ZP = 1e-12  # WENO-ZP / ZPI only (pow(x, 2) rounding, see module doc)


def _config(meta, **extra):
    cfg = {"TESTCASE": meta["testcase"], "ELEMNUMX": meta["nx"], "ELEMNUMY": meta["ny"],
           "RKMETH": meta["rk"], "CFL": meta["cfl"], "SCHEME": meta["scheme"], "SEED": meta["seed"]}
    if meta.get("t_end") is not None:
        cfg["TEND"] = meta["t_end"]
    cfg.update(extra)
    return cfg


def _compare(a, b, scheme, what):
    if scheme in (orc.WENOZP, orc.WENOZPI):
        scale = np.maximum(np.abs(b), np.max(np.abs(b)) * 1e-3)
        assert np.max(np.abs(a - b) / scale) <= REL_TOL_ZP, what
    else:
        assert_same(a, b, what)


@pytest.mark.parametrize("path", fixture_paths("rhs_"), ids=fixture_id)
def test_get_flux_matches_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    with wenofd.Solver(_config(m)) as s:
        info = s.info()
        assert info.dx == m["dx"] and info.dy == m["dy"]
        s.set_state(fx["init"])
        rhs = s.get_flux()
        _compare(rhs, fx["rhs"], m["scheme"], "rhs")
        # every ghost node, corners included, as the reference fills them
        assert_same(s.get_state_ghosted(), fx["ghosted"], "state with ghosts after the boundary fill")
        assert s.calc_dt() == float(fx["dt"])


@pytest.mark.parametrize("path", fixture_paths("run_"), ids=fixture_id)
def test_steps_match_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    with wenofd.Solver(_config(m)) as s:
        s.set_state(fx["init"])
        dts = [s.step() for _ in range(m["steps"])]
        _compare(np.array(dts), fx["dts"], m["scheme"], "time steps")
        _compare(s.get_state(), fx["state"], m["scheme"], "state after steps")
        assert s.info().steps == m["steps"]


@pytest.mark.parametrize("path", fixture_paths("run_"), ids=fixture_id)
def test_graph_loop_matches_reference(path):
    """The device-resident loop (CUDA-graph chunks, dt never leaves the GPU)."""
    fx = load_fixture(path)
    m = fx["meta"]
    with wenofd.Solver(_config(m)) as s:
        s.set_state(fx["init"])
        n = s.advance(max_steps=m["steps"] if m["t_end"] is None else -1)
        assert n == m["steps"]
        _compare(s.get_state(), fx["state"], m["scheme"], "state after advance")
        if m["t_end"] is not None:
            assert s.info().now == pytest.approx(m["t_end"], abs=1e-9)


@pytest.mark.parametrize("tc,nx,ny", [(orc.SMOOTH, 30, 26), (orc.RIEMANN1, 20, 24), (orc.RIEMANN2, 33, 17),
                                      (orc.RTI, 12, 40), (orc.RIEMANN_SEEDED, 21, 29), (orc.SHEAR, 32, 32)])
def test_initialize_matches_oracle(tc, nx, ny):
    """initializeAve on the host of the library == the oracle's restatement."""
    p = orc.Problem(tc, nx, ny, seed=17)
    with wenofd.Solver({"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": 2, "CFL": 0.5,
                        "SCHEME": 1, "SEED": 17}) as s:
        s.initialize()
        assert_same(s.get_state(), p.interior(), "initial state")


@pytest.mark.parametrize("tc,scheme,rk", [(orc.RTI, orc.WENOZ, 2), (orc.RIEMANN1, orc.WENOJS, 1),
                                          (orc.SHEAR, orc.WENOZ, 0)])
def test_odd_sizes_match_oracle(tc, scheme, rk):
    """Tiles that do not divide the grid, both odd extents, every BC kind."""
    nx, ny = 47, 37
    p = orc.Problem(tc, nx, ny, scheme, rk, 0.6, seed=3)
    with wenofd.Solver({"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": rk, "CFL": 0.6,
                        "SCHEME": scheme, "SEED": 3}) as s:
        s.set_state(p.interior())
        p.run(max_steps=6)
        assert s.advance(max_steps=6) == 6
        assert_same(s.get_state(), p.interior(), "state")


def test_nan_state_reports_nan_dt():
    p = orc.Problem(orc.RIEMANN2, 16, 16)
    U = p.interior()
    U[0, 5, 5] = np.nan
    with wenofd.Solver({"TESTCASE": 2, "ELEMNUMX": 16, "ELEMNUMY": 16, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1}) as s:
        s.set_state(U)
        with pytest.raises(wenofd.WenofdError) as e:
            s.calc_dt()
        assert e.value.status == wenofd.NAN_DT
        with pytest.raises(wenofd.WenofdError) as e:
            s.advance(max_steps=3)
        assert e.value.status == wenofd.NAN_DT


def test_short_advance_runs_only_its_steps():
    """A capped advance shorter than a graph chunk replays one-step graphs, so
    it launches the kernels of its own steps and no gated-off chunk tail."""
    with wenofd.Solver({"TESTCASE": 4, "ELEMNUMX": 48, "ELEMNUMY": 40, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1,
                        "SEED": 2}) as s:
        s.initialize()
        assert s.advance(max_steps=1) == 1
        per_step = 10  # gate, time step, finalize, 3 x (ghost fill, stage), time update
        assert s.info().graph_steps == 64
        l0 = s.info().launches
        assert s.advance(max_steps=5) == 5
        assert s.info().launches - l0 == 1 + 5 * per_step
        l0 = s.info().launches
        assert s.advance(max_steps=70) == 70
        assert s.info().launches - l0 == 1 + 70 * per_step
        assert s.info().steps == 76
