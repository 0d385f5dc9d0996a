"""The FP32 precision form: flux and reconstruction arithmetic in FP32, state,
RK sums and the time step in FP64.  Its results are compared with the FP64
path (bitwise the reference) on the same inputs; the bounds below are the
accepted error of the form and are written into the test."""
import numpy as np
import pytest

import oracle as orc
import wenofd
from conftest import fixture_id, fixture_paths, load_fixture

pytestmark = pytest.mark.gpu

RHS_REL_TOL = 2e-4      # max |rhs32 - rhs64| / max |rhs64|
STATE_REL_TOL = 1e-5    # max |U32 - U64| / max |U64| after the fixture's steps


def _config(meta, precision):
    cfg = {"TESTCASE": meta["testcase"], "ELEMNUMX": meta["nx"], "ELEMNUMY": meta["ny"],
           "RKMETH": meta["rk"], "CFL": meta["cfl"], "SCHEME": meta["scheme"], "SEED": meta["seed"],
           "PRECISION": precision}
    if meta.get("t_end") is not None:
        cfg["TEND"] = meta["t_end"]
    return cfg


@pytest.mark.parametrize("path", fixture_paths("rhs_"), ids=fixture_id)
def test_fp32_rhs_close_to_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    with wenofd.Solver(_config(m, wenofd.FP32)) as s:
        s.set_state(fx["init"])
        rhs = s.get_flux()
    assert np.all(np.isfinite(rhs))
    err = np.max(np.abs(rhs - fx["rhs"])) / np.max(np.abs(fx["rhs"]))
    assert err <= RHS_REL_TOL, err


@pytest.mark.parametrize("path", fixture_paths("run_"), ids=fixture_id)
def test_fp32_steps_close_to_reference(path):
    fx = load_fixture(path)
    m = fx["meta"]
    with wenofd.Solver(_config(m, wenofd.FP32)) as s:
        s.set_state(fx["init"])
        n = s.advance(max_steps=m["steps"] if m["t_end"] is None else -1)
        U = s.get_state()
    assert n == m["steps"]
    assert np.all(np.isfinite(U))
    err = np.max(np.abs(U - fx["state"])) / np.max(np.abs(fx["state"]))
    assert err <= STATE_REL_TOL, err


@pytest.mark.parametrize("scheme", [orc.WENOJS, orc.WENOZ, orc.WENOZP, orc.WENOZPI])
def test_fp32_shear_layer_stays_finite_and_close(scheme):
    """The shear layer has flat stencils next to jumps (beta = 0 beside a
    large tau), the case that overflows unguarded FP32 weights."""
    n, steps = 256, 40
    p = orc.Problem(orc.SHEAR, n, n, scheme, 2, 0.7, seed=5)
    init = p.interior()
    out = {}
    for prec in (wenofd.FP64, wenofd.FP32):
        with wenofd.Solver({"TESTCASE": 5, "ELEMNUMX": n, "ELEMNUMY": n, "RKMETH": 2, "CFL": 0.7,
                            "SCHEME": scheme, "SEED": 5, "PRECISION": prec}) as s:
            s.set_state(init)
            assert s.advance(max_steps=steps) == steps
            out[prec] = s.get_state()
    assert np.all(np.isfinite(out[wenofd.FP32]))
    rho32, rho64 = out[wenofd.FP32][0], out[wenofd.FP64][0]
    assert np.mean(np.abs(rho32 - rho64)) <= 1e-5
    assert np.max(np.abs(rho32 - rho64)) <= 1e-3


@pytest.mark.parametrize("tc,n,steps", [(orc.RIEMANN_SEEDED, 300, 0), (orc.RIEMANN_SEEDED, 300, 15),
                                        (orc.SHEAR, 256, 5), (orc.SMOOTH, 120, 3), (orc.RTI, 64, 5),
                                        (orc.RIEMANN1, 200, 10)])
def test_two_pass_time_step_equals_fp64_reduction(tc, n, steps):
    """The FP32 forms reduce the time step in two passes (FP32 screen with an
    error bound, FP64 only where a node can hold the maximum); the result
    must equal the FP64 form's single FP64 pass bit for bit.  Constant
    quadrants (step 0) make whole regions tie for the maximum."""
    p = orc.Problem(tc, n, n, orc.WENOZ, 2, 0.7, seed=19)
    p.run(max_steps=steps)
    U = p.interior()
    dts = []
    for prec in (wenofd.FP64, wenofd.FP32, wenofd.LEARNED):
        with wenofd.Solver({"TESTCASE": tc, "ELEMNUMX": n, "ELEMNUMY": n, "RKMETH": 2, "CFL": 0.7,
                            "SCHEME": 1, "SEED": 19, "PRECISION": prec}) as s:
            s.set_state(U)
            dts.append(s.calc_dt())
    assert dts[0] == dts[1] == dts[2] == p.calc_dt()


@pytest.mark.parametrize("precision", [wenofd.FP32, wenofd.LEARNED])
@pytest.mark.parametrize("tile_i", [0, 31])
def test_fused_screen_steps_equal_separate_steps(precision, tile_i):
    """Inside wenofd_advance the last RK stage of a step also screens the
    next time step per stage tile, and the reduction then refines only the
    tiles that can hold the maximum.  The steps must equal, bit for bit,
    steps driven one call at a time (calc_dt: full screen + refine; rk_step)."""
    import mlp_oracle

    n, steps = 200, 8
    cfg = {"TESTCASE": 5, "ELEMNUMX": n, "ELEMNUMY": n + 17, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1, "SEED": 5,
           "PRECISION": precision, "TILE_I": tile_i}
    params = mlp_oracle.init_params(3)

    def make():
        s = wenofd.Solver(cfg)
        s.initialize()
        if precision == wenofd.LEARNED:
            s.set_indicator(params, 0.5)
        return s

    with make() as a:
        assert a.advance(max_steps=steps) == steps
        Ua, ta = a.get_state(), a.info().now
    with make() as b:
        now = 0.0
        for _ in range(steps):
            dt = b.calc_dt()
            b.rk_step(dt)
            now += dt
            b.set_time(now)
        Ub = b.get_state()
    assert ta == now
    assert np.array_equal(Ua, Ub)


@pytest.mark.parametrize("nx,ny", [(6, 6), (7, 9), (16, 31), (33, 65), (100, 7)])
@pytest.mark.parametrize("tile_i", [15, 31])
def test_tma_tiles_on_small_and_ragged_grids(nx, ny, tile_i):
    """The per-solve FP32 tiles take their halo and flags by TMA in boxes of
    40 x (TI + 6) nodes and 48 x (TI + 4) flag bytes: on grids smaller than a
    box or not a multiple of the tile the boxes run past the arrays (zero
    fill) and past the tiles' last nodes.  The batched kernel runs the same
    tile arithmetic with per-thread 128-bit loads instead, so the two must
    agree (to the last bit here), on every boundary kind.  On the smallest
    Riemann grids a shock crosses most nodes and FP32 rounding grows: the FP32
    form sits up to ~3e-4 from FP64 there, and the learned form with every
    node flagged (the WENO list for every face, whose four lanes group the
    arithmetic differently) up to ~2e-4 from the FP32 form; both are held to
    1e-3."""
    for tc in (orc.RIEMANN_SEEDED, orc.RIEMANN1, orc.SMOOTH):
        cfg = {"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "SEED": 4}

        def run(precision, params=None, batched=False):
            with wenofd.Solver(dict(cfg, PRECISION=precision, TILE_I=tile_i)) as s:
                s.initialize()
                if params is not None:
                    s.set_indicator(params, 0.5)
                if batched:
                    with wenofd.Batch([s]) as b:
                        b.configure(tile_i=tile_i)
                        assert b.advance(5) == 5
                else:
                    assert s.advance(max_steps=5) == 5
                return s.get_state()

        U64 = run(wenofd.FP64) if tile_i == 15 else None
        U32 = run(wenofd.FP32)
        scale = np.max(np.abs(U32))
        assert np.all(np.isfinite(U32))
        assert np.max(np.abs(U32 - run(wenofd.FP32, batched=True))) <= 1e-12 * scale, (tc, nx, ny)
        every = np.zeros(wenofd.MLP_PARAMS, dtype=np.float32)
        every[2720] = 50.0
        Ul = run(wenofd.LEARNED, every)
        if U64 is not None:
            assert np.max(np.abs(U32 - U64)) <= 1e-3 * scale, (tc, nx, ny)
        assert np.max(np.abs(Ul - U32)) <= 1e-3 * scale, (tc, nx, ny)
