"""Batches: independent solves of different sizes, cases and boundary
conditions advanced by one persistent kernel (wenofd_batch_*).

A member's steps are those of wenofd_advance on its own handle: FP64 members
bit for bit (and so the oracle's).  FP32 members run the same FP32 stage
code compiled into another kernel, where the compiler may contract a
different set of FP32 multiply-adds, so they are held to the FP32 form's own
accepted error against the FP64 solve (the bound of the FP32 form's tests).
Learned-form members (the batched tensor-core indicator between batched
launches) route with the single solve's flags and are held to the same bound
against their single solves."""
import numpy as np
import pytest

import mlp_oracle
import oracle as orc
import wenofd

pytestmark = pytest.mark.gpu

FP32_REL_TOL = 1e-5  # max |U32 - U64| / max |U64| after the steps below

# (testcase, nx, ny, seed, extra keys): uneven sizes, periodic / slip /
# SPECIAL / symmetric boundaries, gravity (RTI)
MEMBERS = [
    (orc.RIEMANN_SEEDED, 48, 40, 3, {}),
    (orc.SMOOTH, 64, 64, 0, {}),
    (orc.SHEAR, 100, 37, 5, {}),
    (orc.RIEMANN1, 33, 90, 0, {}),
    (orc.RTI, 24, 96, 0, {}),
    (orc.RIEMANN2, 130, 70, 0, {}),
]


def _cfg(tc, nx, ny, seed, extra, precision, scheme=orc.WENOZ, tend=None):
    c = {"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": 2, "CFL": 0.6, "SCHEME": scheme,
         "SEED": seed, "PRECISION": precision}
    c.update(extra)
    if tend is not None:
        c["TEND"] = tend
    return c


def _alone(cfgs, max_steps):
    out = []
    for c in cfgs:
        with wenofd.Solver(c) as s:
            s.initialize()
            n = s.advance(max_steps=max_steps)
            out.append((s.get_state(), s.info().now, n))
    return out


def _batched(cfgs, max_steps, configure=None, autotune=0):
    solvers = [wenofd.Solver(c) for c in cfgs]
    try:
        for s in solvers:
            s.initialize()
        with wenofd.Batch(solvers) as b:
            if configure:
                b.configure(**configure)
            if autotune:
                b.autotune(autotune)
            n = b.advance(max_steps)
            info = b.info()
        return [(s.get_state(), s.info().now, s.info().steps) for s in solvers], n, info
    finally:
        for s in solvers:
            s.close()


@pytest.mark.parametrize("configure", [None, {"tile_i": 7}, {"steps_per_launch": 5}, {"blocks_per_sm": 1}],
                         ids=["default", "tile7", "launch5", "bps1"])
def test_fp64_batch_bitwise_equals_single_solves(configure):
    cfgs = [_cfg(*m, wenofd.FP64) for m in MEMBERS]
    steps = 12
    ref = _alone(cfgs, steps)
    got, n, info = _batched(cfgs, steps, configure)
    assert n == steps
    assert info.members == len(cfgs) and info.cells == sum(m[1] * m[2] for m in MEMBERS)
    for (U, now, k), (Ur, nowr, kr) in zip(got, ref):
        assert k == kr == steps
        assert now == nowr
        assert np.array_equal(U, Ur)


def test_fp64_batch_member_matches_oracle():
    tc, nx, ny, seed, extra = MEMBERS[0]
    p = orc.Problem(tc, nx, ny, orc.WENOZ, 2, 0.6, seed=seed)
    p.run(max_steps=8)
    got, n, _ = _batched([_cfg(*MEMBERS[0], wenofd.FP64), _cfg(*MEMBERS[2], wenofd.FP64)], 8)
    assert n == 8
    assert np.array_equal(got[0][0], p.interior())
    assert got[0][1] == p.now


@pytest.mark.parametrize("rk", [0, 1], ids=["rk1", "ssprk2"])
@pytest.mark.parametrize("configure", [None, {"steps_per_launch": 3}], ids=["default", "launch3"])
def test_rk1_rk2_batches(rk, configure):
    """RKMETH 0 (RK1: one stage, then U^{n+1} = the stage's output) and 1
    (SSP-RK2) batches: FP64 members bit for bit the single solves (and the
    oracle), FP32 members within the FP32 form's bound of their FP64 solve."""
    cfgs = [dict(_cfg(*m, wenofd.FP64), RKMETH=rk) for m in MEMBERS]
    steps = 9
    ref = _alone(cfgs, steps)
    got, n, _ = _batched(cfgs, steps, configure)
    assert n == steps
    for (U, now, k), (Ur, nowr, kr) in zip(got, ref):
        assert k == kr == steps and now == nowr
        assert np.array_equal(U, Ur)
    tc, nx, ny, seed, extra = MEMBERS[0]
    p = orc.Problem(tc, nx, ny, orc.WENOZ, rk, 0.6, seed=seed)
    p.run(max_steps=steps)
    assert np.array_equal(got[0][0], p.interior())
    got32, _, _ = _batched([dict(c, PRECISION=wenofd.FP32) for c in cfgs], steps, configure)
    for (U32, _, k), (U64, _, _) in zip(got32, ref):
        assert k == steps
        assert np.max(np.abs(U32 - U64)) <= FP32_REL_TOL * np.max(np.abs(U64))


@pytest.mark.parametrize("scheme", [orc.WENOJS, orc.WENOZP, orc.WENOZPI])
def test_fp64_batch_other_schemes(scheme):
    cfgs = [_cfg(*m, wenofd.FP64, scheme=scheme) for m in MEMBERS[:4]]
    ref = _alone(cfgs, 6)
    got, n, _ = _batched(cfgs, 6)
    assert n == 6
    for (U, now, _), (Ur, nowr, _) in zip(got, ref):
        assert now == nowr and np.array_equal(U, Ur)


@pytest.mark.parametrize("configure", [None, {"tile_i": 31}], ids=["default", "tile31"])
def test_fp32_batch_close_to_single_solves(configure):
    steps = 12
    ref64 = _alone([_cfg(*m, wenofd.FP64) for m in MEMBERS], steps)
    cfgs = [_cfg(*m, wenofd.FP32) for m in MEMBERS]
    alone32 = _alone(cfgs, steps)
    got, n, _ = _batched(cfgs, steps, configure)
    assert n == steps
    for (U, now, k), (U1, now1, k1), (Ur, nowr, _) in zip(got, alone32, ref64):
        assert k == k1 == steps
        assert np.all(np.isfinite(U))
        scale = np.max(np.abs(Ur))
        assert np.max(np.abs(U - Ur)) / scale <= FP32_REL_TOL
        assert np.max(np.abs(U1 - Ur)) / scale <= FP32_REL_TOL
        assert abs(now - nowr) <= FP32_REL_TOL * nowr


def test_members_stop_at_their_own_end_time():
    """advance(-1): every member runs to its own TEND, as wenofd_advance does."""
    tends = [0.004, 0.011, 0.002]
    cfgs = [_cfg(*m, wenofd.FP64, tend=t) for m, t in zip(MEMBERS[:3], tends)]
    ref = _alone(cfgs, -1)
    got, n, _ = _batched(cfgs, -1)
    assert n == max(r[2] for r in ref)
    for (U, now, k), (Ur, nowr, kr), t in zip(got, ref, tends):
        assert k == kr and now == nowr and abs(now - t) <= 1e-9
        assert np.array_equal(U, Ur)


@pytest.mark.parametrize("precision", [wenofd.FP32, wenofd.LEARNED])
def test_fp32_members_stop_at_their_own_end_time(precision):
    """FP32 and learned members with different TEND: a member that has
    finished no longer holds the others to the full time-step passes (the
    reduction refines candidate tiles once every member that can step has
    screened bounds), and every member ends at its own TEND with its single
    solve's step count."""
    tends = [0.004, 0.011, 0.002]
    members = LEARNED_MEMBERS[:3] if precision == wenofd.LEARNED else MEMBERS[:3]
    cfgs = [dict(_cfg(*m, precision, tend=t), INDICATOR_INTERVAL=2) for m, t in zip(members, tends)]
    P = mlp_oracle.init_params(LEARNED_PARAMS_SEED)

    def run(batched):
        solvers = [wenofd.Solver(c) for c in cfgs]
        try:
            for s in solvers:
                s.initialize()
                if precision == wenofd.LEARNED:
                    s.set_indicator(P, 0.5)
            if batched:
                with wenofd.Batch(solvers) as b:
                    b.configure(steps_per_launch=3)
                    b.advance(-1)
            else:
                for s in solvers:
                    s.advance(max_steps=-1)
            return [(s.get_state(), s.info().now, s.info().steps) for s in solvers]
        finally:
            for s in solvers:
                s.close()

    ref, got = run(False), run(True)
    for (U, now, k), (Ur, nowr, kr), t in zip(got, ref, tends):
        assert k == kr and abs(now - t) <= 1e-9
        assert np.max(np.abs(U - Ur)) <= FP32_REL_TOL * np.max(np.abs(Ur))


@pytest.mark.parametrize("precision", [wenofd.FP64, wenofd.FP32])
def test_autotune_restores_state_and_keeps_results(precision):
    cfgs = [_cfg(*m, precision) for m in MEMBERS]
    ref, _, _ = _batched(cfgs, 5)
    solvers = [wenofd.Solver(c) for c in cfgs]
    try:
        for s in solvers:
            s.initialize()
        before = [s.get_state() for s in solvers]
        with wenofd.Batch(solvers) as b:
            ms = b.autotune(3)
            info = b.info()
            assert ms > 0 and info.tuned_ms_per_step == ms
            assert info.tile_i in ((7, 15) if precision == wenofd.FP64 else (15, 31))
            for s, U0 in zip(solvers, before):
                assert s.info().steps == 0 and s.info().now == 0.0
                assert np.array_equal(s.get_state(), U0)
            assert b.advance(5) == 5
        for s, (Ur, nowr, _) in zip(solvers, ref):
            U = s.get_state()
            if precision == wenofd.FP64:
                assert s.info().now == nowr and np.array_equal(U, Ur)
            else:  # the tuned tile height may select the other FP32 kernel instance
                assert np.max(np.abs(U - Ur)) / np.max(np.abs(Ur)) <= FP32_REL_TOL
    finally:
        for s in solvers:
            s.close()


def test_nan_member_stops_and_others_finish():
    cfgs = [_cfg(*m, wenofd.FP64) for m in MEMBERS[:3]]
    ref = _alone(cfgs, 4)
    solvers = [wenofd.Solver(c) for c in cfgs]
    try:
        for s in solvers:
            s.initialize()
        U = solvers[1].get_state()
        U[0, 5, 7] = np.nan
        solvers[1].set_state(U)
        with wenofd.Batch(solvers) as b:
            with pytest.raises(wenofd.WenofdError) as ei:
                b.advance(4)
        assert ei.value.status == wenofd.NAN_DT and "member 1" in str(ei.value)
        assert solvers[1].info().steps == 0
        for k in (0, 2):
            assert solvers[k].info().steps == 4
            assert np.array_equal(solvers[k].get_state(), ref[k][0])
    finally:
        for s in solvers:
            s.close()


def test_batch_rejects_mixed_or_unsupported_members():
    a = wenofd.Solver(_cfg(*MEMBERS[0], wenofd.FP64))
    b = wenofd.Solver(_cfg(*MEMBERS[1], wenofd.FP64, scheme=orc.WENOJS))
    c = wenofd.Solver(_cfg(*MEMBERS[1], wenofd.FP32))
    d = wenofd.Solver(_cfg(*MEMBERS[1], wenofd.LEARNED))
    e = wenofd.Solver(dict(_cfg(*MEMBERS[1], wenofd.FP64), RKMETH=1))
    f = wenofd.Solver(dict(_cfg(*MEMBERS[0], wenofd.LEARNED), INDICATOR_INTERVAL=2))
    try:
        for bad in ([a, b], [a, c], [a, d], [d, f], [a, e], [a, a]):
            with pytest.raises(wenofd.WenofdError) as ei:
                wenofd.Batch(bad)
            assert ei.value.status == wenofd.BAD_ARG
        with wenofd.Batch([a]) as bt:
            for kw in ({"tile_i": 31}, {"tile_i": 9}, {"blocks_per_sm": -1}):
                with pytest.raises(wenofd.WenofdError) as ei:
                    bt.configure(**kw)
                assert ei.value.status == wenofd.BAD_ARG
    finally:
        for s in (a, b, c, d, e, f):
            s.close()


def test_barrier_give_up_reports_timeout_and_the_batch_recovers():
    """The grid barrier's bounded wait: a test instance of the batched kernel
    (short poll limit) in which block 0 withholds its arrival at the second
    barrier of the launch.  Every block's wait there gives up, later waits end
    quickly, the launch finishes and the host reports WENOFD_TIMEOUT; after the
    members are re-initialised the same batch advances bit for bit like the
    single solves."""
    import time

    cfgs = [_cfg(tc, nx, ny, seed, extra, wenofd.FP64) for tc, nx, ny, seed, extra in MEMBERS[:3]]
    want = _alone(cfgs, 4)
    solvers = [wenofd.Solver(c) for c in cfgs]
    try:
        for s in solvers:
            s.initialize()
        with wenofd.Batch(solvers) as b:
            b.configure(tile_i=15, blocks_per_sm=0, steps_per_launch=2)
            b.test_withhold(block=0, barrier=1)
            t0 = time.perf_counter()
            with pytest.raises(wenofd.WenofdError) as e:
                b.advance(4)
            assert e.value.status == wenofd.TIMEOUT
            assert "barrier" in str(e.value)
            assert time.perf_counter() - t0 < 30.0
            for s in solvers:
                s.initialize()
            assert b.advance(4) == 4
            for s, (U, now, _) in zip(solvers, want):
                assert np.array_equal(s.get_state(), U)
                assert s.info().now == now
    finally:
        for s in solvers:
            s.close()


def test_withhold_hook_rejects_other_batches():
    cfgs = [_cfg(orc.RIEMANN_SEEDED, 40, 40, 1, {}, wenofd.FP32)]
    with wenofd.Solver(cfgs[0]) as s:
        s.initialize()
        with wenofd.Batch([s]) as b:
            with pytest.raises(wenofd.WenofdError) as e:
                b.test_withhold(0, 1)
            assert e.value.status == wenofd.BAD_ARG


# Learned-form members: a seeded four-quadrant Riemann problem, Riemann1
# (SPECIAL boundaries), a shear layer, the Rayleigh-Taylor case (SLIP /
# SPECIAL boundaries, gravity) and the smooth wave, of uneven sizes; a seeded
# untrained network at threshold 0.5 flags 5-25 % of each member's nodes.
# (Its flags do not follow the shocks, so some problems leave the physical
# states within a few steps on linear faces: with it, the seeded Riemann
# problem 48x100 (seed 3) and Riemann2 130x70 reach a NaN time step within 7
# steps alone; these members run all their steps.)
LEARNED_MEMBERS = [
    (orc.RIEMANN_SEEDED, 80, 64, 6, {}),
    (orc.RIEMANN1, 33, 90, 0, {}),
    (orc.SHEAR, 100, 37, 5, {}),
    (orc.RTI, 24, 96, 0, {}),
    (orc.SMOOTH, 64, 48, 0, {}),
]
LEARNED_PARAMS_SEED = 7


def _learned_run(interval, steps, batched, rk=2, configure=None, autotune=0, weights=(True,) * 5, late=0,
                 guard=0.0, members=None):
    """States, times, step counts and routing flags of the learned members
    after `late` steps without indicator weights (every face WENO), then
    loading the weights of the members marked in `weights`, then `steps`
    steps: in one batch, or each member alone (wenofd_advance)."""
    P = mlp_oracle.init_params(LEARNED_PARAMS_SEED)
    cfgs = [dict(_cfg(*m, wenofd.LEARNED), RKMETH=rk, INDICATOR_INTERVAL=interval, INDICATOR_GUARD=guard)
            for m in (members or LEARNED_MEMBERS)]
    solvers = [wenofd.Solver(c) for c in cfgs]
    try:
        for s in solvers:
            s.initialize()
        if batched:
            with wenofd.Batch(solvers) as b:
                if configure:
                    b.configure(**configure)
                if late:
                    assert b.advance(late) == late
                for s, w in zip(solvers, weights):
                    if w:
                        s.set_indicator(P, 0.5)
                if autotune:
                    b.autotune(autotune)
                assert b.advance(steps) == steps
        else:
            for s, w in zip(solvers, weights):
                if late:
                    assert s.advance(max_steps=late) == late
                if w:
                    s.set_indicator(P, 0.5)
                assert s.advance(max_steps=steps) == steps
        return [(s.get_state(), s.info().now, s.info().steps, s.routing_flags()) for s in solvers]
    finally:
        for s in solvers:
            s.close()


def _assert_learned_close(got, ref, same_flags=True):
    for (U, now, k, fl), (Ur, nowr, kr, flr) in zip(got, ref):
        assert k == kr
        assert np.all(np.isfinite(U))
        assert np.max(np.abs(U - Ur)) <= FP32_REL_TOL * np.max(np.abs(Ur))
        assert abs(now - nowr) <= 1e-12 * nowr
        if same_flags:
            assert np.array_equal(fl, flr)
        else:  # the other tile height's kernel: FP32 rounding may flip a borderline flag
            assert np.count_nonzero(fl != flr) <= 1e-3 * fl.size


@pytest.mark.parametrize("interval", [1, 3])
@pytest.mark.parametrize("configure", [None, {"steps_per_launch": 5}, {"tile_i": 31}], ids=["default", "launch5", "tile31"])
def test_learned_batch_matches_single_solves(interval, configure):
    """The batched indicator runs on the first step of the advance call and
    then every INDICATOR_INTERVAL steps, as the single solve's does, and its
    flags route the batched stage tiles: every member's flags equal its
    single solve's, its state agrees to the FP32 form's bound."""
    steps = 7
    ref = _learned_run(interval, steps, False)
    got = _learned_run(interval, steps, True, configure=configure)
    assert any(0.0 < r[3].mean() < 1.0 for r in ref)
    _assert_learned_close(got, ref, same_flags=configure is None or "tile_i" not in configure)


def test_learned_batch_ssprk2_and_autotune():
    steps = 6
    ref = _learned_run(2, steps, False, rk=1)
    got = _learned_run(2, steps, True, rk=1, autotune=2)
    _assert_learned_close(got, ref, same_flags=False)


def test_learned_batch_without_weights_and_weights_loaded_later():
    """A member without indicator weights routes every face to WENO (its
    flags stay 1), as its single solve does; weights loaded between two
    batch advances reach the second one."""
    weights = (True, False, True, False, True)
    ref = _learned_run(2, 5, False, weights=weights, late=2)
    got = _learned_run(2, 5, True, weights=weights, late=2)
    _assert_learned_close(got, ref)
    for (_, _, _, fl), w in zip(got, weights):
        if not w:
            assert np.all(fl == 1)


def test_learned_batch_with_guard_matches_single_solves():
    """INDICATOR_GUARD reaches the batched indicator: guarded members,
    including the seeded Riemann problem that stops with NAN_DT unguarded
    (48x100, seed 3), run their steps with the single solves' flags."""
    members = LEARNED_MEMBERS[:3] + [(orc.RIEMANN_SEEDED, 48, 100, 3, {})]
    ref = _learned_run(2, 12, False, weights=(True,) * 4, guard=0.5, members=members)
    got = _learned_run(2, 12, True, weights=(True,) * 4, guard=0.5, members=members)
    _assert_learned_close(got, ref)
