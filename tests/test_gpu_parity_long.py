"""Parity over whole runs, against the reference's own outputs.

The fixtures come from the unmodified reference (tests/golden/make_golden_long.py):

* the -ffp-contract=off build (one IEEE rounding per operation), which the
  FP64 CUDA path must equal bit for bit after every step: the seeded
  four-quadrant Riemann problem at 800^2 run to t = 0.3 (the whole run of the
  drop-in configuration) and at 4096^2 for 20 steps, compared by the SHA-256
  of the final state, and the reference's Riemann2 case at 80^2 run to its end
  time 0.8 (382 steps), compared value by value;
* the build with the reference's own flags (makefile:5, -O3 -march=native;
  GCC contracts multiply-adds into FMAs there), which no other build can match
  bit for bit: the FP64 CUDA path is held to 1e-12 relative L-infinity against
  it (per conserved component, max |a - b| / max |b|) on the smooth wave at
  100^2 to t = 1 (3,610 steps) and on the Riemann2 run above.  The observed
  values are printed (pytest -s).
"""
import hashlib
import os

import numpy as np
import pytest

import wenofd
from conftest import GOLDEN, assert_same, load_fixture

pytestmark = pytest.mark.gpu

REL_LINF_NATIVE = 1e-12  # against the reference built with its own flags


def _fixture(name):
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.fail(f"missing fixture {name}.npz (tests/golden/make_golden_long.py)")
    return load_fixture(path)


def _sha256(state):
    return hashlib.sha256(np.ascontiguousarray(state, dtype="<f8").tobytes()).hexdigest()


def _rel_linf(a, b):
    """max over components of max|a - b| / max|b|."""
    return max(float(np.max(np.abs(a[r] - b[r])) / np.max(np.abs(b[r]))) for r in range(4))


def _solver(m, **extra):
    cfg = {"TESTCASE": m["testcase"], "ELEMNUMX": m["nx"], "ELEMNUMY": m["ny"], "RKMETH": m["rk"],
           "CFL": m["cfl"], "SCHEME": m["scheme"], "SEED": m["seed"]}
    if m.get("t_end") is not None:
        cfg["TEND"] = m["t_end"]
    cfg.update(extra)
    return wenofd.Solver(cfg)


@pytest.mark.parametrize("name", ["long_riemannseeded_z_rk3_800_t03", "long_riemannseeded_z_rk3_4096_20steps"])
def test_seeded_riemann_run_is_bitwise_the_reference(name):
    fx = _fixture(name)
    m = fx["meta"]
    with _solver(m) as s:
        s.initialize()
        n = s.advance(max_steps=-1 if m["t_end"] is not None else m["steps"])
        info = s.info()
        gpu = s.get_state()
    assert n == m["steps"]
    assert info.now == m["now"]  # the sum of every step's dt, bit for bit
    sub = m["subsample"]
    assert_same(gpu[0, ::sub, ::sub], fx["rho_sub"], "density subsample")
    assert _sha256(gpu) == m["state_sha256"], "final state differs from the reference's"


def test_riemann2_run_against_both_reference_builds():
    fx = _fixture("native_riemann2_z_rk3_80_t08")
    m = fx["meta"]
    with _solver(m) as s:
        s.initialize()
        n = s.advance(max_steps=-1)
        gpu = s.get_state()
    assert n == m["steps"] == m["steps_exact"]
    assert_same(gpu, fx["state_exact"], "state after the whole run vs the -ffp-contract=off build")
    rel = _rel_linf(gpu, fx["state"])
    print(f"\nRiemann2 80^2, {n} steps to t = 0.8: relative Linf vs the reference's own build {rel:.3e}")
    assert rel <= REL_LINF_NATIVE


def test_smooth_wave_to_t1_against_the_native_reference():
    fx = _fixture("native_smooth_z_rk3_100_t1")
    m = fx["meta"]
    with _solver(m) as s:
        s.initialize()
        n = s.advance(max_steps=-1)
        gpu = s.get_state()
        linf, l1, _ = s.error_norms()
    assert n == m["steps"]
    rel = _rel_linf(gpu, fx["state"])
    print(f"\nsmooth wave 100^2, {n} steps to t = 1: relative Linf vs the reference's own build {rel:.3e}; "
          f"L1 {l1:.10e} (reference {m['l1']:.10e})")
    assert rel <= REL_LINF_NATIVE
    assert l1 == pytest.approx(m["l1"], rel=1e-6) and linf == pytest.approx(m["linf"], rel=1e-6)
