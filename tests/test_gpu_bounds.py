"""The bounds-checked debug library (build.py --bounds-check,
-DWENOFD_BOUNDS_CHECK): every kernel's index guards on, the device-side
counterpart of the reference's assert-checked Array1D/Array2D indexing
(utils/array.h:273-303, 552-583).

A child process loads the checked library (WENOFD_LIBRARY) and runs every
kernel family on tiny, odd, non-square grids -- the stage tiles of both
heights and all forms (FP64, FP32 with TMA halo boxes, learned with the
tensor-core indicator), the boundary fill of every boundary type, the
time-step reductions, the output and norm kernels, the batched kernel with
RK1/RK2/RK3, the time step without allocation, the sampler and the training
kernels.  Its guard record must stay empty, and its results must equal the
release library's on the same inputs: bit for bit where the release path is
bitwise by construction (FP64 solves and batches, every time step, the
sampler, which runs in a unit without multiply-add contraction), and within
the bounds below for FP32 arithmetic, which the guards' extra branches may
compile with a different set of FP32 multiply-adds.

The guard mechanism itself is checked by wenofd_bounds_selftest: one guarded
access one past the end of a 4-element array, which the guard sends to
element 0 (so nothing out of bounds is touched) and records."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fd-weno-eulerequation_gb300")

FP32_REL_TOL = 1e-5   # max |x_checked - x_release| / max |x_release|: FP32-form states and outputs
RHS_REL_TOL = 2e-4    # the same for an FP32-form RHS (the FP32 form's own bound against FP64)
TRAIN_REL_TOL = 1e-3  # the same for parameters after two epochs of training
FLAG_FRACTION = 0.01  # indicator / routing flags that may differ, learned form

# (testcase, nx, ny, seed, scheme, rk, precision, tile_i): odd and non-square
# grids, one or several tiles in each direction, every boundary type (SMOOTH
# and SHEAR periodic, RIEMANN1/2 SPECIAL, RIEMANN_SEEDED symmetric, RTI slip +
# SPECIAL + gravity), every scheme, RK1/2/3, both tile heights of each form
CASES = [
    (4, 16, 12, 3, 1, 2, 0, 15),
    (0, 13, 7, 0, 0, 1, 0, 7),
    (3, 37, 29, 0, 2, 2, 0, 15),
    (1, 70, 45, 0, 3, 0, 0, 7),
    (5, 16, 12, 5, 1, 2, 1, 15),
    (2, 13, 7, 0, 0, 1, 1, 31),
    (3, 37, 29, 0, 3, 2, 1, 31),
    (4, 70, 45, 9, 2, 0, 1, 15),
    (5, 16, 12, 5, 1, 2, 2, 15),
    (1, 37, 29, 0, 1, 1, 2, 31),
    (4, 70, 45, 9, 1, 2, 2, 15),
    (3, 33, 66, 0, 1, 2, 2, 31),
]
STEPS = 6


def _cfg(tc, nx, ny, seed, scheme, rk, prec, tile_i):
    return {"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": rk, "CFL": 0.6, "SCHEME": scheme,
            "SEED": seed, "PRECISION": prec, "TILE_I": tile_i, "INDICATOR_INTERVAL": 2}


def run_all(out_path):
    """Every kernel family once on the CASES; results saved to out_path."""
    import torch

    import wenofd

    out = {}
    params = wenofd.mlp_init(11)
    for k, c in enumerate(CASES):
        cfg = _cfg(*c)
        with wenofd.Solver(cfg) as s:
            s.initialize()
            if c[6] == wenofd.LEARNED:
                s.set_indicator(params, 0.5)
            out[f"c{k}_rhs"] = s.get_flux()
            out[f"c{k}_dt"] = np.array([s.calc_dt()])
            s.set_time(0.0)
            out[f"c{k}_n"] = np.array([s.advance(max_steps=STEPS)])
            out[f"c{k}_U"] = s.get_state()
            out[f"c{k}_G"] = s.get_state_ghosted()
            out[f"c{k}_out"] = s.output_variables()
            out[f"c{k}_sums"] = s.conservation_sums()
            if c[0] == 0:
                out[f"c{k}_norms"] = s.error_norms()
            if c[6] == wenofd.LEARNED:
                out[f"c{k}_flags"] = s.indicator_flags()
                out[f"c{k}_routing"] = s.routing_flags()
    # batches: FP64 with RK1, SSP-RK2, SSP-RK3; one FP32 batch; learned
    # batches (the batched indicator and the routed batched kernel) with
    # both tile heights
    members = [(4, 16, 12, 3), (3, 37, 29, 0), (1, 70, 45, 0), (0, 13, 7, 0)]
    for rk, prec, tile in ((0, 0, 0), (1, 0, 0), (2, 0, 0), (2, 1, 0), (2, 2, 15), (1, 2, 31)):
        solvers = [wenofd.Solver(_cfg(tc, nx, ny, sd, 1, rk, prec, 0)) for tc, nx, ny, sd in members]
        try:
            for s in solvers:
                s.initialize()
                if prec == wenofd.LEARNED:
                    s.set_indicator(params, 0.5)
            with wenofd.Batch(solvers) as b:
                if tile:
                    b.configure(tile_i=tile)
                b.advance(STEPS)
            for m, s in enumerate(solvers):
                out[f"b{rk}{prec}_{m}"] = s.get_state()
                if prec == wenofd.LEARNED:
                    out[f"bflags{rk}{prec}_{m}"] = s.routing_flags()
        finally:
            for s in solvers:
                s.close()
    # the time step without allocation, on a dense device state
    with wenofd.Solver(_cfg(4, 37, 29, 3, 1, 2, 0, 0)) as s:
        s.initialize()
        U = torch.from_numpy(s.get_state()).cuda()
    dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = wenofd.lib().wenofd_calc_dt_noalloc(U.data_ptr(), 37, 29, 1.0 / 36, 1.0 / 28, 1.4, 0.6, 0.0, 1.0,
                                             dt.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    out["noalloc_dt"] = dt.cpu().numpy()
    # sampler (on an initial state, so both libraries sample the same
    # nodes) and training kernels
    cap = 4000
    X = torch.zeros((cap, wenofd.MLP_INPUTS), dtype=torch.float32, device="cuda")
    y = torch.zeros(cap, dtype=torch.float32, device="cuda")
    with wenofd.Solver(_cfg(4, 70, 45, 9, 1, 2, 1, 15)) as s:
        s.initialize()
        rows = s.indicator_sample(600, 5, X.data_ptr(), y.data_ptr(), cap)
    out["sample_X"] = X[:rows].cpu().numpy()
    out["sample_y"] = y[:rows].cpu().numpy()
    P = torch.from_numpy(params.copy()).cuda()
    out["train_loss"] = wenofd.mlp_train(P.data_ptr(), X.data_ptr(), y.data_ptr(), rows, 2, 256, 3e-3, 7)
    torch.cuda.synchronize()
    out["train_P"] = P.cpu().numpy()
    rep = wenofd.bounds_report(reset=False)
    out["guard"] = np.array([rep["count"], rep["line"], rep["index"], rep["extent"]])
    out["guard_where"] = np.array(rep["where"])
    st = wenofd.bounds_selftest()
    out["selftest"] = np.array([st["count"], st["line"], st["index"], st["extent"]])
    out["selftest_where"] = np.array(st["where"])
    np.savez(out_path, **out)


def _bound(k):
    """How a result compares between the two libraries: None = bit for bit,
    else (kind, bound)."""
    if k.startswith("c"):  # single solve c<case>_<what>
        case, what = k[1:].split("_", 1)
        if CASES[int(case)][6] == 0 or what in ("dt", "n"):
            return None
        if what in ("flags", "routing"):
            return ("fraction", FLAG_FRACTION)
        return ("rel", RHS_REL_TOL if what == "rhs" else FP32_REL_TOL)
    if k.startswith("bflags"):  # learned batch member's routing flags
        return ("fraction", FLAG_FRACTION)
    if k.startswith("b"):  # batch b<rk><precision>_<member>
        return None if k[2] == "0" else ("rel", FP32_REL_TOL)
    if k.startswith("train"):
        return ("rel", TRAIN_REL_TOL)
    return None


@pytest.mark.gpu
def test_bounds_selftest_release():
    sys.path.insert(0, os.path.join(PKG, "python"))
    import wenofd

    st = wenofd.bounds_selftest()
    assert (st["count"], st["index"], st["extent"]) == (1, 4, 4), st
    assert st["where"].startswith("aux_kernels.cu:"), st
    assert wenofd.bounds_report()["count"] == -1  # the release library has no guards


@pytest.mark.gpu
def test_bounds_checked_library_matches_release(tmp_path):
    sys.path.insert(0, PKG)
    import build

    lib = build.build_checked()
    env = dict(os.environ, WENOFD_LIBRARY=lib)
    checked = str(tmp_path / "checked.npz")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), checked], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    env.pop("WENOFD_LIBRARY")
    release = str(tmp_path / "release.npz")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), release], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    a, b = np.load(checked), np.load(release)
    # the checked library's guards saw no index out of range ...
    assert a["guard"][0] == 0, f"{a['guard']} at {a['guard_where']}"
    # ... and they work: the self-test's one violation is recorded
    assert tuple(a["selftest"][[0, 2, 3]]) == (1, 4, 4)
    assert str(a["selftest_where"]).startswith("aux_kernels.cu:")
    assert b["guard"][0] == -1
    for k in b.files:
        if k.startswith(("guard", "selftest")):
            continue
        x, y = a[k], b[k]
        assert x.shape == y.shape, k
        bound = _bound(k)
        if bound is None:
            same = (x == y) | (np.isnan(x) & np.isnan(y)) if x.dtype.kind == "f" else (x == y)
            assert same.all(), f"{k}: {np.count_nonzero(~same)} values differ"
        elif bound[0] == "fraction":
            assert np.count_nonzero(x != y) <= bound[1] * x.size, k
        else:
            err = np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300)
            assert err <= bound[1], (k, err)


if __name__ == "__main__":
    sys.path.insert(0, os.path.join(PKG, "python"))
    run_all(sys.argv[1])
