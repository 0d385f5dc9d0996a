"""Long-run fixtures from the REFERENCE itself, for parity beyond a few steps.

Two builds of the unmodified reference sources (``make -C oracle ref
REF=<checkout>``), both driven by oracle/ref_driver.cpp:

* ``wenofd_ref``         -ffp-contract=off: one IEEE rounding per operation,
  the arithmetic the FP64 CUDA path reproduces bit for bit;
* ``wenofd_ref_native``  the reference's own flags (makefile:5, -O3
  -march=native -g): GCC contracts multiply-adds into FMAs wherever the
  target has them, so its results differ from the first build in the last
  bits, and a GPU path can only be held to a tolerance against it.

Fixtures written (tests/test_gpu_parity_long.py reads them):

    long_riemannseeded_z_rk3_800_t03.npz
        the seeded four-quadrant Riemann problem (seed 7) at 800^2, WENO-Z,
        SSP-RK3, CFL 0.7, run to t = 0.3 by the -ffp-contract=off build.
        The state is 20 MB, so the fixture holds its SHA-256 (float64
        little-endian, [4][800][800], ej fastest), every time step, and a
        subsample of the density for diagnosis.
    long_riemannseeded_z_rk3_4096_20steps.npz
        the same problem at 4096^2 for 20 steps (hash, time steps, subsample).
    native_smooth_z_rk3_100_t1.npz
        the smooth advected wave at 100^2, WENO-Z, SSP-RK3, CFL 0.05, to
        t = 1 (README.md:69's configuration), native build: the whole final
        state, the time steps and the density error norms.
    native_riemann2_z_rk3_80_t08.npz
        the reference's own Riemann2 case at 80^2, WENO-Z, SSP-RK3, CFL 0.7,
        run to its end time 0.8, native build: the whole final state and time
        steps, and the same run of the -ffp-contract=off build beside it.

Run where the reference checkout exists (the 4096^2 case takes several
minutes per step on one core; the whole script about an hour):
    make -C oracle ref REF=<checkout> && python tests/golden/make_golden_long.py
"""
from __future__ import annotations

import hashlib
import json
import os
import platform
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle as orc  # noqa: E402
from make_golden import run_ref  # noqa: E402

REF_BIN = orc.REF_BIN
REF_BIN_NATIVE = orc.REF_BIN + "_native"


def state_hash(state: np.ndarray) -> str:
    """SHA-256 of an interior state as float64 little-endian, C order."""
    return hashlib.sha256(np.ascontiguousarray(state, dtype="<f8").tobytes()).hexdigest()


def cpu_note() -> str:
    flags = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("flags") or line.startswith("Features"):
                    flags = " ".join(x for x in line.split(":", 1)[1].split() if x in ("fma", "avx2", "avx512f",
                                                                                       "asimd"))
                    break
    except OSError:
        pass
    return f"{platform.machine()} ({flags})"


def hashed_case(name: str, n: int, seed: int, steps: int, t_end: float | None, sub: int) -> None:
    t0 = time.time()
    with tempfile.TemporaryDirectory() as wd:
        res = run_ref(wd, "run", orc.RIEMANN_SEEDED, n, n, orc.WENOZ, 2, 0.7, seed, steps, t_end)
    st = res["state"]
    meta = dict(testcase=orc.RIEMANN_SEEDED, nx=n, ny=n, scheme=orc.WENOZ, rk=2, cfl=0.7, seed=seed,
                t_end=t_end, steps=int(res["steps"]), now=float(res["now"]), build="-ffp-contract=off",
                state_sha256=state_hash(st), subsample=sub, wall_s=round(time.time() - t0, 1))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), dts=res["dts"],
                        rho_sub=st[0, ::sub, ::sub], abs_sums=np.abs(st).sum(axis=(1, 2)))
    print(f"{name}: {meta['steps']} steps, t = {meta['now']}, {meta['wall_s']} s")


def native_smooth() -> None:
    name = "native_smooth_z_rk3_100_t1"
    t0 = time.time()
    with tempfile.TemporaryDirectory() as wd:
        res = run_ref(wd, "accuracy", orc.SMOOTH, 100, 100, orc.WENOZ, 2, 0.05, binary=REF_BIN_NATIVE)
    meta = dict(testcase=orc.SMOOTH, nx=100, ny=100, scheme=orc.WENOZ, rk=2, cfl=0.05, seed=0, t_end=None,
                steps=int(res["steps"]), now=float(res["now"]), build="-O3 -march=native -g (makefile:5)",
                host=cpu_note(), linf=res.get("linf"), l1=res.get("l1"), l2=res.get("l2"),
                wall_s=round(time.time() - t0, 1))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), state=res["state"],
                        dts=res["dts"])
    print(f"{name}: {meta['steps']} steps, L1 {meta['l1']}, {meta['wall_s']} s")


def native_riemann2() -> None:
    name = "native_riemann2_z_rk3_80_t08"
    t0 = time.time()
    with tempfile.TemporaryDirectory() as wd:
        nat = run_ref(wd, "run", orc.RIEMANN2, 80, 80, orc.WENOZ, 2, 0.7, binary=REF_BIN_NATIVE)
    with tempfile.TemporaryDirectory() as wd:
        exact = run_ref(wd, "run", orc.RIEMANN2, 80, 80, orc.WENOZ, 2, 0.7, binary=REF_BIN)
    meta = dict(testcase=orc.RIEMANN2, nx=80, ny=80, scheme=orc.WENOZ, rk=2, cfl=0.7, seed=0, t_end=None,
                steps=int(nat["steps"]), steps_exact=int(exact["steps"]), now=float(nat["now"]),
                build="-O3 -march=native -g (makefile:5); state_exact: -ffp-contract=off", host=cpu_note(),
                wall_s=round(time.time() - t0, 1))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=np.array(json.dumps(meta)), state=nat["state"],
                        dts=nat["dts"], state_exact=exact["state"], dts_exact=exact["dts"])
    print(f"{name}: {meta['steps']} steps (exact build {meta['steps_exact']}), {meta['wall_s']} s")


def main() -> None:
    for b in (REF_BIN, REF_BIN_NATIVE):
        if not os.path.exists(b):
            sys.exit("build the reference first: make -C oracle ref REF=<checkout>")
    which = sys.argv[1:] or ["native_riemann2", "native_smooth", "800", "4096"]
    if "native_riemann2" in which:
        native_riemann2()
    if "native_smooth" in which:
        native_smooth()
    if "800" in which:
        hashed_case("long_riemannseeded_z_rk3_800_t03", 800, 7, -1, 0.3, 25)
    if "4096" in which:
        hashed_case("long_riemannseeded_z_rk3_4096_20steps", 4096, 7, 20, None, 128)


if __name__ == "__main__":
    main()
