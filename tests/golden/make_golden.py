"""Generate the golden fixtures in this directory from the REFERENCE itself.

The reference's own sources (infinity-07/FD-WENO-EulerEquation: src/WENOFD.cpp
plus its headers), unmodified, are compiled against a single-rank MPI shim by
``make -C oracle ref`` (with -ffp-contract=off, so every operation is one IEEE
rounding) and driven by oracle/ref_driver.cpp.  This script runs that binary
on small configurations and stores its inputs and outputs as .npz files.  The
tests then hold the C restatement (oracle/) and the CUDA path to these
outputs bit for bit.

Run it where the reference checkout exists:
    make -C oracle ref && python tests/golden/make_golden.py
The fixtures are committed; the reference is not needed to run the tests.

Fixture layout (one .npz per case):
    meta   JSON string: testcase, nx, ny, scheme, rk, cfl, seed, t_end, mode,
           steps, domain/bc overrides
    init   interior initial state, float64 (4, NX, NY), ej fastest
    rhs    (mode rhs) interior RHS of one assembleRHS()
    ghosted (mode rhs) full state (4, NX+8, NY+8) after the boundary fill
    dt     (mode rhs) calculateDeltaT() of the initial state at t = 0
    state  (mode run) interior state after `steps` steps
    dts    (mode run) the time step of every step
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as orc  # noqa: E402

REF_BIN = orc.REF_BIN

# (name, mode, testcase, nx, ny, scheme, rk, cfl, seed, steps, t_end override)
CASES = [
    ("rhs_smooth_z_20x16", "rhs", orc.SMOOTH, 20, 16, orc.WENOZ, 2, 0.6, 0, 0, None),
    ("rhs_smooth_js_20x16", "rhs", orc.SMOOTH, 20, 16, orc.WENOJS, 2, 0.6, 0, 0, None),
    ("rhs_smooth_zp_18x14", "rhs", orc.SMOOTH, 18, 14, orc.WENOZP, 2, 0.6, 0, 0, None),
    ("rhs_smooth_zpi_18x14", "rhs", orc.SMOOTH, 18, 14, orc.WENOZPI, 2, 0.6, 0, 0, None),
    ("rhs_riemann1_z_16x16", "rhs", orc.RIEMANN1, 16, 16, orc.WENOZ, 2, 0.7, 0, 0, None),
    ("rhs_riemann2_z_17x13", "rhs", orc.RIEMANN2, 17, 13, orc.WENOZ, 2, 0.7, 0, 0, None),
    ("rhs_rti_js_12x24", "rhs", orc.RTI, 12, 24, orc.WENOJS, 2, 0.7, 0, 0, None),
    ("rhs_riemannseeded_z_24x20", "rhs", orc.RIEMANN_SEEDED, 24, 20, orc.WENOZ, 2, 0.7, 7, 0, None),
    ("rhs_shear_z_20x20", "rhs", orc.SHEAR, 20, 20, orc.WENOZ, 2, 0.7, 3, 0, None),
    ("run_smooth_z_rk3_24x20", "run", orc.SMOOTH, 24, 20, orc.WENOZ, 2, 0.6, 0, 20, None),
    ("run_smooth_js_rk2_22x18", "run", orc.SMOOTH, 22, 18, orc.WENOJS, 1, 0.5, 0, 15, None),
    ("run_smooth_z_rk1_16x16", "run", orc.SMOOTH, 16, 16, orc.WENOZ, 0, 0.3, 0, 10, None),
    ("run_riemannseeded_z_rk3_32x28", "run", orc.RIEMANN_SEEDED, 32, 28, orc.WENOZ, 2, 0.7, 11, 30, None),
    ("run_riemann2_z_rk3_40x40_t005", "run", orc.RIEMANN2, 40, 40, orc.WENOZ, 2, 0.7, 0, -1, 0.05),
    ("run_rti_js_rk3_16x40", "run", orc.RTI, 16, 40, orc.WENOJS, 2, 0.7, 0, 20, None),
    ("run_shear_z_rk3_32x32", "run", orc.SHEAR, 32, 32, orc.WENOZ, 2, 0.7, 5, 25, None),
    ("run_riemann1_zpi_rk3_24x24", "run", orc.RIEMANN1, 24, 24, orc.WENOZPI, 2, 0.7, 0, 12, None),
    ("run_smooth_zp_rk3_20x20", "run", orc.SMOOTH, 20, 20, orc.WENOZP, 2, 0.6, 0, 12, None),
]

# The reference's cases are native TESTCASE values; the seeded cases are
# expressed through overrides of a native case.
BASE_TESTCASE = {orc.RIEMANN_SEEDED: orc.RIEMANN2, orc.SHEAR: orc.SMOOTH}


def run_ref(workdir: str, mode: str, testcase: int, nx: int, ny: int, scheme: int, rk: int,
            cfl: float, seed: int = 0, steps: int = -1, t_end: float | None = None,
            init: np.ndarray | None = None, binary: str = REF_BIN) -> dict:
    """Run the compiled reference once; return its outputs as arrays."""
    base = BASE_TESTCASE.get(testcase, testcase)
    cfg = os.path.join(workdir, "config.cfg")
    with open(cfg, "w") as f:
        f.write(f"TESTCASE = {base}\nELEMNUMX = {nx}\nELEMNUMY = {ny}\nRKMETH = {rk}\n"
                f"CFL = {cfl!r}\nSCHEME = {scheme}\n")
    out = os.path.join(workdir, "out")
    args = [binary, cfg, mode, out]
    if steps is not None and steps >= 0:
        args += ["--steps", str(steps)]
    if t_end is not None:
        args += ["--tend", repr(float(t_end))]
    prob = orc.Problem(testcase, nx, ny, scheme, rk, cfl, seed)
    if testcase == orc.RIEMANN_SEEDED:
        args += ["--riemann"] + [repr(float(q)) for q in prob.case.quad]
    if testcase == orc.SHEAR:
        c = prob.case
        args += ["--domain", repr(c.xl), repr(c.xr), repr(c.yl), repr(c.yr)]
        if init is None:
            init = prob.interior()
    if init is not None:
        p = os.path.join(workdir, "init.bin")
        np.ascontiguousarray(init, dtype=np.float64).tofile(p)
        args += ["--init", p]
    r = subprocess.run(args, cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed: {r.stderr[-2000:]}")
    res = {}
    with open(out + ".meta") as f:
        for line in f:
            k, v = line.strip().split("=", 1)
            res[k] = float(v)
    shp = (4, nx, ny)
    res["init"] = np.fromfile(out + ".init").reshape(shp)
    if mode == "rhs":
        res["rhs"] = np.fromfile(out + ".rhs").reshape(shp)
        res["ghosted"] = np.fromfile(out + ".ghosted").reshape(4, nx + 8, ny + 8)
    else:
        res["state"] = np.fromfile(out + ".state").reshape(shp)
        res["dts"] = np.fromfile(out + ".dts")
    return res


# CWENOFD::run of the reference, unchanged (mode fullrun): its output files
# pin the drop-in host class's writers (outputAve, outputError,
# outputAccuracy).
OUTPUT_CASES = [("ref_output_smooth_16x12", "TESTCASE = 0\nELEMNUMX = 16\nELEMNUMY = 12\nRKMETH = 2\n"
                 "CFL = 0.6\nSCHEME = 1\n")]


def make_output_goldens() -> None:
    import glob
    import shutil
    for name, cfg in OUTPUT_CASES:
        dst = os.path.join(HERE, name)
        os.makedirs(dst, exist_ok=True)
        with tempfile.TemporaryDirectory() as wd:
            with open(os.path.join(wd, "config.cfg"), "w") as f:
                f.write(cfg)
            r = subprocess.run([REF_BIN, "config.cfg", "fullrun", "out"], cwd=wd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stderr[-2000:])
            (run_dir,) = glob.glob(os.path.join(wd, "output", "*_SMOOTH_*"))
            for fn in ("solution_initial.plt", "solution_final.plt", "error_final.plt", "accuracy_final.csv"):
                shutil.copy(os.path.join(run_dir, fn), os.path.join(dst, fn))
            shutil.copy(os.path.join(wd, "config.cfg"), os.path.join(dst, "config.cfg"))
        print(f"{name}: reference output files")


def main() -> None:
    if not os.path.exists(REF_BIN):
        sys.exit("build the reference first: make -C oracle ref")
    make_output_goldens()
    for (name, mode, tc, nx, ny, sch, rk, cfl, seed, steps, t_end) in CASES:
        with tempfile.TemporaryDirectory() as wd:
            res = run_ref(wd, mode, tc, nx, ny, sch, rk, cfl, seed, steps, t_end)
        meta = dict(testcase=tc, nx=nx, ny=ny, scheme=sch, rk=rk, cfl=cfl, seed=seed, mode=mode,
                    steps=int(res.get("steps", 0)), t_end=t_end, dx=res["dx"], dy=res["dy"])
        arrays = {"meta": np.array(json.dumps(meta)), "init": res["init"]}
        if mode == "rhs":
            arrays.update(rhs=res["rhs"], ghosted=res["ghosted"], dt=np.array(res["dt"]))
        else:
            arrays.update(state=res["state"], dts=res["dts"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(f"{name}: {meta['steps']} steps")


if __name__ == "__main__":
    main()
