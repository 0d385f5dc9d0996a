"""The drop-in host driver (host/main.cpp + host/WENOFD.cpp): the reference's
flow -- read ./input/config.cfg, CWENOFD::run, write solution_initial.plt,
solution_final.plt, error_final.plt and accuracy_final.csv into
./output/<timestamp>_<CASE>_<SCHEME>_<NX>x<NY>/ -- on the GPU.  Its files are
compared with the files the reference itself wrote for the same config
(tests/golden/ref_output_smooth_16x12, made by make_golden.py)."""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

EXE = os.path.join(ROOT, "fd-weno-eulerequation_gb300", "_build", "wenofd")
REF = os.path.join(GOLDEN, "ref_output_smooth_16x12")


def _run_driver(tmp_path, cfg_text):
    os.makedirs(tmp_path / "input", exist_ok=True)
    (tmp_path / "input" / "config.cfg").write_text(cfg_text)
    return subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=300)


def test_driver_rejects_bad_testcase(tmp_path):
    r = _run_driver(tmp_path, "TESTCASE = 9\nELEMNUMX = 16\nELEMNUMY = 12\nRKMETH = 2\nCFL = 0.6\nSCHEME = 1\n")
    assert r.returncode == 1
    assert "Invalid example number" in r.stderr


def test_driver_missing_config(tmp_path):
    r = subprocess.run([EXE], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Failed to open file" in r.stderr


@pytest.mark.gpu
def test_driver_reproduces_reference_output_files(tmp_path):
    r = _run_driver(tmp_path, open(os.path.join(REF, "config.cfg")).read())
    assert r.returncode == 0, r.stderr
    (out,) = glob.glob(str(tmp_path / "output" / "*_SMOOTH_WENOZ_16x12"))
    for fn in ("solution_initial.plt", "solution_final.plt", "error_final.plt"):
        ours = open(os.path.join(out, fn)).read()
        ref = open(os.path.join(REF, fn)).read()
        assert ours == ref, fn
    ours = open(os.path.join(out, "accuracy_final.csv")).read().splitlines()
    ref = open(os.path.join(REF, "accuracy_final.csv")).read().splitlines()
    assert ours[0] == ref[0]
    a = np.array([float(x) for x in ours[1].split(",")])
    b = np.array([float(x) for x in ref[1].split(",")])
    assert np.allclose(a, b, rtol=1e-9, atol=0)
    # the reference's progress line (src/WENOFD.cpp:247-272) after step 1 and
    # after every device chunk (a multiple of 20 steps), so at counts 1 mod 20
    prog = [ln for ln in r.stdout.splitlines() if ln.startswith("Iteration count: ")]
    counts = [int(ln.split(",")[0].split(": ")[1]) for ln in prog]
    assert counts and counts[0] == 1 and all(c % 20 == 1 for c in counts) and counts == sorted(counts)
    assert all(", DeltaT: " in ln and " seconds, Progress: " in ln and ln.endswith("]") for ln in prog)
    shutil.rmtree(tmp_path / "output")
