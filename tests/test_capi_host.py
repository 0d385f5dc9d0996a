"""The C-ABI library without a GPU: it loads, exports every entry point that
include/wenofd.h declares, and rejects bad configurations the way the
reference fails on them (before any device work)."""
import os
import re

import numpy as np
import pytest

import wenofd
from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "wenofd.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wenofd_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = wenofd.lib()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(wenofd.EXPORTED)


def test_version_string():
    assert b"sm_103a" in wenofd.lib().wenofd_version()


@pytest.mark.parametrize("cfg,needle", [
    ({"ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1}, "TESTCASE"),
    ({"TESTCASE": 9, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1}, "Invalid example"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 5, "CFL": 0.5, "SCHEME": 1}, "Runge-Kutta"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 7}, "scheme"),
    ({"TESTCASE": 0, "ELEMNUMX": "x", "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1}, "ELEMNUMX"),
    ({"TESTCASE": 0, "ELEMNUMX": 3, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1}, "at least"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": -1.0, "SCHEME": 1}, "CFL"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "PRECISION": 4},
     "PRECISION"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "INDICATOR_INTERVAL": 0},
     "INDICATOR_INTERVAL"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "LABEL_DEVIATION": 0},
     "LABEL_DEVIATION"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "INDICATOR_GUARD": -0.5},
     "INDICATOR_GUARD"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1, "INDICATOR_GUARD": "x"},
     "INDICATOR_GUARD"),
    ({"TESTCASE": 0, "ELEMNUMX": 10, "ELEMNUMY": 10, "RKMETH": 2, "CFL": 0.5, "SCHEME": 1,
      "LABEL_DEVIATION": "x"}, "LABEL_DEVIATION"),
])
def test_bad_config_is_rejected(cfg, needle):
    with pytest.raises(wenofd.WenofdError) as e:
        wenofd.Solver(cfg)
    assert e.value.status == wenofd.BAD_CONFIG
    assert needle in str(e.value)


def test_missing_config_file(tmp_path):
    with pytest.raises(wenofd.WenofdError) as e:
        wenofd.Solver(config_file=str(tmp_path / "nope.cfg"))
    assert e.value.status == wenofd.BAD_CONFIG
    assert "Failed to open file" in str(e.value)


def test_config_file_parser_semantics(tmp_path):
    """utils/readConfig.hpp:39-80: comments, blank lines, '\\r', spaces,
    lines without '=' skipped.  A bad value still fails, so a file whose
    keys parse reaches the device stage only when a GPU is present."""
    p = tmp_path / "config.cfg"
    p.write_bytes(b"# comment\r\n\r\nTESTCASE = 9\r\nno equals sign here\nELEMNUMX = 20 \n"
                  b"ELEMNUMY=20\nRKMETH = 2\nCFL = 0.5\nSCHEME = 1\n")
    with pytest.raises(wenofd.WenofdError) as e:
        wenofd.Solver(config_file=str(p))
    assert "Invalid example" in str(e.value)


def test_mlp_init_is_seeded_and_scaled():
    """wenofd_mlp_init (host only): the same seed gives the same parameters,
    weights within their He-uniform ranges, biases zero."""
    a, b, c = wenofd.mlp_init(7), wenofd.mlp_init(7), wenofd.mlp_init(8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    w1, b1, w2, b2, w3, b3 = a[:1600], a[1600:1632], a[1632:2656], a[2656:2688], a[2688:2720], a[2720]
    assert np.abs(w1).max() <= np.sqrt(6 / 50) and np.abs(w1).max() > 0.9 * np.sqrt(6 / 50)
    assert np.abs(w2).max() <= np.sqrt(6 / 32) and np.abs(w3).max() <= np.sqrt(6 / 32)
    assert not b1.any() and not b2.any() and b3 == 0.0
    assert abs(float(w1.mean())) < 0.05


def test_bounds_report_release_and_checked_exports():
    """The release library reports no guards (count -1, no GPU needed); the
    bounds-checked debug library, when built, exports the same ABI."""
    import ctypes

    rep = wenofd.bounds_report()
    assert rep["count"] == -1 and rep["where"] == ""
    checked = os.path.join(ROOT, "fd-weno-eulerequation_gb300", "_build_check", "libwenofd.so")
    if not os.path.exists(checked):
        pytest.skip("bounds-checked library not built (build.py --bounds-check)")
    L = ctypes.CDLL(checked)
    for name in wenofd.EXPORTED:
        assert hasattr(L, name), name
