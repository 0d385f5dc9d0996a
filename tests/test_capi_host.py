"""The C-ABI library without a GPU: it loads, exports every entry point that
include/wenofd.h declares, and rejects bad configurations the way the
reference fails on them (before any device work)."""
import os
import re

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
