"""The output / restart path through the C ABI: outputAve's variables computed
on the device (wenofd_output_variables) against the reference's formula
(utils/equations.hpp:679-694) evaluated on the downloaded state, and binary
restart (wenofd_save_state / wenofd_load_state): a run continued from a saved
state is bit for bit the uninterrupted run, in every precision form."""
import numpy as np
import pytest

import mlp_oracle
import oracle as orc
import wenofd

pytestmark = pytest.mark.gpu


def _cfg(precision=wenofd.FP64, **extra):
    c = {"TESTCASE": orc.RIEMANN_SEEDED, "ELEMNUMX": 96, "ELEMNUMY": 80, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1,
         "SEED": 12, "PRECISION": precision}
    c.update(extra)
    return c


def test_output_variables_match_the_reference_formula():
    with wenofd.Solver(_cfg()) as s:
        s.initialize()
        s.advance(max_steps=6)
        U = s.get_state()
        got = s.output_variables()
        gamma = s.info().gamma
    rho, E = U[0], U[3]
    u = U[1] / U[0]
    v = U[2] / U[0]
    pre = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v))
    c = np.sqrt(gamma * pre / rho)
    want = np.stack([rho, u, v, pre, c, E])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("precision", [wenofd.FP64, wenofd.FP32, wenofd.LEARNED])
def test_restart_continues_bit_for_bit(tmp_path, precision):
    path = str(tmp_path / "state.bin")
    params = mlp_oracle.init_params(3) if precision == wenofd.LEARNED else None

    def solver():
        s = wenofd.Solver(_cfg(precision))
        if params is not None:
            s.set_indicator(params, 0.5)
        return s

    with solver() as a:
        a.initialize()
        assert a.advance(max_steps=7) == 7
        a.save_state(path)
        assert a.advance(max_steps=9) == 9
        want, now, steps = a.get_state(), a.info().now, a.info().steps
    with solver() as b:
        b.load_state(path)
        assert b.info().steps == 7
        assert b.advance(max_steps=9) == 9
        assert np.array_equal(b.get_state(), want)
        assert b.info().now == now and b.info().steps == steps == 16


def test_load_rejects_other_grids_and_other_files(tmp_path):
    path = str(tmp_path / "state.bin")
    with wenofd.Solver(_cfg()) as a:
        a.initialize()
        a.save_state(path)
    with wenofd.Solver(_cfg(ELEMNUMX=64)) as b:
        with pytest.raises(wenofd.WenofdError) as e:
            b.load_state(path)
        assert e.value.status == wenofd.BAD_CONFIG
    junk = tmp_path / "junk.bin"
    junk.write_bytes(b"not a state file" * 8)
    with wenofd.Solver(_cfg()) as c:
        with pytest.raises(wenofd.WenofdError) as e:
            c.load_state(str(junk))
        assert e.value.status == wenofd.BAD_ARG
        with open(path, "rb") as f:
            head = f.read(200)
        short = tmp_path / "short.bin"
        short.write_bytes(head)  # header and a fragment of the state
        with pytest.raises(wenofd.WenofdError) as e:
            c.load_state(str(short))
        assert "truncated" in str(e.value)
