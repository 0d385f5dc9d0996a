"""wenofd_calc_dt_noalloc: the time step of a caller-owned device state with no
allocation (for callers whose GPU memory belongs to their own pool, or whose
loop cannot take the device-wide synchronisation of cudaMalloc/cudaFree).

Its result must equal the handle API's wenofd_calc_dt bit for bit (both are
calculateDeltaT's arithmetic), on two calls in a row that share the library's
fixed scratch array.  This file is collected last on purpose."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle as orc
import wenofd

pytestmark = pytest.mark.gpu


def _noalloc(torch, state, nx, ny, info, now):
    dev_state = torch.from_numpy(np.ascontiguousarray(state)).to("cuda")
    dev_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = wenofd.lib().wenofd_calc_dt_noalloc(
        C.c_void_p(dev_state.data_ptr()), nx, ny, info.dx, info.dy, info.gamma, info.cfl, now, info.t_end,
        C.c_void_p(dev_dt.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == wenofd.OK, wenofd.lib().wenofd_last_error().decode()
    torch.cuda.synchronize()
    return float(dev_dt.cpu()[0])


def _reference_dt(tc, nx, ny, state, seed):
    with wenofd.Solver({"TESTCASE": tc, "ELEMNUMX": nx, "ELEMNUMY": ny, "RKMETH": 2, "CFL": 0.7,
                        "SCHEME": 1, "SEED": seed}) as s:
        s.set_state(state)
        return s.calc_dt(), s.info()


def test_noalloc_dt_matches_handle_api_twice():
    torch = pytest.importorskip("torch")
    # first call: a large grid (1024 blocks of partial maxima)
    nx1, ny1 = 700, 500
    p1 = orc.Problem(orc.RIEMANN_SEEDED, nx1, ny1, orc.WENOZ, 2, 0.7, seed=3)
    p1.run(max_steps=3)
    s1 = p1.interior()
    want1, info1 = _reference_dt(orc.RIEMANN_SEEDED, nx1, ny1, s1, 3)
    got1 = _noalloc(torch, s1, nx1, ny1, info1, 0.0)
    assert got1 == want1
    # second call right after: a small grid, fewer blocks; the scratch still
    # holds the first call's partial maxima beyond them
    nx2, ny2 = 40, 30
    p2 = orc.Problem(orc.SHEAR, nx2, ny2, orc.WENOZ, 2, 0.7, seed=9)
    s2 = p2.interior()
    want2, info2 = _reference_dt(orc.SHEAR, nx2, ny2, s2, 9)
    got2 = _noalloc(torch, s2, nx2, ny2, info2, 0.0)
    assert got2 == want2
    # and the oracle's calculateDeltaT agrees
    assert got2 == p2.calc_dt()


def test_noalloc_dt_clips_to_end_time_and_flags_nan():
    torch = pytest.importorskip("torch")
    nx, ny = 64, 48
    p = orc.Problem(orc.RIEMANN2, nx, ny)
    s = p.interior()
    _, info = _reference_dt(orc.RIEMANN2, nx, ny, s, 0)
    assert _noalloc(torch, s, nx, ny, info, info.t_end - 1e-7) == pytest.approx(1e-7, rel=1e-6)
    s[1, 10, 10] = np.nan
    assert np.isnan(_noalloc(torch, s, nx, ny, info, 0.0))


def test_noalloc_rejects_grids_beyond_its_limit():
    L = wenofd.lib()
    rc = L.wenofd_calc_dt_noalloc(C.c_void_p(16), 20000, 20000, 1e-3, 1e-3, 1.4, 0.5, 0.0, 1.0,
                                  C.c_void_p(16), None)
    assert rc == wenofd.BAD_ARG
    assert "exceeds the maximum" in L.wenofd_last_error().decode()


def test_warm_calls_allocate_no_device_memory():
    """The reason the entry point exists: after the first call on a device
    (which loads its kernels and looks up the scratch address), further calls
    take no device memory at all."""
    torch = pytest.importorskip("torch")
    nx, ny = 300, 200
    p = orc.Problem(orc.RIEMANN_SEEDED, nx, ny, orc.WENOZ, 2, 0.7, seed=5)
    s = p.interior()
    want, info = _reference_dt(orc.RIEMANN_SEEDED, nx, ny, s, 5)
    assert _noalloc(torch, s, nx, ny, info, 0.0) == want  # warm-up call
    dev_state = torch.from_numpy(np.ascontiguousarray(s)).to("cuda")
    dev_dt = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        rc = wenofd.lib().wenofd_calc_dt_noalloc(
            C.c_void_p(dev_state.data_ptr()), nx, ny, info.dx, info.dy, info.gamma, info.cfl, 0.0, info.t_end,
            C.c_void_p(dev_dt.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == wenofd.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert float(dev_dt.cpu()[0]) == want


# Run in a child process: cudaDeviceReset ends this process's context, which
# the parent's torch still uses.  Plain CUDA runtime calls through ctypes.
_RESET_CHILD = r"""
import ctypes as C, sys
import numpy as np
sys.path[:0] = sys.argv[1:3]
import oracle as orc, wenofd
L = wenofd.lib()
rt = C.CDLL("libcudart.so.13")  # the runtime libwenofd.so already loaded
nx, ny = 96, 80
p = orc.Problem(orc.RIEMANN_SEEDED, nx, ny, orc.WENOZ, 2, 0.7, seed=13)
U = np.ascontiguousarray(p.interior())
want = p.calc_dt()
g = {"dx": p.grid.dx, "dy": p.grid.dy, "gamma": p.grid.gamma, "t_end": p.t_end}
def once():
    dU, dd = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(dU), C.c_size_t(U.nbytes)) == 0
    assert rt.cudaMalloc(C.byref(dd), C.c_size_t(8)) == 0
    assert rt.cudaMemcpy(dU, U.ctypes.data_as(C.c_void_p), C.c_size_t(U.nbytes), 1) == 0
    rc = L.wenofd_calc_dt_noalloc(dU, nx, ny, C.c_double(g["dx"]), C.c_double(g["dy"]), C.c_double(g["gamma"]),
                                  C.c_double(0.7), C.c_double(0.0), C.c_double(g["t_end"]), dd, None)
    assert rc == 0, L.wenofd_last_error()
    out = C.c_double()
    assert rt.cudaMemcpy(C.byref(out), dd, C.c_size_t(8), 2) == 0
    rt.cudaFree(dU)
    rt.cudaFree(dd)
    return out.value
a = once()
assert rt.cudaDeviceReset() == 0
b = once()
print(a == want, b == want)
"""


def test_call_after_device_reset_looks_the_scratch_up_again():
    """A device reset tears down the context that held the scratch array; the
    next call sees a new context and looks the array's address up again."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    paths = [os.path.join(root, "oracle"), os.path.join(root, "fd-weno-eulerequation_gb300", "python")]
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD] + paths, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.split() == ["True", "True"]
