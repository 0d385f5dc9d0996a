"""ctypes binding of the wenofd C ABI (include/wenofd.h).

The solver runs only through libwenofd.so's CUDA kernels: there is no CPU
fallback, and importing this module raises if the library is missing.

    import wenofd
    s = wenofd.Solver({"TESTCASE": 4, "ELEMNUMX": 800, "ELEMNUMY": 800,
                       "RKMETH": 2, "CFL": 0.7, "SCHEME": 1, "SEED": 7})
    s.initialize()
    s.advance(max_steps=100)
    U = s.get_state()          # float64 (4, NX, NY), ej fastest
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
# WENOFD_LIBRARY selects another build of the library, e.g. the bounds-checked
# one (_build_check/libwenofd.so, build.py --bounds-check).
LIB_PATH = os.environ.get("WENOFD_LIBRARY") or os.path.join(PKG, "_build", "libwenofd.so")

OK, BAD_CONFIG, CUDA_ERROR, NAN_DT, TIMEOUT, BAD_ARG, NO_EXACT = range(7)
FP64, FP32, LEARNED = 0, 1, 2
MLP_INPUTS, MLP_PARAMS = 50, 2721
SMOOTH, RIEMANN1, RIEMANN2, RTI, RIEMANN_SEEDED, SHEAR = range(6)
WENOJS, WENOZ, WENOZP, WENOZPI = range(4)
RK1, RK2, RK3 = range(3)


class WenofdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"wenofd status {status}: {message}")
        self.status = status


class Info(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int),
        ("testcase", C.c_int), ("scheme", C.c_int), ("rk", C.c_int), ("precision", C.c_int),
        ("bc_left", C.c_int), ("bc_right", C.c_int), ("bc_bottom", C.c_int), ("bc_top", C.c_int),
        ("has_exact", C.c_int), ("pitch", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("cfl", C.c_double), ("t_end", C.c_double),
        ("now", C.c_double), ("gamma", C.c_double),
        ("xl", C.c_double), ("xr", C.c_double), ("yl", C.c_double), ("yr", C.c_double),
        ("steps", C.c_longlong),
        ("launches", C.c_longlong),
        ("graph_steps", C.c_int),
        ("dt", C.c_double),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("members", C.c_int), ("precision", C.c_int), ("tile_i", C.c_int), ("blocks_per_sm", C.c_int),
        ("grid", C.c_int), ("steps_per_launch", C.c_int), ("graph", C.c_int),
        ("cells", C.c_longlong), ("launches", C.c_longlong), ("tuned_ms_per_step", C.c_double),
    ]


_lib = None


def lib() -> C.CDLL:
    """Load libwenofd.so (build it with fd-weno-eulerequation_gb300/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libwenofd.so not built: {LIB_PATH} (run fd-weno-eulerequation_gb300/build.py)")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        P = C.POINTER(C.c_double)
        L.wenofd_last_error.restype = C.c_char_p
        L.wenofd_version.restype = C.c_char_p
        L.wenofd_create.argtypes = [C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int, C.POINTER(H)]
        L.wenofd_create_from_file.argtypes = [C.c_char_p, C.POINTER(H)]
        L.wenofd_destroy.argtypes = [H]
        L.wenofd_set_stream.argtypes = [H, C.c_void_p]
        L.wenofd_get_info.argtypes = [H, C.POINTER(Info)]
        for name in ("wenofd_initialize", "wenofd_fill_boundary"):
            getattr(L, name).argtypes = [H]
        for name in ("wenofd_set_state", "wenofd_get_state", "wenofd_get_state_ghosted", "wenofd_get_flux",
                     "wenofd_set_boundary_values",
                     "wenofd_calc_dt", "wenofd_step", "wenofd_error_norms", "wenofd_conservation_sums"):
            getattr(L, name).argtypes = [H, P]
        L.wenofd_set_state_device.argtypes = [H, C.c_void_p]
        L.wenofd_get_state_device.argtypes = [H, C.c_void_p]
        L.wenofd_set_time.argtypes = [H, C.c_double]
        L.wenofd_rk_step.argtypes = [H, C.c_double]
        L.wenofd_advance.argtypes = [H, C.c_longlong, C.POINTER(C.c_longlong)]
        L.wenofd_time_stages.argtypes = [H, C.c_int, P]
        VP = C.c_void_p
        L.wenofd_set_indicator.argtypes = [H, C.POINTER(C.c_float), C.c_float]
        L.wenofd_indicator_flags.argtypes = [H, C.POINTER(C.c_ubyte)]
        L.wenofd_routing_flags.argtypes = [H, C.POINTER(C.c_ubyte)]
        L.wenofd_indicator_data.argtypes = [H, VP, VP]
        L.wenofd_mlp_forward.argtypes = [VP, VP, C.c_longlong, VP, VP]
        L.wenofd_mlp_backward.argtypes = [VP, VP, VP, C.c_longlong, VP, VP, VP]
        L.wenofd_mlp_adam.argtypes = [VP, VP, VP, VP, C.c_int, C.c_float, VP]
        L.wenofd_mlp_train.argtypes = [VP, VP, VP, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_ulonglong,
                                       C.POINTER(C.c_float), VP]
        D = C.c_double
        L.wenofd_calc_dt_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, D, D, D, D, D, D, C.c_void_p,
                                             C.c_void_p]
        L.wenofd_batch_create.argtypes = [C.POINTER(H), C.c_int, C.POINTER(H)]
        L.wenofd_batch_destroy.argtypes = [H]
        L.wenofd_batch_configure.argtypes = [H, C.c_int, C.c_int, C.c_int]
        L.wenofd_batch_autotune.argtypes = [H, C.c_int, P]
        L.wenofd_batch_advance.argtypes = [H, C.c_longlong, C.POINTER(C.c_longlong)]
        L.wenofd_batch_get_info.argtypes = [H, C.POINTER(BatchInfo)]
        L.wenofd_batch_test_withhold.argtypes = [H, C.c_int, C.c_int]
        L.wenofd_output_variables.argtypes = [H, P]
        L.wenofd_indicator_sample.argtypes = [H, C.c_longlong, C.c_ulonglong, VP, VP, C.c_longlong,
                                              C.POINTER(C.c_longlong)]
        L.wenofd_mlp_init.argtypes = [C.POINTER(C.c_float), C.c_ulonglong]
        L.wenofd_save_state.argtypes = [H, C.c_char_p]
        L.wenofd_load_state.argtypes = [H, C.c_char_p]
        L.wenofd_bounds_report.argtypes = [C.POINTER(C.c_longlong), C.c_char_p, C.c_int, C.c_int]
        L.wenofd_bounds_selftest.argtypes = [C.POINTER(C.c_longlong), C.c_char_p, C.c_int]
        for f in ("wenofd_batch_create", "wenofd_batch_destroy", "wenofd_batch_configure", "wenofd_batch_autotune",
                  "wenofd_batch_advance", "wenofd_batch_get_info", "wenofd_batch_test_withhold"):
            getattr(L, f).restype = C.c_int
        for f in ("wenofd_create", "wenofd_create_from_file", "wenofd_destroy", "wenofd_set_stream",
                  "wenofd_get_info", "wenofd_initialize", "wenofd_fill_boundary", "wenofd_set_state",
                  "wenofd_get_state", "wenofd_get_state_ghosted", "wenofd_get_flux", "wenofd_calc_dt",
                  "wenofd_step", "wenofd_error_norms", "wenofd_conservation_sums", "wenofd_set_state_device",
                  "wenofd_get_state_device", "wenofd_set_time", "wenofd_rk_step", "wenofd_advance",
                  "wenofd_time_stages", "wenofd_calc_dt_noalloc", "wenofd_set_boundary_values",
                  "wenofd_set_indicator", "wenofd_indicator_flags", "wenofd_routing_flags", "wenofd_indicator_data",
                  "wenofd_mlp_forward", "wenofd_output_variables", "wenofd_save_state", "wenofd_load_state",
                  "wenofd_indicator_sample", "wenofd_mlp_init", "wenofd_bounds_report", "wenofd_bounds_selftest",
                  "wenofd_mlp_backward", "wenofd_mlp_adam", "wenofd_mlp_train"):
            getattr(L, f).restype = C.c_int
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != OK:
        raise WenofdError(rc, lib().wenofd_last_error().decode())


def _dptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Solver:
    """One device-resident solve behind the C ABI (the CWENOFD hot path)."""

    def __init__(self, config: dict | None = None, config_file: str | None = None):
        L = lib()
        self._h = C.c_void_p()
        if config_file is not None:
            _check(L.wenofd_create_from_file(config_file.encode(), C.byref(self._h)))
        else:
            keys = [str(k).encode() for k in config]
            vals = [(repr(v) if isinstance(v, float) else str(v)).encode() for v in config.values()]
            K = (C.c_char_p * len(keys))(*keys)
            V = (C.c_char_p * len(vals))(*vals)
            _check(L.wenofd_create(K, V, len(keys), C.byref(self._h)))
        i = self.info()
        self.nx, self.ny = i.nx, i.ny

    def close(self) -> None:
        if self._h:
            lib().wenofd_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def info(self) -> Info:
        i = Info()
        _check(lib().wenofd_get_info(self._h, C.byref(i)))
        return i

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(lib().wenofd_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def initialize(self) -> None:
        _check(lib().wenofd_initialize(self._h))

    def set_state(self, U: np.ndarray) -> None:
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != (4, self.nx, self.ny):
            raise ValueError(f"state shape {U.shape} != {(4, self.nx, self.ny)}")
        _check(lib().wenofd_set_state(self._h, _dptr(U)))

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty((4, self.nx, self.ny)) if out is None else out
        _check(lib().wenofd_get_state(self._h, _dptr(out)))
        return out

    def get_state_ghosted(self) -> np.ndarray:
        out = np.empty((4, self.nx + 8, self.ny + 8))
        _check(lib().wenofd_get_state_ghosted(self._h, _dptr(out)))
        return out

    def set_time(self, now: float) -> None:
        _check(lib().wenofd_set_time(self._h, now))

    def set_boundary_values(self, table: np.ndarray) -> None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        if table.size != 8 * (self.nx + 8) + 8 * (self.ny + 8):
            raise ValueError("SPECIAL table size mismatch")
        _check(lib().wenofd_set_boundary_values(self._h, _dptr(table)))

    def fill_boundary(self) -> None:
        _check(lib().wenofd_fill_boundary(self._h))

    def get_flux(self) -> np.ndarray:
        out = np.empty((4, self.nx, self.ny))
        _check(lib().wenofd_get_flux(self._h, _dptr(out)))
        return out

    def calc_dt(self) -> float:
        dt = np.zeros(1)
        _check(lib().wenofd_calc_dt(self._h, _dptr(dt)))
        return float(dt[0])

    def rk_step(self, dt: float) -> None:
        _check(lib().wenofd_rk_step(self._h, dt))

    def step(self) -> float:
        dt = np.zeros(1)
        _check(lib().wenofd_step(self._h, _dptr(dt)))
        return float(dt[0])

    def advance(self, max_steps: int = -1) -> int:
        n = C.c_longlong(0)
        _check(lib().wenofd_advance(self._h, max_steps, C.byref(n)))
        return n.value

    def error_norms(self) -> np.ndarray:
        out = np.zeros(3)
        _check(lib().wenofd_error_norms(self._h, _dptr(out)))
        return out

    def set_state_ptr(self, host_ptr: int) -> None:
        """Upload from a raw host address (e.g. pinned memory), [4][NX][NY] float64."""
        _check(lib().wenofd_set_state(self._h, C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double))))

    def get_state_ptr(self, host_ptr: int) -> None:
        _check(lib().wenofd_get_state(self._h, C.cast(C.c_void_p(host_ptr), C.POINTER(C.c_double))))

    def time_stages(self, reps: int) -> float:
        ms = np.zeros(1)
        _check(lib().wenofd_time_stages(self._h, reps, _dptr(ms)))
        return float(ms[0])

    def set_indicator(self, params: np.ndarray, threshold: float = 0.5) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != MLP_PARAMS:
            raise ValueError(f"expected {MLP_PARAMS} parameters")
        _check(lib().wenofd_set_indicator(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), threshold))

    def indicator_flags(self) -> np.ndarray:
        out = np.zeros((self.nx, self.ny), dtype=np.uint8)
        _check(lib().wenofd_indicator_flags(self._h, out.ctypes.data_as(C.POINTER(C.c_ubyte))))
        return out

    def routing_flags(self) -> np.ndarray:
        """The stored flags that routed the last step (no indicator run)."""
        out = np.zeros((self.nx, self.ny), dtype=np.uint8)
        _check(lib().wenofd_routing_flags(self._h, out.ctypes.data_as(C.POINTER(C.c_ubyte))))
        return out

    def indicator_data(self, dev_features: int | None, dev_labels: int | None) -> None:
        """Features [NX*NY][50] float32 / labels [NX*NY] uint8 into device buffers."""
        _check(lib().wenofd_indicator_data(self._h, C.c_void_p(dev_features or 0), C.c_void_p(dev_labels or 0)))

    def conservation_sums(self) -> np.ndarray:
        out = np.zeros(4)
        _check(lib().wenofd_conservation_sums(self._h, _dptr(out)))
        return out

    def output_variables(self) -> np.ndarray:
        """outputAve's (rho, u, v, pre, c, E), (6, NX, NY), computed on the device."""
        i = self.info()
        out = np.zeros((6, i.nx, i.ny))
        _check(lib().wenofd_output_variables(self._h, _dptr(out)))
        return out

    def indicator_sample(self, per_snapshot: int, seed: int, x_ptr: int, y_ptr: int, capacity: int) -> int:
        """Balanced device-side training sample of the current state
        (wenofd_indicator_sample); returns the rows written."""
        rows = C.c_longlong()
        _check(lib().wenofd_indicator_sample(self._h, per_snapshot, seed, C.c_void_p(x_ptr), C.c_void_p(y_ptr),
                                             capacity, C.byref(rows)))
        return rows.value

    def save_state(self, path: str) -> None:
        _check(lib().wenofd_save_state(self._h, os.fsencode(path)))

    def load_state(self, path: str) -> None:
        _check(lib().wenofd_load_state(self._h, os.fsencode(path)))


class Batch:
    """Many Solver handles advanced together by one persistent kernel
    (wenofd_batch_*).  Members keep their own state: read it through them."""

    def __init__(self, members: list[Solver]):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m._h for m in self.members])
        self._h = C.c_void_p()
        _check(lib().wenofd_batch_create(arr, len(self.members), C.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().wenofd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def configure(self, tile_i: int = 0, blocks_per_sm: int = 0, steps_per_launch: int = 0) -> None:
        _check(lib().wenofd_batch_configure(self._h, tile_i, blocks_per_sm, steps_per_launch))

    def autotune(self, steps: int = 3) -> float:
        ms = C.c_double()
        _check(lib().wenofd_batch_autotune(self._h, steps, C.byref(ms)))
        return ms.value

    def advance(self, max_steps: int = -1) -> int:
        n = C.c_longlong()
        _check(lib().wenofd_batch_advance(self._h, max_steps, C.byref(n)))
        return n.value

    def info(self) -> BatchInfo:
        i = BatchInfo()
        _check(lib().wenofd_batch_get_info(self._h, C.byref(i)))
        return i

    def test_withhold(self, block: int = 0, barrier: int = 1) -> None:
        """Arm the barrier give-up test (wenofd_batch_test_withhold)."""
        _check(lib().wenofd_batch_test_withhold(self._h, block, barrier))


EXPORTED = [
    "wenofd_last_error", "wenofd_version", "wenofd_create", "wenofd_create_from_file", "wenofd_destroy",
    "wenofd_set_stream", "wenofd_get_info", "wenofd_initialize", "wenofd_set_state", "wenofd_get_state",
    "wenofd_set_state_device", "wenofd_get_state_device", "wenofd_get_state_ghosted", "wenofd_set_time",
    "wenofd_fill_boundary", "wenofd_get_flux", "wenofd_calc_dt", "wenofd_rk_step", "wenofd_step",
    "wenofd_advance", "wenofd_error_norms", "wenofd_conservation_sums", "wenofd_time_stages",
    "wenofd_calc_dt_noalloc", "wenofd_set_boundary_values", "wenofd_set_indicator", "wenofd_indicator_flags",
    "wenofd_routing_flags",
    "wenofd_indicator_data", "wenofd_mlp_forward", "wenofd_mlp_backward", "wenofd_mlp_adam", "wenofd_mlp_train",
    "wenofd_batch_create", "wenofd_batch_destroy", "wenofd_batch_configure", "wenofd_batch_autotune",
    "wenofd_batch_advance", "wenofd_batch_get_info", "wenofd_batch_test_withhold", "wenofd_output_variables",
    "wenofd_save_state", "wenofd_load_state", "wenofd_indicator_sample", "wenofd_mlp_init",
    "wenofd_bounds_report", "wenofd_bounds_selftest",
]


def mlp_init(seed: int) -> np.ndarray:
    """Initial network parameters (wenofd_mlp_init, host only)."""
    out = np.zeros(MLP_PARAMS, dtype=np.float32)
    _check(lib().wenofd_mlp_init(out.ctypes.data_as(C.POINTER(C.c_float)), seed))
    return out


def mlp_forward(params_ptr: int, x_ptr: int, n: int, logits_ptr: int, stream: int = 0) -> None:
    _check(lib().wenofd_mlp_forward(C.c_void_p(params_ptr), C.c_void_p(x_ptr), n, C.c_void_p(logits_ptr),
                                    C.c_void_p(stream)))


def mlp_backward(params_ptr: int, x_ptr: int, y_ptr: int, n: int, grad_ptr: int, loss_ptr: int,
                 stream: int = 0) -> None:
    _check(lib().wenofd_mlp_backward(C.c_void_p(params_ptr), C.c_void_p(x_ptr), C.c_void_p(y_ptr), n,
                                     C.c_void_p(grad_ptr), C.c_void_p(loss_ptr), C.c_void_p(stream)))


def mlp_adam(params_ptr: int, grad_ptr: int, m_ptr: int, v_ptr: int, step: int, lr: float, stream: int = 0) -> None:
    _check(lib().wenofd_mlp_adam(C.c_void_p(params_ptr), C.c_void_p(grad_ptr), C.c_void_p(m_ptr),
                                 C.c_void_p(v_ptr), step, lr, C.c_void_p(stream)))


def mlp_train(params_ptr: int, x_ptr: int, y_ptr: int, n: int, epochs: int, batch: int, lr: float, seed: int,
              stream: int = 0) -> np.ndarray:
    losses = np.zeros(epochs, dtype=np.float32)
    _check(lib().wenofd_mlp_train(C.c_void_p(params_ptr), C.c_void_p(x_ptr), C.c_void_p(y_ptr), n, epochs, batch,
                                  lr, seed, losses.ctypes.data_as(C.POINTER(C.c_float)), C.c_void_p(stream)))
    return losses


def bounds_report(reset: bool = False) -> dict:
    """The device guard record of the bounds-checked library
    (wenofd_bounds_report): count (-1 in the release library), and the first
    violation's line, index, extent and "file:line"."""
    r = (C.c_longlong * 4)()
    where = C.create_string_buffer(128)
    _check(lib().wenofd_bounds_report(r, where, 128, 1 if reset else 0))
    return {"count": r[0], "line": r[1], "index": r[2], "extent": r[3], "where": where.value.decode()}


def bounds_selftest() -> dict:
    """One guarded access one past the end of a 4-element array against a
    private record (wenofd_bounds_selftest), reported like bounds_report."""
    r = (C.c_longlong * 4)()
    where = C.create_string_buffer(128)
    _check(lib().wenofd_bounds_selftest(r, where, 128))
    return {"count": r[0], "line": r[1], "index": r[2], "extent": r[3], "where": where.value.decode()}
