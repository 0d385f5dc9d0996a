"""ctypes view of the C restatement in wenofd_oracle.c.

TEST INFRASTRUCTURE, NOT PRODUCT.  Imported only by tests/, by
``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg, always as the
checker or the CPU baseline, never as the measured GPU path.

Full states are float64 arrays of shape (4, NX+8, NY+8) (ej fastest), the
structure-of-arrays form of the reference's m_Uh[ei][ej].vector[r]; interior
states are (4, NX, NY).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "wenofd_ref")
NG = 4

PERIOD, SLIP, SPECIAL, SYMMETRIC = 0, 1, 2, 3
WENOJS, WENOZ, WENOZP, WENOZPI = 0, 1, 2, 3
SMOOTH, RIEMANN1, RIEMANN2, RTI, RIEMANN_SEEDED, SHEAR = 0, 1, 2, 3, 4, 5


class Case(C.Structure):
    _fields_ = [
        ("testcase", C.c_int),
        ("xl", C.c_double), ("xr", C.c_double), ("yl", C.c_double), ("yr", C.c_double),
        ("t_end", C.c_double), ("gamma", C.c_double),
        ("bc_left", C.c_int), ("bc_right", C.c_int), ("bc_bottom", C.c_int), ("bc_top", C.c_int),
        ("gravity", C.c_int), ("exact", C.c_int),
        ("quad", C.c_double * 16),
        ("interface", C.c_double),
        ("seed", C.c_ulonglong),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("scheme", C.c_int),
        ("bc_left", C.c_int), ("bc_right", C.c_int), ("bc_bottom", C.c_int), ("bc_top", C.c_int),
        ("gravity", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("gamma", C.c_double),
        ("zp_lambda", C.c_double),
        ("xl", C.c_double), ("yl", C.c_double),
        ("special", C.POINTER(C.c_double)),
    ]


def build() -> None:
    """Compile the restatement (``make`` in this directory)."""
    subprocess.run(["make", "-s", "-C", HERE, "_build/liboracle.so"], check=True)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        D, I, P = C.c_double, C.c_int, C.POINTER(C.c_double)
        L.orc_weno5.restype = D
        L.orc_weno5.argtypes = [I, D, D, D, D, D, D]
        L.orc_wenoz_weights.argtypes = [D, D, D, D, D, P]
        L.orc_phys_flux.argtypes = [I, D, P, P]
        L.orc_max_eig.restype = D
        L.orc_max_eig.argtypes = [I, D, P]
        L.orc_flux_split.argtypes = [I, D, P, P, P]
        L.orc_eigen_lr.argtypes = [I, D, P, P, P]
        L.orc_case_setup.argtypes = [I, C.c_ulonglong, C.POINTER(Case)]
        L.orc_grid_setup.argtypes = [C.POINTER(Case), I, I, I, C.POINTER(Grid)]
        L.orc_node_x.restype = D
        L.orc_node_x.argtypes = [C.POINTER(Grid), I]
        L.orc_node_y.restype = D
        L.orc_node_y.argtypes = [C.POINTER(Grid), I]
        L.orc_u0.argtypes = [C.POINTER(Case), D, D, P]
        L.orc_initial_state.argtypes = [C.POINTER(Case), C.POINTER(Grid), P]
        L.orc_special_table_size.restype = C.c_long
        L.orc_special_table_size.argtypes = [C.POINTER(Grid)]
        L.orc_special_table.argtypes = [C.POINTER(Case), C.POINTER(Grid), P]
        L.orc_fill_boundary.argtypes = [C.POINTER(Grid), P]
        L.orc_assemble_rhs.argtypes = [C.POINTER(Grid), P, P]
        L.orc_fill_boundary_slab.argtypes = [C.POINTER(Grid), P, I, I]
        L.orc_assemble_rhs_ghosted.argtypes = [C.POINTER(Grid), P, P]
        L.orc_calc_dt.restype = I
        L.orc_calc_dt.argtypes = [C.POINTER(Grid), P, D, D, D, P]
        L.orc_rk_step.argtypes = [C.POINTER(Grid), I, P, P, P, D]
        L.orc_run.restype = I
        L.orc_run.argtypes = [C.POINTER(Grid), I, D, P, P, P, P, D, C.c_long,
                              C.POINTER(C.c_long), P, C.c_long]
        L.orc_error_norms.argtypes = [C.POINTER(Grid), P, D, P]
        L.orc_conservation_sums.argtypes = [C.POINTER(Grid), P, P]
        L.orc_cell_features.argtypes = [C.POINTER(Grid), P, C.POINTER(C.c_float)]
        L.orc_cell_labels.argtypes = [C.POINTER(Grid), P, C.POINTER(C.c_ubyte)]
        L.orc_cell_labels_at.argtypes = [C.POINTER(Grid), P, C.POINTER(C.c_ubyte), D]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def weno5(scheme, a, b, c, d, e, zp_lambda=0.0) -> float:
    return lib().orc_weno5(scheme, a, b, c, d, e, zp_lambda)


def wenoz_weights(a, b, c, d, e) -> np.ndarray:
    w = np.zeros(3)
    lib().orc_wenoz_weights(a, b, c, d, e, _p(w))
    return w


def flux_split(direction: int, gamma: float, U) -> tuple[np.ndarray, np.ndarray]:
    U = np.ascontiguousarray(U, dtype=np.float64)
    fm, fp = np.zeros(4), np.zeros(4)
    lib().orc_flux_split(direction, gamma, _p(U), _p(fm), _p(fp))
    return fm, fp


def eigen_lr(direction: int, gamma: float, U) -> tuple[np.ndarray, np.ndarray]:
    U = np.ascontiguousarray(U, dtype=np.float64)
    L, R = np.zeros(16), np.zeros(16)
    lib().orc_eigen_lr(direction, gamma, _p(U), _p(L), _p(R))
    return L.reshape(4, 4), R.reshape(4, 4)


class Problem:
    """One configured solve on the CPU restatement."""

    def __init__(self, testcase: int, nx: int, ny: int, scheme: int = WENOZ, rk: int = 2,
                 cfl: float = 0.6, seed: int = 0, t_end: float | None = None):
        L = lib()
        self.case = Case()
        L.orc_case_setup(testcase, seed, C.byref(self.case))
        self.grid = Grid()
        L.orc_grid_setup(C.byref(self.case), nx, ny, scheme, C.byref(self.grid))
        self.nx, self.ny, self.rk, self.cfl = nx, ny, rk, cfl
        self.t_end = self.case.t_end if t_end is None else t_end
        self.now = 0.0
        shape = (4, nx + 2 * NG, ny + 2 * NG)
        self.U = np.zeros(shape)
        self.Un = np.zeros(shape)
        self.rhs = np.zeros(shape)
        self.special = np.zeros(L.orc_special_table_size(C.byref(self.grid)))
        L.orc_special_table(C.byref(self.case), C.byref(self.grid), _p(self.special))
        self.grid.special = _p(self.special)
        L.orc_initial_state(C.byref(self.case), C.byref(self.grid), _p(self.U))

    # interior view helpers
    def interior(self, A: np.ndarray | None = None) -> np.ndarray:
        A = self.U if A is None else A
        return A[:, NG:NG + self.nx, NG:NG + self.ny].copy()

    def set_interior(self, V: np.ndarray) -> None:
        self.U[:, NG:NG + self.nx, NG:NG + self.ny] = V

    def fill_boundary(self) -> None:
        lib().orc_fill_boundary(C.byref(self.grid), _p(self.U))

    def assemble_rhs(self) -> np.ndarray:
        lib().orc_assemble_rhs(C.byref(self.grid), _p(self.U), _p(self.rhs))
        return self.interior(self.rhs)

    def calc_dt(self) -> float:
        dt = np.zeros(1)
        if lib().orc_calc_dt(C.byref(self.grid), _p(self.U), self.cfl, self.now, self.t_end, _p(dt)):
            raise FloatingPointError("time step is NaN")
        return float(dt[0])

    def rk_step(self, dt: float) -> None:
        lib().orc_rk_step(C.byref(self.grid), self.rk, _p(self.U), _p(self.Un), _p(self.rhs), dt)

    def run(self, max_steps: int = -1) -> tuple[int, np.ndarray]:
        now = C.c_double(self.now)
        steps = C.c_long(0)
        cap = max_steps if max_steps >= 0 else 1 << 20
        dts = np.zeros(min(cap, 1 << 20) + 1)
        rc = lib().orc_run(C.byref(self.grid), self.rk, self.cfl, _p(self.U), _p(self.Un), _p(self.rhs),
                           C.byref(now), self.t_end, max_steps, C.byref(steps), _p(dts), len(dts))
        self.now = now.value
        if rc:
            raise FloatingPointError("time step is NaN")
        return steps.value, dts[:steps.value].copy()

    def error_norms(self, t: float | None = None) -> np.ndarray:
        out = np.zeros(3)
        lib().orc_error_norms(C.byref(self.grid), _p(self.U), self.now if t is None else t, _p(out))
        return out

    def cell_features(self) -> np.ndarray:
        """(NX*NY, 50) float32 indicator features of the current state (fills ghosts)."""
        self.fill_boundary()
        out = np.zeros((self.nx * self.ny, 50), dtype=np.float32)
        lib().orc_cell_features(C.byref(self.grid), _p(self.U), out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def cell_labels(self, deviation: float = 1e-2) -> np.ndarray:
        """(NX*NY,) uint8 WENO-Z weight-deviation labels of the current state
        (1 where a face of the node deviates by more than `deviation`)."""
        self.fill_boundary()
        out = np.zeros(self.nx * self.ny, dtype=np.uint8)
        lib().orc_cell_labels_at(C.byref(self.grid), _p(self.U), out.ctypes.data_as(C.POINTER(C.c_ubyte)),
                                 deviation)
        return out

    def conservation_sums(self) -> np.ndarray:
        out = np.zeros(4)
        lib().orc_conservation_sums(C.byref(self.grid), _p(self.U), _p(out))
        return out


def ref_available() -> bool:
    return os.path.exists(REF_BIN)


class Slab:
    """One rank's x-slab of a Problem, as the reference's MPI ranks hold it
    (src/WENOFD.cpp:36-70): nodes [start, start + count) of the x interior
    with 4 ghost columns each side, all y nodes.  Used by the multi-rank
    tests as the per-rank compute; the ghost exchange between ranks is the
    product's (wenofd.partition)."""

    def __init__(self, prob: "Problem", start: int, count: int):
        self.prob, self.start, self.count = prob, start, count
        self.grid = Grid()
        C.memmove(C.byref(self.grid), C.byref(prob.grid), C.sizeof(Grid))
        self.grid.nx = count
        nxt_g, nyt = prob.nx + 2 * NG, prob.ny + 2 * NG
        cols = slice(start, start + count + 2 * NG)
        ytab = prob.special[:8 * nxt_g].reshape(8, nxt_g)[:, cols]
        self.special = np.concatenate([ytab.reshape(-1), prob.special[8 * nxt_g:8 * nxt_g + 8 * nyt]])
        self.grid.special = _p(self.special)
        self.U = np.ascontiguousarray(prob.U[:, cols, :])
        self.Un = np.zeros_like(self.U)
        self.rhs = np.zeros_like(self.U)

    def interior(self, A: np.ndarray | None = None) -> np.ndarray:
        A = self.U if A is None else A
        return A[:, NG:NG + self.count, NG:NG + self.prob.ny].copy()

    def fill_boundary(self, left_edge: bool, right_edge: bool) -> None:
        lib().orc_fill_boundary_slab(C.byref(self.grid), _p(self.U), int(left_edge), int(right_edge))

    def assemble_rhs(self) -> np.ndarray:
        lib().orc_assemble_rhs_ghosted(C.byref(self.grid), _p(self.U), _p(self.rhs))
        return self.interior(self.rhs)

    def local_dt(self, cfl: float, now: float, t_end: float) -> float:
        dt = np.zeros(1)
        lib().orc_calc_dt(C.byref(self.grid), _p(self.U), cfl, now, t_end, _p(dt))
        return float(dt[0])

