"""ctypes view of the C oracle (TEST INFRASTRUCTURE ONLY).

Wraps ``libspc_oracle.so`` (built from ``spc_oracle.c``) with numpy arrays in
the reference's array-of-structures layout [x0, y0, phi0, x1, ...].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_oracle

EULER, SRK, RK4, EULER_PTR = 0, 1, 2, 3

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle.build_restatement()
        L = C.CDLL(path)
        P = C.c_void_p
        D = C.c_double
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        lp = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.c_int, D, D, D, D, D, D]
        L.orc_destroy.argtypes = [P]
        L.orc_num_cells.argtypes = [P]
        L.orc_uses_cell_list.argtypes = [P]
        L.orc_clamped_cells.argtypes = [P]
        L.orc_clamped_cells.restype = C.c_longlong
        L.orc_min_image.argtypes = [P, D, D, D, D, C.POINTER(D), C.POINTER(D)]
        L.orc_wrap_point.argtypes = [P, D, D, C.POINTER(D), C.POINTER(D)]
        L.orc_wrap_state.argtypes = [P, dp]
        L.orc_rhs_rk.argtypes = [P, dp, dp, dp, D, D, C.c_void_p]
        L.orc_rhs_srk.argtypes = [P, dp, dp, dp, C.c_void_p]
        L.orc_step_euler.argtypes = [P, dp, D, D, dp, C.c_void_p]
        L.orc_step_euler_ptr.argtypes = [P, dp, D, D, dp]
        L.orc_step_srk.argtypes = [P, dp, D, D, dp, C.c_void_p]
        L.orc_step_rk4.argtypes = [P, dp, D, D]
        L.orc_run.restype = D
        L.orc_run.argtypes = [P, C.c_int, dp, D, D, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_get_rk4_buffers.argtypes = [P, dp]
        L.orc_set_rk4_buffers.argtypes = [P, dp]
        L.orc_neighbour_lists.restype = C.c_longlong
        L.orc_neighbour_lists.argtypes = [P, dp, lp, ip, C.c_longlong]
        L.orc_order_params.argtypes = [P, dp, C.POINTER(D), C.POINTER(D),
                                       C.POINTER(C.c_float), C.POINTER(C.c_float),
                                       C.POINTER(D)]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
        L.orc_va_create.restype = P
        L.orc_va_create.argtypes = [C.c_int, D, D, D, D, D, D, D, D, D]
        L.orc_va_rhs_rk.argtypes = [P, dp, dp, dp, D, D, C.c_void_p]
        L.orc_va_rhs_srk.argtypes = [P, dp, dp, dp, C.c_void_p]
        L.orc_va_run.restype = D
        L.orc_va_run.argtypes = [P, C.c_int, dp, D, D, C.c_int, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleSystem:
    """One ChimeraSystem with its steppers' persistent buffers."""

    def __init__(self, n, L, v0, sigma, rho, alpha, D_phi):
        self.n = int(n)
        self.h = lib().orc_create(self.n, L, v0, sigma, rho, alpha, D_phi)
        if not self.h:
            raise ValueError("bad oracle parameters")

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_cells(self) -> int:
        return lib().orc_num_cells(self.h)

    @property
    def uses_cell_list(self) -> bool:
        return bool(lib().orc_uses_cell_list(self.h))

    @property
    def clamped_cells(self) -> int:
        return lib().orc_clamped_cells(self.h)

    def min_image(self, xi, yi, xj, yj):
        dx, dy = C.c_double(), C.c_double()
        lib().orc_min_image(self.h, xi, yi, xj, yj, C.byref(dx), C.byref(dy))
        return dx.value, dy.value

    def wrap_point(self, x, y):
        a, b = C.c_double(), C.c_double()
        lib().orc_wrap_point(self.h, x, y, C.byref(a), C.byref(b))
        return a.value, b.value

    def rhs_rk(self, state, k_prev, k_next, k_coef, dt, with_counts=False):
        counts = np.zeros(self.n, np.int32) if with_counts else None
        lib().orc_rhs_rk(self.h, state, k_prev, k_next, k_coef, dt, _ptr(counts))
        return counts

    def rhs_srk(self, state, with_counts=False):
        d = np.zeros(3 * self.n)
        a = np.zeros(2 * self.n)
        counts = np.zeros(self.n, np.int32) if with_counts else None
        lib().orc_rhs_srk(self.h, state, d, a, _ptr(counts))
        return d, a, counts

    def run(self, stepper, state, t0, dt, nsteps, noise=None, omega=None):
        noise = None if noise is None else np.ascontiguousarray(noise, np.float64)
        omega = None if omega is None else np.ascontiguousarray(omega, np.float64)
        return lib().orc_run(self.h, stepper, state, t0, dt, nsteps, _ptr(noise), _ptr(omega))

    def get_rk4_buffers(self):
        out = np.zeros(12 * self.n)
        lib().orc_get_rk4_buffers(self.h, out)
        return out

    def set_rk4_buffers(self, buf):
        lib().orc_set_rk4_buffers(self.h, np.ascontiguousarray(buf, np.float64))

    def neighbour_lists(self, stage_state):
        offsets = np.zeros(self.n + 1, np.int64)
        cap = 0
        idx = np.zeros(1, np.int32)
        total = lib().orc_neighbour_lists(self.h, stage_state, offsets, idx, cap)
        idx = np.zeros(max(total, 1), np.int32)
        lib().orc_neighbour_lists(self.h, stage_state, offsets, idx, total)
        return offsets, idx[:total]

    def order_params(self, state):
        R, psi, Rl = C.c_double(), C.c_double(), C.c_double()
        Rf, pf = C.c_float(), C.c_float()
        lib().orc_order_params(self.h, state, C.byref(R), C.byref(psi), C.byref(Rf),
                               C.byref(pf), C.byref(Rl))
        return {"R": R.value, "psi": psi.value, "R_f32": Rf.value, "psi_f32": pf.value,
                "R_local": Rl.value}


class OracleVortexArrays(OracleSystem):
    """One VortexArraysSystemPtr with its steppers' persistent buffers."""

    def __init__(self, n, L, velocity, mu_plus, mu_minus, xi_a, xi_r, D_phi, kappa, rho):
        self.n = int(n)
        self.h = lib().orc_va_create(self.n, L, velocity, mu_plus, mu_minus, xi_a, xi_r, D_phi,
                                     kappa, rho)
        if not self.h:
            raise ValueError("bad oracle parameters")

    def rhs_rk(self, state, k_prev, k_next, k_coef, dt, with_counts=False):
        counts = np.zeros(3 * self.n, np.int32) if with_counts else None
        lib().orc_va_rhs_rk(self.h, state, k_prev, k_next, k_coef, dt, _ptr(counts))
        return counts

    def rhs_srk(self, state, with_counts=False):
        d = np.zeros(3 * self.n)
        a = np.zeros(2 * self.n)
        counts = np.zeros(3 * self.n, np.int32) if with_counts else None
        lib().orc_va_rhs_srk(self.h, state, d, a, _ptr(counts))
        return d, a, counts

    def run(self, stepper, state, t0, dt, nsteps, noise=None, omega=None):
        noise = None if noise is None else np.ascontiguousarray(noise, np.float64)
        return lib().orc_va_run(self.h, stepper, state, t0, dt, nsteps, _ptr(noise))


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(v) for v in o]
