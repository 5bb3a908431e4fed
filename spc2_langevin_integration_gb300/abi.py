"""ctypes binding of the C-ABI in include/spc_gb300.h.

This is the reference-facing boundary as a Python caller sees it (the C++
adapters in ``host/`` are the drop-in for the reference's own C++ callers).
The library is the in-tree ``_build/libspc_gb300.so``; if it is missing or
fails to load, :func:`lib` raises - there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

MODEL_CHIMERA, MODEL_VORTEX, MODEL_VORTEX_ARRAYS = 0, 1, 2
STEPPER_EULER, STEPPER_SRK, STEPPER_RK4, STEPPER_EULER_PTR = 0, 1, 2, 3
NEIGHBOUR_CELL, NEIGHBOUR_VERLET = 0, 1
PRECISION_FP64, PRECISION_FP32C, PRECISION_FP32X = 0, 1, 2
FLAG_EXACT_ALL = 0x1
TUNE_SPARSE_BELOW = 1
TUNE_VERLET_ROW_LIMIT = 2
TUNE_TILE_SPLIT = 3
TUNE_CELL_UNITS = 4
TUNE_SUBCELLS = 5

SPC_OK = 0
ERRORS = {
    -1: "SPC_ERR_INVALID", -2: "SPC_ERR_CUDA", -3: "SPC_ERR_NOMEM", -4: "SPC_ERR_STATE",
    -5: "SPC_ERR_NOISE", -6: "SPC_ERR_DEVICE", -7: "SPC_ERR_CAPACITY",
}


class SpcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("stepper", C.c_int32), ("neighbour", C.c_int32),
        ("precision", C.c_int32), ("L", C.c_double), ("v0", C.c_double),
        ("sigma", C.c_double), ("rho", C.c_double), ("alpha", C.c_double),
        ("D_phi", C.c_double), ("rho_0", C.c_double), ("skin", C.c_double),
        ("seed", C.c_uint64), ("system_id", C.c_uint32), ("flags", C.c_uint32),
        ("mu_plus", C.c_double), ("mu_minus", C.c_double), ("xi_a", C.c_double),
        ("xi_r", C.c_double), ("kappa", C.c_double),
    ]


class BatchConfig(C.Structure):
    _fields_ = [
        ("stepper", C.c_int32), ("precision", C.c_int32), ("max_systems", C.c_int32),
        ("pad", C.c_int32), ("max_particles", C.c_int64), ("max_cells", C.c_int64),
    ]


class Tuning(C.Structure):
    """spc_tuning: one tuning candidate and its measured cost."""
    _fields_ = [
        ("neighbour", C.c_int32), ("tile_split", C.c_int32), ("skin", C.c_double),
        ("sparse_below", C.c_double), ("ms_per_step", C.c_double), ("cell_units", C.c_int32),
        ("subcells", C.c_int32),
    ]

    def as_dict(self):
        return {"neighbour": "verlet" if self.neighbour == NEIGHBOUR_VERLET else "cell",
                "tile_split": self.tile_split, "skin": self.skin,
                "sparse_below": self.sparse_below, "cell_units": self.cell_units,
                "subcells": self.subcells, "ms_per_step": self.ms_per_step}


_lib = None


def library_path() -> str:
    return _build.LIB


def lib() -> C.CDLL:
    """Load the CUDA library (building it first when nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not _build.up_to_date():
        try:
            _build.build_library()
        except Exception as e:  # no nvcc here: only an existing build can load
            if not os.path.exists(path):
                raise RuntimeError(f"CUDA library missing and could not be built: {e}") from e
    L = C.CDLL(path)
    H = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.spc_abi_version.restype = C.c_int
    L.spc_last_error.restype = C.c_char_p
    L.spc_last_error.argtypes = [H]
    L.spc_create.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(H)]
    L.spc_destroy.argtypes = [H]
    L.spc_get_params.argtypes = [H, C.POINTER(Params), C.POINTER(C.c_int32)]
    for f in ("spc_upload_state", "spc_download_state", "spc_upload_omega",
              "spc_download_rk4_buffers", "spc_upload_rk4_buffers"):
        getattr(L, f).argtypes = [H, C.c_void_p]
    L.spc_step.argtypes = [H, dp, C.c_double, C.c_int32]
    L.spc_step_graph.argtypes = [H, dp, C.c_double, C.c_int32]
    L.spc_get_step_counter.argtypes = [H, C.POINTER(C.c_uint64)]
    L.spc_set_step_counter.argtypes = [H, C.c_uint64]
    L.spc_inject_noise.argtypes = [H, C.c_void_p, C.c_int64]
    L.spc_clear_noise.argtypes = [H]
    L.spc_export_noise.argtypes = [H, C.c_uint64, C.c_int32, C.c_void_p]
    L.spc_noise_per_particle.argtypes = [H]
    L.spc_rhs_rk.argtypes = [H, C.c_void_p, C.c_double, C.c_double, C.c_void_p]
    L.spc_rhs_srk.argtypes = [H, C.c_void_p, C.c_void_p]
    L.spc_neighbours.argtypes = [H, C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    L.spc_order_params.argtypes = [H, dp, dp, dp]
    L.spc_diagnostics.argtypes = [H, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64)]
    L.spc_synchronize.argtypes = [H]
    L.spc_stream.restype = C.c_void_p
    L.spc_stream.argtypes = [H]
    L.spc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32)]
    L.spc_profile_steps.argtypes = [H, C.c_double, C.c_int32, dp, C.c_int32]
    L.spc_batch_footprint.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]
    L.spc_batch_create.argtypes = [C.POINTER(BatchConfig), C.POINTER(H)]
    L.spc_batch_destroy.argtypes = [H]
    L.spc_batch_last_error.restype = C.c_char_p
    L.spc_batch_last_error.argtypes = [H]
    L.spc_batch_admit.argtypes = [H, C.POINTER(Params), C.c_int32, C.c_void_p, C.c_void_p,
                                  C.c_int64, C.POINTER(C.c_int32)]
    L.spc_batch_release.argtypes = [H, C.c_int32]
    L.spc_batch_step.argtypes = [H, C.c_double, C.c_int32]
    L.spc_batch_step_graph.argtypes = [H, C.c_double, C.c_int32]
    L.spc_batch_download.argtypes = [H, C.c_int32, C.c_void_p]
    L.spc_batch_upload.argtypes = [H, C.c_int32, C.c_void_p]
    L.spc_batch_status.argtypes = [H, C.c_int32, C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]
    L.spc_batch_usage.argtypes = [H, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int32)]
    L.spc_batch_order_params.argtypes = [H, C.c_int32, dp, dp]
    L.spc_batch_order_params_all.argtypes = [H, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.spc_batch_synchronize.argtypes = [H]
    L.spc_batch_stream.restype = C.c_void_p
    L.spc_batch_stream.argtypes = [H]
    L.spc_batch_profile_steps.argtypes = [H, C.c_double, C.c_int32, dp, C.c_int32]
    L.spc_set_tuning.argtypes = [H, C.c_int32, C.c_double]
    L.spc_get_tuning.argtypes = [H, C.c_int32, dp]
    L.spc_batch_set_tuning.argtypes = [H, C.c_int32, C.c_double]
    L.spc_batch_get_tuning.argtypes = [H, C.c_int32, dp]
    L.spc_autotune.argtypes = [C.POINTER(Params), C.c_int32, C.c_void_p, C.c_void_p, C.c_double,
                               C.c_int32, C.POINTER(Params), dp, dp, C.c_int32,
                               C.POINTER(C.c_int32)]
    L.spc_autotune_ex.argtypes = [C.POINTER(Params), C.c_int32, C.c_void_p, C.c_void_p, C.c_double,
                                  C.c_int32, C.POINTER(Tuning), C.c_int32, C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32)]
    L.spc_retune.argtypes = [H, C.c_double, C.c_int32, C.POINTER(Tuning), C.c_int32,
                             C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.spc_batch_retune.argtypes = [H, C.c_double, C.c_int32, C.POINTER(Tuning), C.c_int32,
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.spc_prepare_graph.argtypes = [H, C.c_double, C.c_int32]
    L.spc_graph_nodes.argtypes = [H, C.POINTER(C.c_int64)]
    L.spc_run.argtypes = [H, dp, C.c_double, C.c_int64, C.c_int32, C.c_void_p, OBSERVE_FN,
                          C.c_void_p, C.POINTER(C.c_int64)]
    L.spc_run_graph_nodes.argtypes = [H, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    L.spc_check_division.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
    L.spc_check_sincos.argtypes = [C.c_int64, C.c_void_p, C.POINTER(C.c_int64)]
    L.spc_alloc_pinned.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    L.spc_free_pinned.argtypes = [C.c_void_p]
    _lib = L
    return L


def check_division(a, b) -> int:
    """Pairs (a[i], b[i]) whose quotient differs in any bit between the
    correctly rounded division and the FP64 kernels' reciprocal form, on the
    device (spc_check_division)."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    if a.shape != b.shape:
        raise ValueError("a and b differ in shape")
    bad = C.c_int64()
    L = lib()
    rc = L.spc_check_division(a.size, _ptr(a), _ptr(b), C.byref(bad))
    if rc != 0:
        raise SpcError(rc, L.spc_last_error(None).decode())
    return bad.value


def check_sincos(x) -> int:
    """Values whose sin / cos from separate launches differ in any bit from
    one sincos, on the device (spc_check_sincos)."""
    x = np.ascontiguousarray(x, np.float64)
    bad = C.c_int64()
    L = lib()
    rc = L.spc_check_sincos(x.size, _ptr(x), C.byref(bad))
    if rc != 0:
        raise SpcError(rc, L.spc_last_error(None).decode())
    return bad.value


# int (*)(void *user, int64_t step, double t, const double *aos3n)
OBSERVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_double))


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _f64(a, n: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def make_params(*, L, v0, sigma=0.0, rho, alpha=0.0, D_phi, rho_0=1.0, model=MODEL_CHIMERA,
                stepper=STEPPER_EULER, neighbour=NEIGHBOUR_CELL, precision=PRECISION_FP64,
                skin=0.05, seed=0, system_id=0, flags=0, mu_plus=0.0, mu_minus=0.0, xi_a=0.0,
                xi_r=0.0, kappa=0.0) -> Params:
    return Params(model, stepper, neighbour, precision, L, v0, sigma, rho, alpha, D_phi, rho_0,
                  skin, seed, system_id, flags, mu_plus, mu_minus, xi_a, xi_r, kappa)


def make_va_params(*, L, velocity, mu_plus, mu_minus, xi_a, xi_r, D_phi, kappa, rho,
                   stepper=STEPPER_SRK, seed=0, system_id=0, flags=0) -> Params:
    """VortexArraysSystemPtr parameters in the reference's ctor order."""
    return make_params(L=L, v0=velocity, rho=rho, D_phi=D_phi, model=MODEL_VORTEX_ARRAYS,
                       stepper=stepper, seed=seed, system_id=system_id, flags=flags,
                       mu_plus=mu_plus, mu_minus=mu_minus, xi_a=xi_a, xi_r=xi_r, kappa=kappa)


class System:
    """One particle system on the GPU (a handle of the C-ABI)."""

    def __init__(self, n: int, params: Params):
        self._L = lib()
        self.n = int(n)
        self.params = params
        h = C.c_void_p()
        self._check(self._L.spc_create(C.byref(params), self.n, C.byref(h)), None)
        self.h = h
        self.t = 0.0

    def _check(self, rc: int, h=None):
        if rc != SPC_OK:
            msg = self._L.spc_last_error(h if h is not None else getattr(self, "h", None))
            raise SpcError(rc, (msg or b"").decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.spc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state ---------------------------------------------------------------
    def upload_state(self, aos):
        a = _f64(aos, 3 * self.n)
        self._check(self._L.spc_upload_state(self.h, _ptr(a)), self.h)

    def download_state(self, out=None) -> np.ndarray:
        out = np.empty(3 * self.n) if out is None else out
        self._check(self._L.spc_download_state(self.h, _ptr(out)), self.h)
        return out

    def upload_omega(self, omega):
        a = _f64(omega, self.n)
        self._check(self._L.spc_upload_omega(self.h, _ptr(a)), self.h)

    def download_rk4_buffers(self) -> np.ndarray:
        out = np.empty(12 * self.n)
        self._check(self._L.spc_download_rk4_buffers(self.h, _ptr(out)), self.h)
        return out

    def upload_rk4_buffers(self, buf):
        a = _f64(buf, 12 * self.n)
        self._check(self._L.spc_upload_rk4_buffers(self.h, _ptr(a)), self.h)

    # stepping ------------------------------------------------------------
    def step(self, dt: float, nsteps: int, graph: bool = False) -> float:
        t = C.c_double(self.t)
        f = self._L.spc_step_graph if graph else self._L.spc_step
        self._check(f(self.h, C.byref(t), dt, int(nsteps)), self.h)
        self.t = t.value
        return self.t

    def prepare_graph(self, dt: float, nsteps: int):
        """spc_prepare_graph: capture the step graph without running it."""
        self._check(self._L.spc_prepare_graph(self.h, dt, int(nsteps)), self.h)

    def run(self, dt: float, nsteps: int, period: int = 1, observe=None, fn=None) -> int:
        """The engine loop with its observers on the device (spc_run): after
        step k (1-based) with observe[k % period] set, fn(k, t, state) gets a
        copy of the AoS state; a true return from fn stops the run.  Returns
        the number of steps taken."""
        t = C.c_double(self.t)
        done = C.c_int64()
        obs = None
        cb = OBSERVE_FN()
        errors = []
        if fn is not None:
            mask = np.ones(period, np.uint8) if observe is None else np.asarray(observe, np.uint8)
            if mask.size != period:
                raise ValueError(f"observe needs {period} entries")
            obs = np.ascontiguousarray(mask)
            n3 = 3 * self.n

            def tramp(_user, step, tt, state):
                try:
                    return 1 if fn(int(step), float(tt), np.ctypeslib.as_array(state, (n3,)).copy()) else 0
                except BaseException as e:  # raised again after the C call returns
                    errors.append(e)
                    return 1
            cb = OBSERVE_FN(tramp)
        rc = self._L.spc_run(self.h, C.byref(t), float(dt), int(nsteps), int(period),
                             _ptr(obs) if obs is not None else None, cb, None, C.byref(done))
        self.t = t.value
        if errors:
            raise errors[0]
        self._check(rc, self.h)
        return done.value

    def run_graph_nodes(self) -> tuple[int, int]:
        """(kernel nodes, steps) of spc_run's captured chunk graph."""
        v, st = C.c_int64(), C.c_int32()
        self._check(self._L.spc_run_graph_nodes(self.h, C.byref(v), C.byref(st)), self.h)
        return v.value, st.value

    @property
    def step_counter(self) -> int:
        v = C.c_uint64()
        self._check(self._L.spc_get_step_counter(self.h, C.byref(v)), self.h)
        return v.value

    @step_counter.setter
    def step_counter(self, v: int):
        self._check(self._L.spc_set_step_counter(self.h, int(v)), self.h)

    @property
    def noise_per_particle(self) -> int:
        return self._L.spc_noise_per_particle(self.h)

    def inject_noise(self, normals):
        a = np.ascontiguousarray(normals, dtype=np.float64)
        self._keep_noise = a
        self._check(self._L.spc_inject_noise(self.h, _ptr(a), a.size), self.h)

    def clear_noise(self):
        self._check(self._L.spc_clear_noise(self.h), self.h)

    def export_noise(self, first_step: int, nsteps: int) -> np.ndarray:
        out = np.empty(max(nsteps * self.n * self.noise_per_particle, 1))
        self._check(self._L.spc_export_noise(self.h, int(first_step), int(nsteps), _ptr(out)),
                    self.h)
        return out[: nsteps * self.n * self.noise_per_particle]

    # parity hooks --------------------------------------------------------
    def rhs_rk(self, k_prev, k_coef: float, dt: float, k_next_init=None) -> np.ndarray:
        kp = _f64(k_prev, 3 * self.n)
        kn = np.zeros(3 * self.n) if k_next_init is None else _f64(k_next_init, 3 * self.n).copy()
        self._check(self._L.spc_rhs_rk(self.h, _ptr(kp), k_coef, dt, _ptr(kn)), self.h)
        return kn

    def rhs_srk(self):
        d = np.empty(3 * self.n)
        a = np.empty(2 * self.n)
        self._check(self._L.spc_rhs_srk(self.h, _ptr(d), _ptr(a)), self.h)
        return d, a

    def neighbour_counts(self) -> np.ndarray:
        """n_i of every particle (in the order of the state), without the lists."""
        counts = np.empty(self.n, np.int32)
        total = C.c_int64()
        self._check(self._L.spc_neighbours(self.h, _ptr(counts), None, 0, C.byref(total)), self.h)
        return counts

    def neighbours(self):
        counts = np.empty(self.n, np.int32)
        total = C.c_int64()
        self._check(self._L.spc_neighbours(self.h, _ptr(counts), None, 0, C.byref(total)), self.h)
        idx = np.empty(max(total.value, 1), np.int32)
        self._check(self._L.spc_neighbours(self.h, _ptr(counts), _ptr(idx), idx.size,
                                           C.byref(total)), self.h)
        offsets = np.zeros(self.n + 1, np.int64)
        np.cumsum(counts, out=offsets[1:])
        return offsets, idx[: total.value]

    def order_params(self):
        R, psi, Rl = C.c_double(), C.c_double(), C.c_double()
        self._check(self._L.spc_order_params(self.h, C.byref(R), C.byref(psi), C.byref(Rl)),
                    self.h)
        return {"R": R.value, "psi": psi.value, "R_local": Rl.value}

    def diagnostics(self):
        c, v, e = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self._L.spc_diagnostics(self.h, C.byref(c), C.byref(v), C.byref(e)), self.h)
        return {"clamped_cells": c.value, "verlet_rebuilds": v.value, "error_word": e.value}

    def graph_nodes(self) -> int:
        v = C.c_int64()
        self._check(self._L.spc_graph_nodes(self.h, C.byref(v)), self.h)
        return v.value

    def retune(self, dt: float, trial_steps: int = 10):
        """spc_retune: re-time the kernel choices on the current state (which is
        left as it was) and keep the fastest.  Returns (candidates, best index)."""
        cands = (Tuning * 16)()
        cnt, best = C.c_int32(), C.c_int32()
        self._check(self._L.spc_retune(self.h, dt, int(trial_steps), cands, 16, C.byref(cnt),
                                       C.byref(best)), self.h)
        return [cands[k].as_dict() for k in range(min(cnt.value, 16))], best.value

    def set_tuning(self, key: int, value: float):
        self._check(self._L.spc_set_tuning(self.h, int(key), float(value)), self.h)

    def get_tuning(self, key: int) -> float:
        v = C.c_double()
        self._check(self._L.spc_get_tuning(self.h, int(key), C.byref(v)), self.h)
        return v.value

    def profile_steps(self, dt: float, nsteps: int) -> dict:
        out = (C.c_double * 6)()
        self._check(self._L.spc_profile_steps(self.h, dt, int(nsteps), out, 6), self.h)
        keys = ("stage", "sort", "gather", "pass1", "pass2", "step")
        return {k: out[i] for i, k in enumerate(keys)}

    def synchronize(self):
        self._check(self._L.spc_synchronize(self.h), self.h)

    @property
    def stream(self) -> int:
        return self._L.spc_stream(self.h)


def philox4x32_10(ctr, key):
    """Philox4x32-10 evaluated on the device."""
    L = lib()
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (C.c_uint32 * 4)()
    rc = L.spc_philox4x32_10(c, k, o)
    if rc != SPC_OK:
        raise SpcError(rc, (L.spc_last_error(None) or b"").decode())
    return [int(v) for v in o]


def header_functions() -> list[str]:
    """Names of the functions include/spc_gb300.h declares."""
    import re
    path = os.path.join(_build.ROOT, "include", "spc_gb300.h")
    text = open(path).read()
    return sorted(set(re.findall(r"^\s*(?:int|void \*|const char \*)\s*(spc_\w+)\(", text, re.M)))


def footprint(stepper: int, precision: int):
    """(bytes per pool particle, bytes per cell) a batch reserves."""
    bp, bc = C.c_int64(), C.c_int64()
    lib().spc_batch_footprint(stepper, precision, C.byref(bp), C.byref(bc))
    return bp.value, bc.value


def cells_of(L: float, rho: float) -> int:
    """Cells a system occupies in a batch: int(L/rho)^2, or 1 when rho > L/4."""
    return 1 if not (rho <= 0.25 * L) else int(L / rho) ** 2


class Batch:
    """Many systems advanced together (the C-ABI's spc_batch)."""

    def __init__(self, stepper: int, precision: int, max_systems: int, max_particles: int,
                 max_cells: int):
        self._L = lib()
        self.stepper, self.precision = stepper, precision
        cfg = BatchConfig(stepper, precision, int(max_systems), 0, int(max_particles),
                          int(max_cells))
        h = C.c_void_p()
        rc = self._L.spc_batch_create(C.byref(cfg), C.byref(h))
        if rc != SPC_OK:
            raise SpcError(rc, (self._L.spc_batch_last_error(None) or b"").decode())
        self.h = h
        self.n = {}
        self.capacity = {"particles": int(max_particles), "cells": int(max_cells),
                         "systems": int(max_systems)}

    def _check(self, rc: int):
        if rc != SPC_OK:
            raise SpcError(rc, (self._L.spc_batch_last_error(self.h) or b"").decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.spc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def admit(self, n: int, params: Params, state, omega=None, steps: int = -1) -> int:
        st = _f64(state, 3 * n)
        om = None if omega is None else _f64(omega, n)
        slot = C.c_int32()
        self._check(self._L.spc_batch_admit(self.h, C.byref(params), int(n), _ptr(st),
                                            None if om is None else _ptr(om), int(steps),
                                            C.byref(slot)))
        self.n[slot.value] = int(n)
        return slot.value

    def release(self, slot: int):
        self._check(self._L.spc_batch_release(self.h, int(slot)))
        self.n.pop(slot, None)

    def step(self, dt: float, nsteps: int, graph: bool = False):
        f = self._L.spc_batch_step_graph if graph else self._L.spc_batch_step
        self._check(f(self.h, dt, int(nsteps)))

    def download(self, slot: int, out=None) -> np.ndarray:
        out = np.empty(3 * self.n[slot]) if out is None else out
        self._check(self._L.spc_batch_download(self.h, int(slot), _ptr(out)))
        return out

    def upload(self, slot: int, state):
        st = _f64(state, 3 * self.n[slot])
        self._check(self._L.spc_batch_upload(self.h, int(slot), _ptr(st)))

    def status(self, slot: int):
        done, rem = C.c_uint64(), C.c_int64()
        self._check(self._L.spc_batch_status(self.h, int(slot), C.byref(done), C.byref(rem)))
        return done.value, rem.value

    def usage(self):
        p, c, s = C.c_int64(), C.c_int64(), C.c_int32()
        self._check(self._L.spc_batch_usage(self.h, C.byref(p), C.byref(c), C.byref(s)))
        return {"particles": p.value, "cells": c.value, "systems": s.value}

    def order_params(self, slot: int):
        R, psi = C.c_double(), C.c_double()
        self._check(self._L.spc_batch_order_params(self.h, int(slot), C.byref(R), C.byref(psi)))
        return {"R": R.value, "psi": psi.value}

    def order_params_all(self, cap: int, local: bool = True):
        """R, psi and (local=True) R_local of slots [0, cap) as float64
        arrays, NaN where a slot holds no system."""
        R, psi = np.empty(cap), np.empty(cap)
        Rl = np.empty(cap) if local else None
        self._check(self._L.spc_batch_order_params_all(self.h, int(cap), _ptr(R), _ptr(psi),
                                                       _ptr(Rl) if local else None))
        return {"R": R, "psi": psi, "R_local": Rl}

    def synchronize(self):
        self._check(self._L.spc_batch_synchronize(self.h))

    def retune(self, dt: float, trial_steps: int = 10):
        """spc_batch_retune (see System.retune)."""
        cands = (Tuning * 16)()
        cnt, best = C.c_int32(), C.c_int32()
        self._check(self._L.spc_batch_retune(self.h, dt, int(trial_steps), cands, 16, C.byref(cnt),
                                             C.byref(best)))
        return [cands[k].as_dict() for k in range(min(cnt.value, 16))], best.value

    def set_tuning(self, key: int, value: float):
        self._check(self._L.spc_batch_set_tuning(self.h, int(key), float(value)))

    def get_tuning(self, key: int) -> float:
        v = C.c_double()
        self._check(self._L.spc_batch_get_tuning(self.h, int(key), C.byref(v)))
        return v.value

    def profile_steps(self, dt: float, nsteps: int) -> dict:
        out = (C.c_double * 6)()
        self._check(self._L.spc_batch_profile_steps(self.h, dt, int(nsteps), out, 6))
        keys = ("stage", "sort", "gather", "pass1", "pass2", "step")
        return {k: out[i] for i, k in enumerate(keys)}

    @property
    def stream(self) -> int:
        return self._L.spc_batch_stream(self.h)


def autotune(n: int, params: Params, state, omega=None, dt: float = 0.01, trial_steps: int = 20):
    """Time the neighbour-method candidates on this state (spc_autotune) and
    return (best params, sparse_below tuning, per-candidate ms per step)."""
    L = lib()
    st = _f64(state, 3 * n)
    om = None if omega is None else _f64(omega, n)
    best = Params()
    sb = C.c_double()
    ms = (C.c_double * 16)()
    cnt = C.c_int32()
    rc = L.spc_autotune(C.byref(params), int(n), _ptr(st), None if om is None else _ptr(om), dt,
                        int(trial_steps), C.byref(best), C.byref(sb), ms, 16, C.byref(cnt))
    if rc != SPC_OK:
        raise SpcError(rc, (L.spc_last_error(None) or b"").decode())
    return best, sb.value, [ms[k] for k in range(min(cnt.value, 16))]


def autotune_ex(n: int, params: Params, state, omega=None, dt: float = 0.01, trial_steps: int = 20):
    """spc_autotune_ex: every tuning candidate timed on this state (neighbour
    method, skin, kernel choice, CTAs per cell).  Returns (candidates, best)."""
    L = lib()
    st = _f64(state, 3 * n)
    om = None if omega is None else _f64(omega, n)
    cands = (Tuning * 32)()
    cnt, best = C.c_int32(), C.c_int32()
    rc = L.spc_autotune_ex(C.byref(params), int(n), _ptr(st), None if om is None else _ptr(om), dt,
                           int(trial_steps), cands, 32, C.byref(cnt), C.byref(best))
    if rc != SPC_OK:
        raise SpcError(rc, (L.spc_last_error(None) or b"").decode())
    return [cands[k].as_dict() for k in range(min(cnt.value, 32))], best.value


def params_with(params: Params, tuning: dict) -> Params:
    """A copy of params with a candidate's neighbour method and skin."""
    q = Params.from_buffer_copy(params)
    q.neighbour = NEIGHBOUR_VERLET if tuning["neighbour"] == "verlet" else NEIGHBOUR_CELL
    if q.neighbour == NEIGHBOUR_VERLET:
        q.skin = tuning["skin"]
    return q
