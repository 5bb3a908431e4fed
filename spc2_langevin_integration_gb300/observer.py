"""Observer files in the reference's formats, for Python callers.

* Frames (Observers/BinaryObserver.cpp:186-191): per saved step the time as
  float32, then the 3N state values as float32 in array-of-structures order
  [x0, y0, phi0, x1, ...], appended to one .bin file.
* Summary statistics (BinaryObserver.cpp:196-234): one text line per saved
  step, "t<TAB>|R|<TAB>arg R", R = (1/N) sum_i (cos phi_i, sin phi_i) with each
  term rounded to float and the sum accumulated in float in index order,
  printed with six significant digits.
* Restart files (SimulationEngine.cpp:52-73): 3N float32 values from the
  start of the file.

The C++ drop-in writes the same bytes (host/spc_observer.cpp).  Device-resident
runs download the state on the observation cadence (System.download_state).
"""
from __future__ import annotations

import os
from typing import Iterator

import numpy as np


def frame_bytes(t: float, state) -> bytes:
    st = np.asarray(state, dtype=np.float64)
    return np.float32(t).tobytes() + st.astype(np.float32).tobytes()


def order_parameter_f32(state) -> tuple[np.float32, np.float32]:
    """|R| and arg R exactly as the reference's observer computes them."""
    phi = np.asarray(state, dtype=np.float64)[2::3]
    c = np.cos(phi).astype(np.float32)
    s = np.sin(phi).astype(np.float32)
    # complex<float> += term by term, in index order (cumsum accumulates in order)
    re = np.cumsum(c, dtype=np.float32)[-1] if c.size else np.float32(0.0)
    im = np.cumsum(s, dtype=np.float32)[-1] if s.size else np.float32(0.0)
    n = np.float32(phi.size)
    re, im = np.float32(re / n), np.float32(im / n)
    return np.float32(np.hypot(re, im)), np.float32(np.arctan2(im, re))


def summary_line(t: float, state) -> str:
    r, psi = order_parameter_f32(state)
    return "%g\t%g\t%g\n" % (float(np.float32(t)), float(r), float(psi))


def file_tag(v0, sigma, rho, alpha, D_phi, n, rho_0, trial=0) -> str:
    """The reference's file-name pattern (BinaryObserver.cpp:47-55), with
    C++ default stream formatting of the numbers."""
    g = lambda x: "%g" % x  # noqa: E731
    return (f"v0_{g(v0)}_sigma_{g(sigma)}_rho_{g(rho)}_alpha_{g(alpha)}_Dphi_{g(D_phi)}"
            f"_N_{int(n)}_rho0_{g(rho_0)}_0_{int(trial)}")


class BinaryObserver:
    """SaveSystemState / SaveSummaryStatistics with the reference's cadence
    counters (every `state_every`-th / `summary_every`-th call)."""

    def __init__(self, folder: str, v0, sigma, rho, alpha, D_phi, n, rho_0, trial=0,
                 state_every: int = 1, summary_every: int = 1):
        tag = file_tag(v0, sigma, rho, alpha, D_phi, n, rho_0, trial)
        self.simulation_file = os.path.join(folder, tag + ".bin")
        self.summary_file = os.path.join(folder, "summary_statistics_" + tag + ".txt")
        for f in (self.simulation_file, self.summary_file):
            if os.path.exists(f):
                os.remove(f)
        self.every = (int(state_every), int(summary_every))
        self.counter = [0, 0]

    def save_system_state(self, state, t: float):
        if self.counter[0] % self.every[0] == 0:
            with open(self.simulation_file, "ab") as f:
                f.write(frame_bytes(t, state))
        self.counter[0] += 1

    def save_summary_statistics(self, state, t: float):
        if self.counter[1] % self.every[1] == 0:
            with open(self.summary_file, "a") as f:
                f.write(summary_line(t, state))
        self.counter[1] += 1


def read_frames(path: str, n: int) -> Iterator[tuple[float, np.ndarray]]:
    """(t, float32 state) of every frame of a .bin file."""
    raw = np.fromfile(path, dtype=np.float32)
    per = 1 + 3 * n
    if raw.size % per:
        raise ValueError(f"{path}: {raw.size} floats is not a whole number of frames of N={n}")
    for k in range(raw.size // per):
        fr = raw[k * per:(k + 1) * per]
        yield float(fr[0]), fr[1:].copy()


def read_restart(path: str, n: int) -> np.ndarray:
    """The double state from a restart file (3N float32 from byte 0)."""
    raw = np.fromfile(path, dtype=np.float32, count=3 * n)
    if raw.size != 3 * n:
        raise ValueError(f"{path}: fewer than 3N float32 values")
    return raw.astype(np.float64)


def write_restart(path: str, state) -> None:
    np.asarray(state, dtype=np.float64).astype(np.float32).tofile(path)
