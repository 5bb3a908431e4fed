"""Runs the reference's own code (``oracle/_ref/spc_ref``) on injected inputs.

TEST INFRASTRUCTURE ONLY: used to pin the C restatement and to generate the
golden vectors under ``tests/golden``.  Needs the reference checkout at build
time; the binary is built by ``build_oracle.build_reference()``.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

from . import build_oracle

MODE_RUN, MODE_RHS_RK, MODE_RHS_SRK, MODE_OBSERVE = 0, 1, 2, 3
FAMILY_VECTOR, FAMILY_PTR, FAMILY_VA = 0, 1, 2
STEP_EULER, STEP_SRK, STEP_RK4 = 0, 1, 2


def available() -> bool:
    return build_oracle.reference_available() or os.path.exists(build_oracle.REF_BIN)


def run_reference(n, L, *, mode, family=FAMILY_VECTOR, stepper=STEP_EULER, nsteps=0,
                  record_every=0, v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005,
                  rho_0=1.0, t0=0.0, dt=0.01, k_coef=0.0, state=None, k_prev=None,
                  k_next_init=None, noise=None, binary=None, extra_env=None, va=None):
    """Returns the raw float64 output of the reference driver (or of another
    program reading the same input format, e.g. the drop-in driver)."""
    if binary is None:
        binary = build_oracle.build_reference()
    if binary is None:
        binary = build_oracle.REF_BIN
    n3 = 3 * n
    z = np.zeros(n3)
    state = np.ascontiguousarray(state if state is not None else z, np.float64)
    k_prev = np.ascontiguousarray(k_prev if k_prev is not None else z, np.float64)
    k_next_init = np.ascontiguousarray(k_next_init if k_next_init is not None else z,
                                       np.float64)
    noise = np.ascontiguousarray(noise if noise is not None else np.zeros(0), np.float64)
    hdr = b"SPCREF01" + struct.pack("<6i", mode, family, stepper, nsteps, record_every, 0)
    hdr += struct.pack("<9d", v0, sigma, rho, alpha, D_phi, rho_0, t0, dt, k_coef)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(hdr)
            f.write(state.tobytes())
            f.write(k_prev.tobytes())
            f.write(k_next_init.tobytes())
            f.write(struct.pack("<q", noise.size))
            f.write(noise.tobytes())
            if family == FAMILY_VA:
                # mu_plus, mu_minus, xi_a, xi_r, kappa
                f.write(struct.pack("<5d", *[float(v) for v in va]))
        env = dict(os.environ, SPC_REF_N=str(n), SPC_REF_L=repr(float(L)), **(extra_env or {}))
        subprocess.run([binary, fin, fout], check=True, env=env,
                       stdout=subprocess.DEVNULL)
        return np.fromfile(fout, dtype=np.float64)
