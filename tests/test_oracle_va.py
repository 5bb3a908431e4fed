"""The oracle's VortexArraysSystemPtr restatement against the reference's own
build (golden vectors made by tests/golden/make_golden.py): trajectories of
the SRK-Ptr, Euler-Ptr and RK4-Ptr steppers and both right-hand-side forms,
bit for bit; plus closed-form checks of the model's pieces."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from tests._helpers import load_golden, va_golden_cases, va_params

STEPPER = {0: po.EULER_PTR, 1: po.SRK, 2: po.RK4}


@pytest.mark.parametrize("name", va_golden_cases())
def test_va_oracle_matches_reference_trajectory(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    o = po.OracleVortexArrays(n, L, **va_params(g))
    st = g["state0"].copy()
    every, nsteps = int(g["record_every"]), int(g["nsteps"])
    stepper = STEPPER[int(g["stepper"])]
    per = {po.EULER_PTR: n, po.SRK: 2 * n, po.RK4: 0}[stepper]
    frames, done = [], 0
    while done < nsteps:
        k = min(every - done % every, nsteps - done)
        noise = g["noise"][done * per:(done + k) * per] if per else None
        o.run(stepper, st, 0.0, float(g["dt"]), k, noise)
        done += k
        frames.append(st.copy())
    for got, ref in zip(frames, g["trajectory"]):
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", va_golden_cases())
def test_va_oracle_matches_reference_rhs(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    o = po.OracleVortexArrays(n, L, **va_params(g))
    kn = g["k_next_init"].copy()
    o.rhs_rk(g["state0"], g["k_prev"], kn, float(g["k_coef"]), float(g["dt"]))
    assert np.array_equal(kn, g["rhs_rk"])
    d, a, _ = o.rhs_srk(g["state0"])
    assert np.array_equal(d, g["srk_derivative"])
    assert np.array_equal(a, g["srk_additional"])


def test_va_two_particle_closed_form():
    # two particles at distance r < xi_a on the x axis: alignment mu+ (1 - r^2/xi_a^2)
    # sin(phi_j - phi_i), cohesion -kappa sin(atan2(dy, dx) - phi_i) when r <= xi_r
    prm = dict(velocity=0.1, mu_plus=2.0, mu_minus=1.0, xi_a=0.1, xi_r=0.05, D_phi=0.0,
               kappa=3.0, rho=0.2)
    L = 1.0
    o = po.OracleVortexArrays(2, L, **prm)
    r = 0.03
    st = np.array([0.5, 0.5, 0.3, 0.5 + r, 0.5, 1.1])
    d, a, counts = o.rhs_srk(st, with_counts=True)
    align = 2.0 * (1.0 - r * r / 0.01) * math.sin(1.1 - 0.3)
    coh = -3.0 * math.sin(math.atan2(0.0, r) - 0.3)
    assert counts[:3].tolist() == [1, 0, 1]
    assert abs(d[2] - (align + coh)) < 1e-14
    assert d[0] == 0.1 * math.cos(0.3) and d[1] == 0.1 * math.sin(0.3)


def test_va_antialignment_band():
    # xi_a < r <= rho: strength -4 mu- (r - xi_a)(rho - r)/(rho - xi_a)^2, counted in [1]
    prm = dict(velocity=0.0, mu_plus=2.0, mu_minus=1.5, xi_a=0.05, xi_r=0.01, D_phi=0.0,
               kappa=0.0, rho=0.2)
    o = po.OracleVortexArrays(2, 1.0, **prm)
    r = 0.12
    st = np.array([0.2, 0.2, 0.0, 0.2, 0.2 + r, 0.7])
    d, _, counts = o.rhs_srk(st, with_counts=True)
    s = -1.5 * 4.0 * (r - 0.05) * (0.2 - r) / 0.15 / 0.15
    assert counts[:3].tolist() == [0, 1, 0]
    assert abs(d[2] - s * math.sin(0.7)) < 1e-14
