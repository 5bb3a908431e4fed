"""CPU checks of the oracle (the C restatement of the reference's path).

The restatement is pinned against the golden vectors that the reference's own
code produced (tests/golden/make_golden.py) and against known answers that
follow from the reference's formulas by hand.
"""
import math
import platform

import numpy as np
import pytest

from oracle import pyoracle as po
from tests._helpers import golden_cases, load_golden, periodic_diff

EXACT = platform.machine() in ("x86_64", "AMD64")


# Random123 known-answer vectors for philox4x32 with 10 rounds
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    assert po.philox4x32_10(ctr, key) == expect


def _sys(n=4, L=1.0, rho=0.1, **kw):
    prm = dict(v0=0.01, sigma=1.0, rho=rho, alpha=1.45, D_phi=0.005)
    prm.update(kw)
    return po.OracleSystem(n, L, **prm)


def test_min_image_truncation_and_ties():
    # dx -= int(dx * 2 / L) * L (PeriodicBoundaryConditions.cpp:22-35): truncation toward zero
    s = _sys(L=1.0)
    assert s.min_image(0.0, 0.0, 0.5, 0.0)[0] == -0.5   # tie at +L/2 maps to -L/2
    assert s.min_image(0.5, 0.0, 0.0, 0.0)[0] == 0.5    # tie at -L/2 maps to +L/2
    assert s.min_image(0.0, 0.0, 0.49, 0.0)[0] == 0.49
    assert s.min_image(0.0, 0.0, 0.75, 0.0)[0] == -0.25
    assert s.min_image(0.3, 0.0, 0.0, 0.0)[0] == -0.3
    assert s.min_image(0.0, 0.9, 0.0, 0.05)[1] == pytest.approx(0.15, abs=1e-15)


def test_wrap_edges():
    s = _sys(L=1.0)
    assert s.wrap_point(-0.0, 0.5)[0] == 0.0
    assert s.wrap_point(1.0, 0.5)[0] == 0.0
    assert s.wrap_point(1.25, 0.5)[0] == 0.25
    assert s.wrap_point(-0.25, 0.5)[0] == 0.75
    # a tiny negative coordinate wraps to exactly L (the cell-index hazard)
    assert s.wrap_point(-1e-17, 0.5)[0] == 1.0
    x = 1.0 - 2.0 ** -53
    assert s.wrap_point(x, 0.5)[0] == x


def test_cutoff_is_inclusive_and_self_excluded():
    # dr^2 == rho^2 exactly counts as a neighbour (ChimeraSystem.cpp:410)
    L, rho = 4.0, 0.25
    s = _sys(n=3, L=L, rho=rho)
    st = np.array([1.0, 1.0, 0.0, 1.25, 1.0, 0.5, 1.0, 1.2500000000000002, 1.0])
    offsets, idx = s.neighbour_lists(st)
    assert list(np.diff(offsets)) == [1, 1, 0]
    assert list(idx) == [1, 0]


def test_isolated_particle_keeps_previous_rate():
    # k_next's phase entry is only written when n_i != 0 (ChimeraSystem.cpp:421-424)
    s = _sys(n=2, L=1.0, rho=0.1)
    st = np.array([0.1, 0.1, 0.3, 0.6, 0.6, -0.2])
    k_prev = np.zeros(6)
    k_next = np.array([0.0, 0.0, 7.0, 0.0, 0.0, -3.0])
    counts = s.rhs_rk(st, k_prev, k_next, 0.0, 0.01, with_counts=True)
    assert list(counts) == [0, 0]
    assert k_next[2] == 7.0 and k_next[5] == -3.0
    assert k_next[0] == 0.01 * math.cos(0.3)


def test_two_particle_closed_form():
    s = _sys(n=2, L=1.0, rho=0.1, sigma=2.0, alpha=0.4)
    st = np.array([0.5, 0.5, 0.3, 0.55, 0.52, 1.1])
    k = np.zeros(6)
    s.rhs_rk(st, np.zeros(6), k, 0.0, 0.01)
    assert k[2] == 2.0 * math.sin(1.1 - 0.3 - 0.4)
    assert k[5] == 2.0 * math.sin(0.3 - 1.1 - 0.4)


def test_clamped_cell_counted():
    # x = -1e-17 wraps to exactly L, whose cell index int(L/L*nc) = nc is out of range
    s = _sys(n=2, L=1.0, rho=0.1)
    st = np.array([-1e-17, 0.5, 0.0, 0.95, 0.5, 0.0])
    offsets, _ = s.neighbour_lists(st)
    assert s.clamped_cells >= 1
    assert list(np.diff(offsets)) == [1, 1]


def _run_oracle(g):
    n, L = int(g["n"]), float(g["L"])
    prm = {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}
    s = po.OracleSystem(n, L, **prm)
    fam, stp = int(g["family"]), int(g["stepper"])
    kind = {0: po.EULER if fam == 0 else po.EULER_PTR, 1: po.SRK, 2: po.RK4}[stp]
    state = g["state0"].copy()
    frames = []
    every, nsteps = int(g["record_every"]), int(g["nsteps"])
    m = {po.EULER: 1, po.EULER_PTR: 1, po.SRK: 2, po.RK4: 0}[kind]
    noise = g["noise"]
    omega = g.get("omega")
    done, t = 0, 0.0
    while done < nsteps:
        k = min(every - done % every, nsteps - done)
        chunk = noise[done * n * m:(done + k) * n * m] if m else None
        t = s.run(kind, state, t, float(g["dt"]), k, chunk, omega)
        done += k
        if done % every == 0 or done == nsteps:
            frames.append(state.copy())
    return s, np.array(frames)


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_trajectory(name):
    g = load_golden(name)
    _, frames = _run_oracle(g)
    ref = g["trajectory"]
    assert frames.shape == ref.shape
    if EXACT:
        assert np.array_equal(frames, ref)
    else:
        assert np.abs(periodic_diff(frames[-1], ref[-1], float(g["L"]))).max() < 1e-12


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_rhs(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    prm = {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}
    s = po.OracleSystem(n, L, **prm)
    k_next = g["k_next_init"].copy()
    s.rhs_rk(g["state0"], g["k_prev"], k_next, float(g["k_coef"]), float(g["dt"]))
    d, a, _ = s.rhs_srk(g["state0"])
    if EXACT:
        assert np.array_equal(k_next, g["rhs_rk"])
        assert np.array_equal(d, g["srk_derivative"])
        assert np.array_equal(a, g["srk_additional"])
    else:
        np.testing.assert_allclose(k_next, g["rhs_rk"], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(d, g["srk_derivative"], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(a, g["srk_additional"], rtol=1e-13, atol=1e-13)


def test_rk4_buffers_persist_across_steps():
    # RungeKutta4Stepper keeps k1..k4 as members (RungeKutta4Stepper.cpp:7-13)
    g = load_golden("chimera_rk4_n1024")
    n, L = int(g["n"]), float(g["L"])
    prm = {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}
    s = po.OracleSystem(n, L, **prm)
    state = g["state0"].copy()
    s.run(po.RK4, state, 0.0, 0.01, 3)
    buf = s.get_rk4_buffers()
    assert np.any(buf != 0.0)
    s2 = po.OracleSystem(n, L, **prm)
    s2.set_rk4_buffers(buf)
    a, b = state.copy(), state.copy()
    s.run(po.RK4, a, 0.0, 0.01, 2)
    s2.run(po.RK4, b, 0.0, 0.01, 2)
    assert np.array_equal(a, b)


def test_order_parameters_of_synchronised_and_random_states():
    n = 400
    s = _sys(n=n, L=1.0, rho=0.1)
    rng = np.random.default_rng(3)
    st = np.zeros(3 * n)
    st[0::3] = rng.uniform(0, 1, n)
    st[1::3] = rng.uniform(0, 1, n)
    st[2::3] = 0.7
    op = s.order_params(st)
    assert op["R"] == pytest.approx(1.0, abs=1e-12)
    assert op["psi"] == pytest.approx(0.7, abs=1e-12)
    assert op["R_local"] == pytest.approx(1.0, abs=1e-12)
    st[2::3] = rng.uniform(-np.pi, np.pi, n)
    op = s.order_params(st)
    assert op["R"] < 0.2 and 0.0 < op["R_local"] < 1.0
