"""Verlet neighbour rows (SPC_NEIGHBOUR_VERLET): parity with the reference
golden vectors and the oracle, agreement with the cell-list path, the
displacement-triggered rebuild, and the overflow fallback.

The rows only change which candidates are tested: every pair is still decided
by the reference's exact FP64 cutoff test, so trajectories carry the cell-list
path's tolerances (1e-9 after 100 steps against the oracle).  Sums run in row
order (a 5x5 stencil of cells, ascending index inside a cell) rather than the
reference's 3x3 order, so against the cell-list path the FP64 results agree to
rounding, not bit for bit.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from spc2_langevin_integration_gb300 import abi
from tests._helpers import golden_cases, init_state, load_golden, periodic_diff

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-9
PRM0 = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
KIND = {abi.STEPPER_EULER: po.EULER, abi.STEPPER_EULER_PTR: po.EULER_PTR,
        abi.STEPPER_SRK: po.SRK, abi.STEPPER_RK4: po.RK4}


def verlet(n, L, prm, stepper, skin=0.05, model=abi.MODEL_CHIMERA,
           precision=abi.PRECISION_FP64, seed=0, neighbour=abi.NEIGHBOUR_VERLET):
    p = abi.make_params(L=L, stepper=stepper, model=model, precision=precision,
                        neighbour=neighbour, skin=skin, seed=seed, **prm)
    return abi.System(n, p)


def golden_stepper(g):
    fam, stp = int(g["family"]), int(g["stepper"])
    if stp == 0:
        return abi.STEPPER_EULER if fam == 0 else abi.STEPPER_EULER_PTR
    return abi.STEPPER_SRK if stp == 1 else abi.STEPPER_RK4


def golden_params(g):
    return {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}


def oracle_run(n, L, prm, stepper, st0, dt, nsteps, noise, omega=None):
    o = po.OracleSystem(n, L, **prm)
    st = st0.copy()
    o.run(KIND[stepper], st, 0.0, dt, nsteps, noise, omega)
    return st


@pytest.mark.parametrize("name", [c for c in golden_cases() if "allpairs" not in c])
def test_verlet_trajectory_matches_reference_golden(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    model = abi.MODEL_VORTEX if "omega" in g else abi.MODEL_CHIMERA
    with verlet(n, L, golden_params(g), golden_stepper(g), model=model) as s:
        s.upload_state(g["state0"])
        if "omega" in g:
            s.upload_omega(g["omega"])
        if s.noise_per_particle:
            s.inject_noise(g["noise"])
        every, nsteps = int(g["record_every"]), int(g["nsteps"])
        frames, done = [], 0
        while done < nsteps:
            k = min(every - done % every, nsteps - done)
            s.step(float(g["dt"]), k)
            done += k
            frames.append(s.download_state())
        assert s.diagnostics()["verlet_rebuilds"] >= 1
    for got, ref in zip(frames, g["trajectory"]):
        assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL


@pytest.mark.parametrize("stepper,n,L,prm,dt,skin", [
    (abi.STEPPER_EULER, 1024, 1.0, PRM0, 0.01, 0.05),
    (abi.STEPPER_SRK, 2048, 2.0, dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01), 0.005, 0.05),
    (abi.STEPPER_RK4, 4096, 4.0, dict(v0=0.01, sigma=1.0, rho=0.25, alpha=1.45, D_phi=0.0), 0.01, 0.05),
    # fast particles, thin skin: a rebuild every few steps
    (abi.STEPPER_EULER, 2048, 1.5, dict(v0=0.6, sigma=1.0, rho=0.1, alpha=1.3, D_phi=0.01), 0.01, 0.03),
])
def test_verlet_100_steps_with_philox_noise(stepper, n, L, prm, dt, skin):
    nsteps = 100
    st0 = init_state(n, L, 61)
    vortex = stepper == abi.STEPPER_SRK
    omega = np.random.default_rng(62).normal(0, 0.5, n) if vortex else None
    with verlet(n, L, prm, stepper, skin=skin, seed=99,
                model=abi.MODEL_VORTEX if vortex else abi.MODEL_CHIMERA) as s:
        s.upload_state(st0)
        if vortex:
            s.upload_omega(omega)
        s.step(dt, nsteps)
        got = s.download_state()
        rebuilds = s.diagnostics()["verlet_rebuilds"]
        noise = s.export_noise(0, nsteps) if s.noise_per_particle else None
    ref = oracle_run(n, L, prm, stepper, st0, dt, nsteps, noise, omega)
    assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL
    # the displacement test rebuilds about every (skin / 2) / (v0 dt) steps
    expect = nsteps * prm["v0"] * dt / (0.5 * skin)
    assert rebuilds >= max(1, int(0.5 * expect))
    assert rebuilds <= 2 * expect + 2


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32C])
def test_verlet_agrees_with_cell_list(precision):
    n, L, dt = 4096, 2.0, 0.005
    prm = dict(v0=0.02, sigma=2.0, rho=0.2, alpha=1.2, D_phi=0.01)
    st0 = init_state(n, L, 63)
    out = {}
    for nb in (abi.NEIGHBOUR_CELL, abi.NEIGHBOUR_VERLET):
        with verlet(n, L, prm, abi.STEPPER_SRK, neighbour=nb, precision=precision, seed=4) as s:
            s.upload_state(st0)
            s.step(dt, 50)
            out[nb] = s.download_state()
    d = np.abs(periodic_diff(out[abi.NEIGHBOUR_CELL], out[abi.NEIGHBOUR_VERLET], L)).max()
    assert d <= (1e-11 if precision == abi.PRECISION_FP64 else 1e-5)


def test_row_overflow_fallback_is_bitwise_fp64():
    """With a row limit of 8 every particle scans its whole stencil instead of
    its row; the accepted terms and their order are the same, so FP64 results
    are identical bit for bit."""
    n, L, dt = 3000, 1.5, 0.01
    prm = dict(v0=0.05, sigma=1.0, rho=0.12, alpha=1.4, D_phi=0.01)
    st0 = init_state(n, L, 64)
    out = []
    for limit in (None, 8):
        with verlet(n, L, prm, abi.STEPPER_SRK, seed=3) as s:
            if limit is not None:
                cap = s.get_tuning(abi.TUNE_VERLET_ROW_LIMIT)
                assert cap >= 64
                s.set_tuning(abi.TUNE_VERLET_ROW_LIMIT, limit)
            s.upload_state(st0)
            s.step(dt, 30)
            out.append(s.download_state())
    assert np.array_equal(out[0], out[1])


def test_graph_replay_and_diagnostics_interleave():
    n, L, dt = 2048, 1.5, 0.01
    prm = dict(v0=0.3, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
    st0 = init_state(n, L, 65)
    with verlet(n, L, prm, abi.STEPPER_EULER, seed=8) as a, \
            verlet(n, L, prm, abi.STEPPER_EULER, seed=8) as b, \
            verlet(n, L, prm, abi.STEPPER_EULER, seed=8) as c:
        for s in (a, b, c):
            s.upload_state(st0)
        a.step(dt, 60)
        for _ in range(3):
            b.step(dt, 20, graph=True)
        assert np.array_equal(a.download_state(), b.download_state())
        # diagnostics read the reference's current cells and force a rebuild
        for _ in range(3):
            c.step(dt, 20)
            _, idx = c.neighbours()
            o = po.OracleSystem(n, L, **prm)
            off, ref_idx = o.neighbour_lists(c.download_state())
            assert np.array_equal(idx, ref_idx)
        assert np.abs(periodic_diff(c.download_state(), a.download_state(), L)).max() <= 1e-11


def test_fp32c_verlet_rhs_error_is_small():
    g = load_golden("chimera_euler_n1024")
    n, L = int(g["n"]), float(g["L"])
    prm = golden_params(g)
    with verlet(n, L, prm, abi.STEPPER_SRK) as s64, \
            verlet(n, L, prm, abi.STEPPER_SRK, precision=abi.PRECISION_FP32C) as s32:
        s64.upload_state(g["state0"])
        s32.upload_state(g["state0"])
        d64, a64 = s64.rhs_srk()
        d32, a32 = s32.rhs_srk()
    assert np.abs(d64 - g["srk_derivative"]).max() <= 1e-12 * max(1.0, np.abs(g["srk_derivative"]).max())
    assert np.abs(d32[2::3] - d64[2::3]).max() <= 2e-6 * prm["sigma"]
    assert np.abs(a32 - a64).max() <= 2e-6


def test_verlet_falls_back_to_cells_when_the_stencil_wraps():
    # L = 0.5, rho = 0.1: five cells per side, r_max = 0.35 needs a 9x9 stencil
    n, L = 300, 0.5
    prm = dict(PRM0)
    st0 = init_state(n, L, 66)
    out = []
    for nb in (abi.NEIGHBOUR_CELL, abi.NEIGHBOUR_VERLET):
        with verlet(n, L, prm, abi.STEPPER_EULER, skin=0.25, neighbour=nb, seed=2) as s:
            s.upload_state(st0)
            s.step(0.01, 20)
            out.append(s.download_state())
            assert s.diagnostics()["verlet_rebuilds"] == 0
    assert np.array_equal(out[0], out[1])


def test_autotune_picks_an_exact_candidate():
    n, L, dt = 4096, 2.0, 0.005
    prm = dict(v0=0.02, sigma=2.0, rho=0.2, alpha=1.2, D_phi=0.01)
    st0 = init_state(n, L, 67)
    p = abi.make_params(L=L, stepper=abi.STEPPER_SRK, seed=12, skin=0.05, **prm)
    best, sparse_below, ms = abi.autotune(n, p, st0, dt=dt, trial_steps=5)
    assert len(ms) == 6 and all(m > 0 for m in ms)
    assert best.neighbour in (abi.NEIGHBOUR_CELL, abi.NEIGHBOUR_VERLET)
    with abi.System(n, best) as s:
        if best.neighbour == abi.NEIGHBOUR_CELL:
            s.set_tuning(abi.TUNE_SPARSE_BELOW, sparse_below)
        s.upload_state(st0)
        s.step(dt, 50)
        got = s.download_state()
        noise = s.export_noise(0, 50)
    ref = oracle_run(n, L, prm, abi.STEPPER_SRK, st0, dt, 50, noise)
    assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL
