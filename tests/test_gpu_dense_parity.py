"""Oracle parity on dense and clustered states.

The neighbour kernels change path once cells fill up: the cell-tile kernels
stage the stencil in several rounds (past 1,024 candidates in FP32C, 768 in
FP32X and FP64), the FP64 cell-tile kernel drains its per-thread queue early,
the warp-per-cell kernels stage 256 candidates per round, and Verlet rows
longer than their limit scan the whole stencil.  The headline vortex workload
runs in those paths once it clusters.  Here each kernel is compared with the
oracle, not with another GPU path, on three states:
* a 4,096-particle patch (all particles in a 0.5 x 0.5 square of an L = 2
  box, rho = 0.25: ~1,000 particles per cell, ~9,000 candidates per particle);
* the vortex workload's initial state (N = 65,536, L = 8, uniform);
* the same workload after 4,000 FP64 steps (tests/golden/states, made by
  tests/golden/make_clustered.py): clustered.
Checks, with the plain form's tolerances (ChimeraSystem.cpp:365-425 for the
sums, :429-645 for the SRK form):
* neighbour sets bit-exact (diagnostics kernel) against the oracle;
* SRK-form right-hand sides (derivative and additional derivative) within
  1e-12 of the oracle's on the scale rule, for FP64 cell-tile, warp-per-cell
  and Verlet rows and for FP32X; FP32C within its 2e-6 bound; the float
  cell-tile kernels also with cell units (cells run as units of 32
  particles x one staging round) and with sub-cells (units of half cells
  over the half stencils);
* 10 SRK steps under the library's Philox noise (the exported normals fed to
  the oracle) within 1e-9 for the same FP64 and FP32X variants.
"""
import functools
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from spc2_langevin_integration_gb300 import abi
from tests._helpers import alignment_scale, periodic_diff
from tests.test_gpu_parity import RHS_TOL, TRAJ_TOL

pytestmark = pytest.mark.gpu

FP32C_TOL = 2e-6
STATES_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "states")
VORTEX = dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01)
# variant: (precision, neighbour, SPARSE_BELOW tuning, cell units: 1, or sub-cells: 2)
VARIANTS = {
    "fp64_tile": (abi.PRECISION_FP64, abi.NEIGHBOUR_CELL, 0.0, 0),
    "fp64_warp": (abi.PRECISION_FP64, abi.NEIGHBOUR_CELL, 1e9, 0),
    "fp64_verlet": (abi.PRECISION_FP64, abi.NEIGHBOUR_VERLET, None, 0),
    "fp32x_tile": (abi.PRECISION_FP32X, abi.NEIGHBOUR_CELL, 0.0, 0),
    "fp32x_units": (abi.PRECISION_FP32X, abi.NEIGHBOUR_CELL, 0.0, 1),
    "fp32x_subcells": (abi.PRECISION_FP32X, abi.NEIGHBOUR_CELL, 0.0, 2),
    "fp32x_warp": (abi.PRECISION_FP32X, abi.NEIGHBOUR_CELL, 1e9, 0),
    "fp32c_tile": (abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, 0.0, 0),
    "fp32c_units": (abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, 0.0, 1),
    "fp32c_subcells": (abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, 0.0, 2),
    "fp32c_warp": (abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, 1e9, 0),
}
STATE_NAMES = ["patch_n4096", "vortex_initial_n65536", "vortex_clustered_n65536"]


@functools.lru_cache(maxsize=None)
def _state(name):
    """(n, L, params, state, omega) of a named state."""
    if name == "patch_n4096":
        n, L = 4096, 2.0
        rng = np.random.default_rng(58)
        st = np.empty(3 * n)
        st[0::3] = 0.6 + 0.5 * rng.random(n)
        st[1::3] = 0.6 + 0.5 * rng.random(n)
        st[2::3] = rng.uniform(-np.pi, np.pi, n)
        return n, L, dict(v0=0.02, sigma=1.0, rho=0.25, alpha=0.4, D_phi=0.01), st, \
            rng.normal(0.0, 0.5, n)
    n, L = 65536, 8.0
    rng = np.random.default_rng(1)
    st = np.empty(3 * n)
    st[0::3] = rng.uniform(0.0, L, n)
    st[1::3] = rng.uniform(0.0, L, n)
    st[2::3] = rng.uniform(-np.pi, np.pi, n)
    omega = rng.normal(0.0, 0.5, n)
    if name == "vortex_initial_n65536":
        return n, L, VORTEX, st, omega
    z = np.load(os.path.join(STATES_DIR, "vortex_clustered_n65536.npz"))
    assert np.array_equal(z["omega"], omega)
    return n, L, VORTEX, z["state"].copy(), omega


def _system(n, L, prm, variant, st, omega, seed=5):
    prec, nb, sb, units = VARIANTS[variant]
    s = abi.System(n, abi.make_params(L=L, stepper=abi.STEPPER_SRK, model=abi.MODEL_VORTEX,
                                      precision=prec, neighbour=nb, skin=0.05, seed=seed, **prm))
    if sb is not None:
        s.set_tuning(abi.TUNE_SPARSE_BELOW, sb)
    if units == 1:
        s.set_tuning(abi.TUNE_CELL_UNITS, 1)
    if units == 2:
        s.set_tuning(abi.TUNE_SUBCELLS, 1)
    s.upload_state(st)
    s.upload_omega(omega)
    return s


@functools.lru_cache(maxsize=None)
def _oracle_rhs(name):
    n, L, prm, st, _ = _state(name)
    o = po.OracleSystem(n, L, **prm)
    d, a, _ = o.rhs_srk(st)
    off, idx = o.neighbour_lists(st)
    scale, counts = alignment_scale(st, off, idx, prm["sigma"], prm["alpha"])
    phi = st[2::3]
    owner = np.repeat(np.arange(n), np.diff(off))
    c = np.abs(np.cos(phi[idx] - phi[owner] - prm["alpha"]))
    nn = np.maximum(counts, 1)
    rate = d[2::3]
    s0 = np.sqrt(2 * prm["D_phi"]) * np.bincount(owner, c, n) / nn
    s1 = np.bincount(owner, np.abs(rate[idx] - rate[owner]) * c, n) / nn + \
        2 * prm["D_phi"] * np.abs(rate)
    return d, a, off, idx, scale, s0, s1, counts


def _candidates(n, L, rho, st):
    """Candidates per particle: the members of its cell's 3x3 stencil."""
    nc = int(L / rho)
    cx = np.minimum((st[0::3] / L * nc).astype(int), nc - 1)
    cy = np.minimum((st[1::3] / L * nc).astype(int), nc - 1)
    occ = np.bincount(cy * nc + cx, minlength=nc * nc).reshape(nc, nc)
    sten = sum(np.roll(np.roll(occ, dy, 0), dx, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1))
    return sten[cy, cx]


@pytest.mark.parametrize("name", STATE_NAMES)
def test_dense_state_is_dense(name):
    """The states reach the paths they are here for: the clustered and patch
    states have particles with more candidates than one FP32C staging round
    (1,024) and more neighbours than four times the uniform mean."""
    n, L, prm, st, _ = _state(name)
    cand = _candidates(n, L, prm["rho"], st)
    counts = _oracle_rhs(name)[7]
    mean = np.pi * prm["rho"] ** 2 * n / L ** 2
    if name == "vortex_initial_n65536":
        assert cand.max() < 1024 and counts.max() < 2 * mean
    else:
        assert cand.max() > 1024, cand.max()
        assert counts.max() > 4 * mean, counts.max()


@pytest.mark.parametrize("name", STATE_NAMES)
def test_dense_neighbour_sets_bit_exact(name):
    n, L, prm, st, omega = _state(name)
    _, _, off_ref, idx_ref = _oracle_rhs(name)[:4]
    with _system(n, L, prm, "fp64_tile", st, omega) as s:
        off, idx = s.neighbours()
    assert np.array_equal(off, off_ref)
    assert np.array_equal(idx, idx_ref)


@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("name", STATE_NAMES)
def test_dense_rhs_matches_oracle(name, variant):
    n, L, prm, st, omega = _state(name)
    d_ref, a_ref, _, _, scale, s0, s1, _ = _oracle_rhs(name)
    with _system(n, L, prm, variant, st, omega) as s:
        d, a = s.rhs_srk()
    tol = FP32C_TOL if variant.startswith("fp32c") else RHS_TOL
    d, dr = d.reshape(-1, 3), d_ref.reshape(-1, 3)
    assert np.all(np.abs(d[:, :2] - dr[:, :2]) <= tol * prm["v0"] + 1e-300)
    if variant.startswith("fp32c"):
        err = np.abs(d[:, 2] - dr[:, 2])
        assert np.all(err <= tol * np.maximum(scale, 1e-3)), err.max()
        return
    bad = np.abs(d[:, 2] - dr[:, 2]) > tol * np.maximum(np.abs(dr[:, 2]), scale)
    assert not bad.any(), (np.flatnonzero(bad)[:5], d[bad][:3], dr[bad][:3])
    a, ar = a.reshape(-1, 2), a_ref.reshape(-1, 2)
    assert np.all(np.abs(a[:, 0] - ar[:, 0]) <= tol * np.maximum(np.abs(ar[:, 0]), s0) + 1e-300)
    assert np.all(np.abs(a[:, 1] - ar[:, 1]) <= tol * np.maximum(np.abs(ar[:, 1]), s1) + 1e-300)


@functools.lru_cache(maxsize=None)
def _oracle_run(name, nsteps):
    """The oracle's SRK trajectory under the normals the library draws for seed 5."""
    n, L, prm, st, omega = _state(name)
    with _system(n, L, prm, "fp64_tile", st, omega) as s:
        noise = s.export_noise(0, nsteps)
    o = po.OracleSystem(n, L, **prm)
    ref = st.copy()
    o.run(po.SRK, ref, 0.0, 0.005, nsteps, noise, omega)
    return ref


@pytest.mark.parametrize("variant", [v for v in sorted(VARIANTS) if not v.startswith("fp32c")])
@pytest.mark.parametrize("name", STATE_NAMES)
def test_dense_trajectory_matches_oracle(name, variant):
    nsteps = 10
    n, L, prm, st, omega = _state(name)
    ref = _oracle_run(name, nsteps)
    with _system(n, L, prm, variant, st, omega) as s:
        s.step(0.005, nsteps)
        got = s.download_state()
    assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL
