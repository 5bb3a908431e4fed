"""The FP32X form (float pair tests, exact fixed-point neighbour sums, FP64
per-particle arithmetic) against the reference's golden vectors, the plain
FP64 form and itself.

FP32X is held to the plain form's own contract:
* right-hand sides within 1e-12 * max(|value|, scale) of the reference's
  (the scale rule of the FP64 parity tests);
* trajectories within 1e-9 of the reference's after up to 100 steps with the
  reference's injected normals;
* neighbour sums that are exact integers, so the cell-tile and
  warp-per-cell kernels, and a system alone or inside a batch, give the same
  bits;
* order-parameter drift within 1e-4 of the FP64 form over 5,000 steps on a
  16-system subset of the batched Chimera ensemble (alpha ~ U[1.2, 1.6]),
  where the FP32C form's float sums let near-cutoff pairs flip and the
  trajectories separate.
"""
import numpy as np
import pytest

from spc2_langevin_integration_gb300 import abi
from tests._helpers import alignment_scale, golden_cases, init_state, load_golden, periodic_diff
from tests.test_gpu_parity import (KERNELS, RHS_TOL, TRAJ_TOL, _phase_rate_ok, golden_params,
                                   golden_stepper, gpu)

pytestmark = pytest.mark.gpu

X = abi.PRECISION_FP32X
DRIFT_TOL = 1e-4


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", golden_cases())
def test_fp32x_rhs_matches_reference_golden(name, kernel):
    from oracle import pyoracle as po
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    prm = golden_params(g)
    o = po.OracleSystem(n, L, **prm)
    with gpu(n, L, prm, abi.STEPPER_RK4, precision=X, kernel=kernel) as s:
        s.upload_state(g["state0"])
        kn = s.rhs_rk(g["k_prev"], float(g["k_coef"]), float(g["dt"]), g["k_next_init"])
        stage = g["state0"] + float(g["k_coef"]) * float(g["dt"]) * g["k_prev"]
        off, idx = o.neighbour_lists(stage)
        scale, counts = alignment_scale(stage, off, idx, prm["sigma"], prm["alpha"])
        _phase_rate_ok(kn, g["rhs_rk"], scale, prm["v0"])
        iso = counts == 0  # stale k for isolated particles (H5)
        assert np.array_equal(kn[2::3][iso], g["k_next_init"][2::3][iso])
        d, a = s.rhs_srk()
    off, idx = o.neighbour_lists(g["state0"])
    scale, counts = alignment_scale(g["state0"], off, idx, prm["sigma"], prm["alpha"])
    _phase_rate_ok(d, g["srk_derivative"], scale, prm["v0"])
    a_ref = g["srk_additional"].reshape(-1, 2)
    a = a.reshape(-1, 2)
    d_ref = g["srk_derivative"][2::3]
    phi = g["state0"][2::3]
    owner = np.repeat(np.arange(n), np.diff(off))
    c = np.abs(np.cos(phi[idx] - phi[owner] - prm["alpha"]))
    nn = np.maximum(counts, 1)
    s0 = np.sqrt(2 * prm["D_phi"]) * np.bincount(owner, c, n) / nn
    s1 = np.bincount(owner, np.abs(d_ref[idx] - d_ref[owner]) * c, n) / nn + \
        2 * prm["D_phi"] * np.abs(d_ref)
    assert np.all(np.abs(a[:, 0] - a_ref[:, 0]) <= RHS_TOL * np.maximum(np.abs(a_ref[:, 0]), s0) + 1e-300)
    assert np.all(np.abs(a[:, 1] - a_ref[:, 1]) <= RHS_TOL * np.maximum(np.abs(a_ref[:, 1]), s1) + 1e-300)


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", golden_cases())
def test_fp32x_trajectory_matches_reference_golden(name, kernel):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    model = abi.MODEL_VORTEX if "omega" in g else abi.MODEL_CHIMERA
    with gpu(n, L, golden_params(g), golden_stepper(g), model=model, precision=X, kernel=kernel) as s:
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
    for got, ref in zip(frames, g["trajectory"]):
        assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL


CASES = [  # (n, L, params, model): dense cells (tile kernel) and sparse cells (warp kernel)
    (4096, 2.0, dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01), abi.MODEL_VORTEX),
    (3000, 1.7, dict(v0=0.02, sigma=1.3, rho=0.09, alpha=1.4, D_phi=0.01), abi.MODEL_CHIMERA),
]


@pytest.mark.parametrize("stepper", [abi.STEPPER_EULER, abi.STEPPER_SRK, abi.STEPPER_RK4])
def test_fp32x_follows_fp64_with_philox_noise(stepper):
    """100 steps under the library's own Philox noise: FP32X within 1e-9 of
    FP64 (the same normals), and its two neighbour kernels bit for bit equal
    (exact integer sums do not depend on how the candidates are split)."""
    for n, L, prm, model in CASES:
        if model == abi.MODEL_VORTEX and stepper == abi.STEPPER_RK4:
            model = abi.MODEL_CHIMERA  # the vortex model pairs with Euler and SRK
        st0 = init_state(n, L, 71)
        omega = np.random.default_rng(72).normal(0.0, 0.5, n)
        out = {}
        for name, prec, kernel in (("fp64", abi.PRECISION_FP64, None), ("tile", X, "tile"),
                                   ("warp", X, "warp")):
            with gpu(n, L, prm, stepper, model=model, precision=prec, seed=9, kernel=kernel) as s:
                s.upload_state(st0)
                if model == abi.MODEL_VORTEX:
                    s.upload_omega(omega)
                s.step(0.005, 100)
                out[name] = s.download_state()
        assert np.array_equal(out["tile"], out["warp"])
        assert np.abs(periodic_diff(out["tile"], out["fp64"], L)).max() <= TRAJ_TOL


def test_fp32x_batch_equals_alone_bitwise():
    """A system's FP32X trajectory is the same bits alone and inside a batch
    with systems of other sizes and parameters (including an all-pairs one)."""
    systems = [(300, 0.6, dict(v0=0.01, sigma=1.0, rho=0.16, alpha=1.45, D_phi=0.005)),  # all pairs
               (2500, 1.58, dict(v0=0.01, sigma=0.8, rho=0.07, alpha=1.3, D_phi=0.01)),
               (6000, 1.2, dict(v0=0.02, sigma=1.6, rho=0.2, alpha=1.5, D_phi=0.0))]
    alone = []
    for k, (n, L, prm) in enumerate(systems):
        with abi.System(n, abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=X, seed=3,
                                           system_id=k, **prm)) as s:
            s.upload_state(init_state(n, L, 80 + k))
            s.step(0.01, 50)
            alone.append(s.download_state())
    ntot = sum(n for n, _, _ in systems)
    ctot = sum(abi.cells_of(L, prm["rho"]) for _, L, prm in systems)
    with abi.Batch(abi.STEPPER_EULER, X, len(systems), ntot, ctot) as b:
        slots = [b.admit(n, abi.make_params(L=L, stepper=abi.STEPPER_EULER, precision=X, seed=3,
                                            system_id=k, **prm), init_state(n, L, 80 + k))
                 for k, (n, L, prm) in enumerate(systems)]
        b.step(0.01, 50, graph=True)
        for s, ref in zip(slots, alone):
            assert np.array_equal(b.download(s), ref)


def test_fp32x_ensemble_drift_within_target():
    """16 systems of the batched Chimera ensemble (N log-uniform in [256,
    32768], density 1000 / L^2, alpha ~ U[1.2, 1.6], sigma ~ U[0.5, 2],
    D ~ U[0, 0.02], rho ~ U[0.05, 0.15], Euler dt = 0.01, seed 2): FP32X and
    FP64 batches with the same Philox counters, R and R_local of every system
    every 250 steps over 5,000 steps, all within 1e-4."""
    import bench
    systems = bench.ensemble_systems()[:16]
    ntot = sum(n for _, n, _, _, _ in systems)
    ctot = sum(abi.cells_of(L, prm["rho"]) for _, _, L, prm, _ in systems)
    series = {}
    for prec in (abi.PRECISION_FP64, X):
        with abi.Batch(abi.STEPPER_EULER, prec, len(systems), ntot, ctot) as b:
            slots = np.array([b.admit(n, abi.make_params(L=L, stepper=abi.STEPPER_EULER,
                                                         precision=prec, seed=2, system_id=k,
                                                         **prm), st)
                              for k, n, L, prm, st in systems])
            rows = []
            for _ in range(20):
                b.step(0.01, 250, graph=True)
                o = b.order_params_all(len(systems))
                rows.append(np.stack([o["R"][slots], o["R_local"][slots]]))
            series[prec] = np.array(rows)  # [points, 2, systems]
    d = np.abs(series[X] - series[abi.PRECISION_FP64])
    assert np.isfinite(d).all()
    assert d[:, 0].max() <= DRIFT_TOL, d[:, 0].max()
    assert d[:, 1].max() <= DRIFT_TOL, d[:, 1].max()
