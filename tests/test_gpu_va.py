"""The vortex-arrays model (SPC_MODEL_VORTEX_ARRAYS, the reference's
VortexArraysSystemPtr) on the GPU through the C-ABI: trajectories against the
reference's golden vectors and against the oracle, both right-hand-side forms,
batches mixing it with Chimera systems, and parameter validation.

Tolerances as for the Chimera model: trajectories within 1e-9 (x, y by
minimum image) after up to 50 steps; right-hand sides within 1e-11 of each
array's largest magnitude (CUDA's and glibc's sin / cos / atan2 differ in the
last ulp; the strength derivative makes terms of ~1e3).
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from spc2_langevin_integration_gb300 import abi
from tests._helpers import init_state, load_golden, periodic_diff, va_golden_cases, va_params

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-9
STEPPER = {0: abi.STEPPER_EULER_PTR, 1: abi.STEPPER_SRK, 2: abi.STEPPER_RK4}
ORC = {abi.STEPPER_EULER_PTR: po.EULER_PTR, abi.STEPPER_SRK: po.SRK, abi.STEPPER_RK4: po.RK4}
PRM = dict(velocity=0.1, mu_plus=100.0, mu_minus=100.0, xi_a=0.04, xi_r=0.02, D_phi=0.01,
           kappa=20.0, rho=0.2)


def va_system(n, L, prm, stepper, seed=0, system_id=0):
    return abi.System(n, abi.make_va_params(L=L, stepper=stepper, seed=seed, system_id=system_id,
                                            **prm))


def close(got, ref, rel=1e-11):
    return np.abs(got - ref).max() <= rel * max(np.abs(ref).max(), 1.0)


@pytest.mark.parametrize("name", va_golden_cases())
def test_va_trajectory_matches_reference_golden(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    with va_system(n, L, va_params(g), STEPPER[int(g["stepper"])]) as s:
        s.upload_state(g["state0"])
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


@pytest.mark.parametrize("name", va_golden_cases())
def test_va_rhs_matches_reference_golden(name):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    with va_system(n, L, va_params(g), abi.STEPPER_RK4) as s:
        s.upload_state(g["state0"])
        kn = s.rhs_rk(g["k_prev"], float(g["k_coef"]), float(g["dt"]), g["k_next_init"])
    assert close(kn, g["rhs_rk"])
    with va_system(n, L, va_params(g), abi.STEPPER_SRK) as s:
        s.upload_state(g["state0"])
        d, a = s.rhs_srk()
    assert close(d, g["srk_derivative"])
    assert close(a[0::2], g["srk_additional"][0::2])
    assert close(a[1::2], g["srk_additional"][1::2])


@pytest.mark.parametrize("stepper", [abi.STEPPER_EULER_PTR, abi.STEPPER_SRK, abi.STEPPER_RK4])
def test_va_50_steps_with_philox_noise(stepper):
    n, L, dt, nsteps = 2048, 1.5, 0.01, 50
    prm = dict(PRM, rho=0.1, xi_a=0.05, xi_r=0.03, mu_plus=20.0, mu_minus=10.0, kappa=5.0)
    st0 = init_state(n, L, 71)
    with va_system(n, L, prm, stepper, seed=21) as s:
        s.upload_state(st0)
        s.step(dt, nsteps)
        got = s.download_state()
        noise = s.export_noise(0, nsteps) if s.noise_per_particle else None
    o = po.OracleVortexArrays(n, L, **prm)
    ref = st0.copy()
    o.run(ORC[stepper], ref, 0.0, dt, nsteps, noise)
    assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL


def test_va_in_a_batch_with_chimera_systems_is_bitwise_alone():
    dt, nsteps = 0.01, 15
    chim = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
    systems = [
        ("va", 1500, 1.2, dict(PRM, rho=0.12, xi_a=0.05, xi_r=0.04)),
        ("ch", 1000, 1.0, chim),
        ("va", 150, 0.6, PRM),  # all pairs (rho > L/4)
        ("ch", 3000, 1.8, dict(chim, rho=0.15)),
    ]

    def params(k, kind, L, prm):
        if kind == "va":
            return abi.make_va_params(L=L, stepper=abi.STEPPER_SRK, seed=5, system_id=k, **prm)
        return abi.make_params(L=L, stepper=abi.STEPPER_SRK, seed=5, system_id=k, **prm)

    tot_n = sum(n for _, n, _, _ in systems)
    tot_c = sum(abi.cells_of(L, p["rho"]) for _, _, L, p in systems)
    with abi.Batch(abi.STEPPER_SRK, abi.PRECISION_FP64, 8, tot_n + 10, tot_c + 10) as b:
        slots = [b.admit(n, params(k, kind, L, p), init_state(n, L, 80 + k))
                 for k, (kind, n, L, p) in enumerate(systems)]
        b.step(dt, nsteps, graph=True)
        got = [b.download(s) for s in slots]
    for k, ((kind, n, L, p), g) in enumerate(zip(systems, got)):
        with abi.System(n, params(k, kind, L, p)) as s:
            s.upload_state(init_state(n, L, 80 + k))
            s.step(dt, nsteps)
            assert np.array_equal(g, s.download_state()), (k, kind)


def test_va_neighbour_diagnostics_and_validation():
    n, L = 1024, 1.0
    st = init_state(n, L, 72)
    with va_system(n, L, PRM, abi.STEPPER_SRK) as s:
        s.upload_state(st)
        off, idx = s.neighbours()  # pairs within rho, in the reference's visiting order
    o = po.OracleSystem(n, L, v0=0.1, sigma=1.0, rho=PRM["rho"], alpha=0.0, D_phi=0.01)
    off_ref, idx_ref = o.neighbour_lists(st)
    assert np.array_equal(off, off_ref) and np.array_equal(idx, idx_ref)
    bad = [dict(stepper=abi.STEPPER_EULER), dict(precision=abi.PRECISION_FP32C)]
    for kw in bad:
        p = abi.make_va_params(L=L, **PRM)
        for k, v in kw.items():
            setattr(p, k, v)
        with pytest.raises(abi.SpcError) as e:
            abi.System(n, p)
        assert e.value.code == -1
