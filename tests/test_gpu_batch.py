"""Batches of independent systems (spc_batch_*): every system's trajectory
must be the same in a batch as alone, bit for bit, in both precision forms.

A system's noise is keyed by (seed, system id, step, particle) and its
neighbour sums never see another system, so batching changes nothing but the
launches; step budgets freeze a system exactly after its own step count.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from spc2_langevin_integration_gb300 import abi
from tests._helpers import init_state, periodic_diff

pytestmark = pytest.mark.gpu

# (n, L, params, vortex): uneven sizes, one all-pairs system (rho > L/4), one
# dense system (~64 per cell: cell-tile passes) beside sparse ones (~6-13 per
# cell: warp-per-cell passes), so one pass runs both kernels over one mask buffer
SYSTEMS = [
    (1500, 1.2, dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005), False),
    (4096, 1.0, dict(v0=0.02, sigma=1.5, rho=0.125, alpha=0.5, D_phi=0.01), True),
    (400, 0.6, dict(v0=0.01, sigma=0.7, rho=0.07, alpha=1.3, D_phi=0.012), False),
    (3000, 1.8, dict(v0=0.02, sigma=2.0, rho=0.12, alpha=0.0, D_phi=0.01), True),
    (256, 0.5, dict(v0=0.01, sigma=1.5, rho=0.14, alpha=1.55, D_phi=0.002), False),  # all pairs
    (900, 0.95, dict(v0=0.015, sigma=1.2, rho=0.09, alpha=1.2, D_phi=0.0), False),
]


def _params(prm, stepper, precision, k, vortex):
    return abi.make_params(L=prm["L"], stepper=stepper, precision=precision, seed=77,
                           system_id=100 + k,
                           model=abi.MODEL_VORTEX if vortex else abi.MODEL_CHIMERA,
                           **{kk: v for kk, v in prm.items() if kk != "L"})


def _inputs(k, n, L, vortex):
    st = init_state(n, L, 500 + k)
    om = np.random.default_rng(600 + k).normal(0, 0.5, n) if vortex else None
    return st, om


def _alone(n, p, st, om, dt, nsteps):
    with abi.System(n, p) as s:
        s.upload_state(st)
        if om is not None:
            s.upload_omega(om)
        s.step(dt, nsteps)
        return s.download_state()


def _systems(stepper):
    out = []
    for k, (n, L, prm, vortex) in enumerate(SYSTEMS):
        if vortex and stepper == abi.STEPPER_RK4:
            vortex = False
        out.append((k, n, L, dict(prm, L=L), vortex))
    return out


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32C])
@pytest.mark.parametrize("stepper", [abi.STEPPER_EULER, abi.STEPPER_SRK, abi.STEPPER_RK4])
def test_batch_equals_alone_bitwise(stepper, precision):
    dt, nsteps = 0.01, 12
    systems = _systems(stepper)
    tot_n = sum(n for _, n, _, _, _ in systems)
    tot_c = sum(abi.cells_of(L, prm["rho"]) for _, _, L, prm, _ in systems)
    with abi.Batch(stepper, precision, 16, tot_n + 100, tot_c + 10) as b:
        slots = []
        for k, n, L, prm, vortex in systems:
            st, om = _inputs(k, n, L, vortex)
            slots.append(b.admit(n, _params(prm, stepper, precision, k, vortex), st, om))
        b.step(dt, nsteps)
        got = [b.download(s) for s in slots]
    for (k, n, L, prm, vortex), g in zip(systems, got):
        st, om = _inputs(k, n, L, vortex)
        ref = _alone(n, _params(prm, stepper, precision, k, vortex), st, om, dt, nsteps)
        assert np.array_equal(g, ref), (k, np.abs(g - ref).max())


def test_batch_step_budgets_and_graph():
    dt = 0.01
    systems = _systems(abi.STEPPER_EULER)
    budgets = [7, 25, -1, 0, 13]
    with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP64, 8, 20000, 5000) as b:
        slots = []
        for (k, n, L, prm, vortex), bud in zip(systems, budgets):
            st, om = _inputs(k, n, L, vortex)
            slots.append(b.admit(n, _params(prm, abi.STEPPER_EULER, abi.PRECISION_FP64, k, vortex),
                                 st, om, steps=bud))
        b.step(dt, 10, graph=True)
        b.step(dt, 10, graph=True)  # replay
        b.step(dt, 10)
        for (k, n, L, prm, vortex), bud, slot in zip(systems, budgets, slots):
            done, rem = b.status(slot)
            want = 30 if bud < 0 else min(bud, 30)
            assert done == want
            st, om = _inputs(k, n, L, vortex)
            ref = _alone(n, _params(prm, abi.STEPPER_EULER, abi.PRECISION_FP64, k, vortex), st, om,
                         dt, want) if want else st
            assert np.array_equal(b.download(slot), ref)


def test_batch_release_and_readmit():
    dt = 0.01
    sysA, sysB, sysC = _systems(abi.STEPPER_SRK)[0], _systems(abi.STEPPER_SRK)[1], \
        _systems(abi.STEPPER_SRK)[4]
    cap_n = sysA[1] + sysB[1] + 10
    with abi.Batch(abi.STEPPER_SRK, abi.PRECISION_FP32C, 2, cap_n, 1000) as b:
        def adm(sy):
            k, n, L, prm, vortex = sy
            st, om = _inputs(k, n, L, vortex)
            return b.admit(n, _params(prm, abi.STEPPER_SRK, abi.PRECISION_FP32C, k, vortex), st, om)
        a_ = adm(sysA)
        bb = adm(sysB)
        with pytest.raises(abi.SpcError) as e:
            adm(sysC)  # no free slot
        assert e.value.code == -7
        b.step(dt, 10)
        b.release(a_)
        c_ = adm(sysC)  # reuses the released pool range
        b.step(dt, 10)
        assert b.usage()["systems"] == 2
        for sy, slot, steps in ((sysB, bb, 20), (sysC, c_, 10)):
            k, n, L, prm, vortex = sy
            st, om = _inputs(k, n, L, vortex)
            ref = _alone(n, _params(prm, abi.STEPPER_SRK, abi.PRECISION_FP32C, k, vortex), st, om,
                         dt, steps)
            assert np.array_equal(b.download(slot), ref)


def test_batch_capacity_is_enforced():
    k, n, L, prm, vortex = _systems(abi.STEPPER_EULER)[0]
    st, om = _inputs(k, n, L, vortex)
    p = _params(prm, abi.STEPPER_EULER, abi.PRECISION_FP64, k, vortex)
    with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP64, 4, n - 1, 10000) as b:
        with pytest.raises(abi.SpcError) as e:
            b.admit(n, p, st)
        assert e.value.code == -7
    with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP64, 4, 10 * n, 10) as b:
        with pytest.raises(abi.SpcError) as e:
            b.admit(n, p, st)  # 144 cells > 10
        assert e.value.code == -7
    with abi.Batch(abi.STEPPER_SRK, abi.PRECISION_FP64, 4, 10 * n, 10000) as b:
        with pytest.raises(abi.SpcError) as e:
            b.admit(n, p, st)  # stepper differs from the batch's
        assert e.value.code == -1


def test_vortex_euler_matches_oracle():
    n, L = 1024, 1.0
    prm = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=0.0, D_phi=0.005)
    st0 = init_state(n, L, 41)
    om = np.random.default_rng(42).normal(0, 0.5, n)
    p = abi.make_params(L=L, stepper=abi.STEPPER_EULER, model=abi.MODEL_VORTEX, seed=9, **prm)
    with abi.System(n, p) as s:
        s.upload_state(st0)
        s.upload_omega(om)
        s.step(0.01, 100)
        got = s.download_state()
        noise = s.export_noise(0, 100)
    o = po.OracleSystem(n, L, **prm)
    ref = st0.copy()
    o.run(po.EULER, ref, 0.0, 0.01, 100, noise, om)
    assert np.abs(periodic_diff(got, ref, L)).max() <= 1e-9


@pytest.mark.parametrize("model", ["chimera", "vortex_arrays"])
def test_kept_pair_values_past_capacity_are_bitwise(model):
    # A single SRK system keeps the first pass's per-pair values for the
    # second (cosines; vortex arrays: strength, derivative, sin, cos) up to a
    # per-particle capacity of about 2.6x the mean pair count.  A clustered
    # state puts most particles far beyond it, so the second pass mixes kept
    # and recomputed values; a batch of one keeps none.  Both must agree bit
    # for bit.
    n, L, dt, nsteps = 4096, 2.0, 0.005, 6
    rng = np.random.default_rng(58)
    st0 = np.empty(3 * n)
    st0[0::3] = 0.6 + 0.5 * rng.random(n)   # all particles in a 0.5 x 0.5 patch:
    st0[1::3] = 0.6 + 0.5 * rng.random(n)   # 16x the mean density
    st0[2::3] = rng.uniform(-np.pi, np.pi, n)
    if model == "chimera":
        p = abi.make_params(L=L, stepper=abi.STEPPER_SRK, precision=abi.PRECISION_FP64, seed=12,
                            v0=0.02, sigma=1.0, rho=0.25, alpha=0.4, D_phi=0.01)
    else:
        p = abi.make_va_params(L=L, velocity=0.1, mu_plus=100.0, mu_minus=100.0, xi_a=0.04, xi_r=0.02,
                               D_phi=0.01, kappa=20.0, rho=0.2, stepper=abi.STEPPER_SRK, seed=12)
    with abi.System(n, p) as s:
        s.upload_state(st0)
        s.step(dt, nsteps)
        alone = s.download_state()
    with abi.Batch(abi.STEPPER_SRK, abi.PRECISION_FP64, 1, n, abi.cells_of(L, p.rho) + 1) as b:
        slot = b.admit(n, p, st0)
        b.step(dt, nsteps)
        batched = b.download(slot)
    assert np.array_equal(alone, batched)
