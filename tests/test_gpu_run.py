"""spc_run, the engine loop with its observers on the device
(SimulationEngine.cpp:149-161): chunks of steps as CUDA-graph replays with
snapshots of the observed steps, copied to the host while later steps run.
Every snapshot must be bitwise the state that stepping one step at a time and
downloading gives, at every cadence, precision, stepper and neighbour method;
a callback can stop the run; bad arguments are errors."""
import numpy as np
import pytest

from spc2_langevin_integration_gb300 import abi
from tests._helpers import init_state

pytestmark = pytest.mark.gpu

VORTEX = dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01)
CHIMERA = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)


def _open(n, L, prm, stepper, st0, omega=None, precision=abi.PRECISION_FP64,
          neighbour=abi.NEIGHBOUR_CELL, seed=4):
    model = abi.MODEL_VORTEX if omega is not None else abi.MODEL_CHIMERA
    s = abi.System(n, abi.make_params(L=L, stepper=stepper, precision=precision, neighbour=neighbour,
                                      seed=seed, model=model, **prm))
    s.upload_state(st0)
    if omega is not None:
        s.upload_omega(omega)
    return s


def _per_step(s, dt, nsteps, observed):
    out = {}
    for k in range(1, nsteps + 1):
        s.step(dt, 1)
        if k in observed:
            out[k] = (s.t, s.download_state())
    return out


CASES = [
    # stepper, precision, neighbour, vortex (omega), period, observe pattern
    (abi.STEPPER_SRK, abi.PRECISION_FP64, abi.NEIGHBOUR_CELL, True, 10, [1, 1] + [0] * 8),
    (abi.STEPPER_SRK, abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, True, 1, [1]),
    (abi.STEPPER_SRK, abi.PRECISION_FP64, abi.NEIGHBOUR_VERLET, True, 7, [0, 0, 1, 0, 0, 0, 1]),
    (abi.STEPPER_RK4, abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, False, 100, [1] + [0] * 99),
    (abi.STEPPER_EULER, abi.PRECISION_FP64, abi.NEIGHBOUR_CELL, False, 3, [0, 1, 0]),
]


@pytest.mark.parametrize("stepper,precision,neighbour,vortex,period,pattern", CASES)
def test_run_snapshots_equal_step_by_step(stepper, precision, neighbour, vortex, period, pattern):
    n, L, dt, nsteps = 4096, 2.0, 0.005, 150  # full chunks and a partial one
    prm = VORTEX if vortex else CHIMERA
    st0 = init_state(n, L, 31)
    omega = np.random.default_rng(32).normal(0, 0.5, n) if vortex else None
    kw = dict(precision=precision, neighbour=neighbour)
    got = []
    with _open(n, L, prm, stepper, st0, omega, **kw) as s:
        done = s.run(dt, nsteps, period, pattern, lambda k, t, st: got.append((k, t, st)) and False)
        assert done == nsteps
        t_end, final = s.t, s.download_state()
        nodes, gsteps = s.run_graph_nodes()
        assert nodes > 0 and gsteps % period == 0
    observed = [k for k in range(1, nsteps + 1) if pattern[k % period]]
    assert [k for k, _, _ in got] == observed
    with _open(n, L, prm, stepper, st0, omega, **kw) as s:
        want = _per_step(s, dt, nsteps, set(observed))
        assert s.t == t_end
        assert np.array_equal(s.download_state(), final)
    for k, t, st in got:
        assert t == want[k][0]
        assert np.array_equal(st, want[k][1]), k


def test_run_without_observer_equals_step():
    n, L, dt = 2048, 1.5, 0.01
    st0 = init_state(n, L, 33)
    with _open(n, L, CHIMERA, abi.STEPPER_SRK, st0) as a, _open(n, L, CHIMERA, abi.STEPPER_SRK, st0) as b:
        assert a.run(dt, 130) == 130
        b.step(dt, 130)
        assert a.t == b.t
        assert np.array_equal(a.download_state(), b.download_state())
        # a later run continues the same noise stream
        a.run(dt, 5)
        b.step(dt, 5)
        assert np.array_equal(a.download_state(), b.download_state())


def test_run_with_injected_noise_runs_eagerly_and_matches():
    n, L, dt, nsteps = 1024, 1.0, 0.01, 70
    st0 = init_state(n, L, 34)
    noise = np.random.default_rng(35).standard_normal(2 * n * nsteps)
    got = []
    with _open(n, L, CHIMERA, abi.STEPPER_SRK, st0) as s:
        s.inject_noise(noise)
        s.run(dt, nsteps, 1, [1], lambda k, t, st: got.append(st) and False)
        assert s.run_graph_nodes()[0] == 0  # no graph under injected noise
    with _open(n, L, CHIMERA, abi.STEPPER_SRK, st0) as s:
        s.inject_noise(noise)
        for k in range(nsteps):
            s.step(dt, 1)
            assert np.array_equal(got[k], s.download_state()), k


def test_run_stops_when_the_callback_asks():
    n, L, dt = 2048, 1.5, 0.01
    st0 = init_state(n, L, 36)
    seen = []
    with _open(n, L, CHIMERA, abi.STEPPER_EULER, st0) as s:
        done = s.run(dt, 1000, 1, [1], lambda k, t, st: seen.append(k) or k == 25)
        assert seen == list(range(1, 26))
        # the chunk holding step 25 and at most one more were enqueued
        assert 25 < done <= 128 and done % 64 == 0
        final, t_end = s.download_state(), s.t
    with _open(n, L, CHIMERA, abi.STEPPER_EULER, st0) as s:
        s.step(dt, done)
        assert np.array_equal(s.download_state(), final) and s.t == t_end


def test_run_callback_exception_propagates():
    n, L = 1024, 1.0
    with _open(n, L, CHIMERA, abi.STEPPER_EULER, init_state(n, L, 37)) as s:
        def boom(k, t, st):
            raise RuntimeError("observer failed")
        with pytest.raises(RuntimeError, match="observer failed"):
            s.run(0.01, 10, 1, [1], boom)


def test_run_rejects_bad_arguments():
    n, L = 1024, 1.0
    with _open(n, L, CHIMERA, abi.STEPPER_EULER, init_state(n, L, 38)) as s:
        for nsteps, period in ((-1, 1), (10, 0)):
            with pytest.raises(abi.SpcError) as e:
                s.run(0.01, nsteps, period)
            assert e.value.code == -1
        with pytest.raises(ValueError):
            s.run(0.01, 10, 4, [1, 0], lambda *a: False)
