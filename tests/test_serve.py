"""Serving loop: scheduling on the CPU with a stand-in batch, and on the GPU
the guarantee that a served result equals the same request run alone."""
import numpy as np
import pytest

from spc2_langevin_integration_gb300 import abi, serve


class FakeBatch:
    """The batch interface with capacity rules and step budgets, no GPU."""

    def __init__(self, max_systems, max_particles, max_cells):
        self.cap = (max_systems, max_particles, max_cells)
        self.capacity = {"particles": max_particles, "cells": max_cells, "systems": max_systems}
        self.sys = {}
        self.steps_taken = 0
        self.log = []

    def usage(self):
        return {"particles": sum(v["n"] for v in self.sys.values()),
                "cells": sum(v["cells"] for v in self.sys.values()), "systems": len(self.sys)}

    def admit(self, n, params, state, omega=None, steps=-1):
        cells = abi.cells_of(params.L, params.rho)
        used_n = sum(v["n"] for v in self.sys.values())
        used_c = sum(v["cells"] for v in self.sys.values())
        if (len(self.sys) >= self.cap[0] or used_n + n > self.cap[1] or
                used_c + cells > self.cap[2]):
            raise abi.SpcError(-7, "capacity")
        slot = next(s for s in range(self.cap[0]) if s not in self.sys)
        assert params.system_id not in [v["id"] for v in self.sys.values()]
        self.sys[slot] = {"n": n, "cells": cells, "rem": steps, "done": 0, "id": params.system_id}
        self.log.append(("admit", params.system_id, self.steps_taken))
        return slot

    def step(self, dt, nsteps):
        self.steps_taken += nsteps
        for v in self.sys.values():
            k = min(nsteps, v["rem"])
            v["rem"] -= k
            v["done"] += k

    def synchronize(self):
        pass

    def status(self, slot):
        return self.sys[slot]["done"], self.sys[slot]["rem"]

    def download(self, slot):
        return np.zeros(3 * self.sys[slot]["n"])

    def release(self, slot):
        self.log.append(("release", self.sys[slot]["id"], self.steps_taken))
        del self.sys[slot]


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-3
        return self.t


def test_trace_matches_the_configured_distributions():
    tr = serve.make_trace(rate=200, duration=20, seed=3)
    assert 3600 < len(tr) < 4400
    ns = np.array([r.n for r in tr])
    assert ns.min() >= 512 and ns.max() <= 262144
    assert abs(np.median(np.log(ns)) - 0.5 * (np.log(512) + np.log(262144))) < 0.3
    steps = np.array([r.steps for r in tr])
    assert steps.min() >= 500 and steps.max() <= 5000
    frac_vortex = np.mean([r.model == abi.MODEL_VORTEX for r in tr])
    assert 0.45 < frac_vortex < 0.55
    assert all(0.05 <= r.rho <= 0.15 for r in tr)
    assert all(abs(r.L ** 2 * 1000 - r.n) < 1e-6 * r.n for r in tr)
    assert all(r.alpha == 0.0 for r in tr if r.model == abi.MODEL_VORTEX)
    # deterministic in the seed
    tr2 = serve.make_trace(rate=200, duration=20, seed=3)
    assert [(r.n, r.steps, r.arrival) for r in tr2] == [(r.n, r.steps, r.arrival) for r in tr]


def test_scheduler_respects_capacity_budgets_and_order():
    tr = serve.make_trace(rate=400, duration=0.5, seed=5, n_range=(100, 3000), steps_range=(20, 200))
    fb = FakeBatch(max_systems=6, max_particles=8000, max_cells=100000)
    srv = serve.Server(fb, abi.STEPPER_EULER, abi.PRECISION_FP32C, chunk=10, clock=FakeClock(),
                       limits=(8000, 100000))
    st = srv.run(tr)
    assert st.completed == len(tr)
    assert st.particle_steps == sum(r.work for r in tr)
    for r in tr:
        assert r.admitted_at >= r.arrival
        assert r.finished_at >= r.admitted_at
    # every system ran exactly its own budget, and at most 6 were resident at once
    assert st.max_active <= 6
    assert st.p50_s is not None and st.p99_s >= st.p50_s
    released = [e for e in fb.log if e[0] == "release"]
    assert len(released) == len(tr)


def test_initial_states_are_drawn_once_per_request(monkeypatch):
    """A queue blocked on capacity does not draw the initial states of the
    requests it cannot admit yet: each request's inputs are generated once."""
    calls = []
    orig = serve.Request.inputs

    def counted(self):
        calls.append(self.rid)
        return orig(self)

    monkeypatch.setattr(serve.Request, "inputs", counted)
    tr = serve.make_trace(rate=400, duration=0.5, seed=5, n_range=(100, 3000), steps_range=(20, 200))
    fb = FakeBatch(max_systems=6, max_particles=8000, max_cells=100000)
    srv = serve.Server(fb, abi.STEPPER_EULER, abi.PRECISION_FP32C, chunk=10, clock=FakeClock(),
                       limits=(8000, 100000))
    st = srv.run(tr)
    assert st.completed == len(tr)
    assert sorted(calls) == sorted(r.rid for r in tr)


def test_requests_that_can_never_fit_are_refused():
    tr = serve.make_trace(rate=50, duration=0.2, seed=7, n_range=(100, 200), steps_range=(10, 20))
    big = serve.Request(rid=999, arrival=0.05, model=abi.MODEL_CHIMERA, n=10**6, L=31.6, v0=0.01,
                        sigma=1.0, rho=0.1, alpha=1.4, D_phi=0.0, steps=10, seed=7)
    fb = FakeBatch(4, 5000, 10**6)
    srv = serve.Server(fb, abi.STEPPER_EULER, abi.PRECISION_FP32C, chunk=5, clock=FakeClock(),
                       limits=(5000, 10**6))
    st = srv.run(tr + [big])
    assert st.completed == len(tr)
    assert [r.rid for r in srv.refused] == [999]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32C])
def test_served_results_equal_alone(precision):
    tr = serve.make_trace(rate=300, duration=0.05, seed=11, n_range=(256, 3000),
                          steps_range=(20, 90))
    assert len(tr) >= 6
    stepper = abi.STEPPER_EULER
    with abi.Batch(stepper, precision, 8, 9000, 20000) as b:
        srv = serve.Server(b, stepper, precision, dt=0.01, chunk=16, keep_results=True,
                           limits=(9000, 20000))
        st = srv.run(tr, time_scale=0.2)
    assert st.completed == len(tr)
    assert st.max_active >= 2  # requests overlapped on the device
    for r in tr:
        st0, om = r.inputs()
        with abi.System(r.n, r.params(stepper, precision)) as s:
            s.upload_state(st0)
            if om is not None:
                s.upload_omega(om)
            s.step(0.01, r.steps)
            alone = s.download_state()
        assert np.array_equal(r.result, alone), r.rid
