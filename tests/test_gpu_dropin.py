"""The C++ drop-in (host/spc_dropin.hpp, host/spc_observer.hpp) as a
reference-style program uses it: the engine loop of SimulationEngine.cpp:149-161
written against the reference's class names (host/dropin_driver.cpp), fed the
golden inputs, must reproduce the reference's golden trajectories and
right-hand sides; with SPC_OUTPUT_DIR set, its observer files must be the
bytes the reference's observer writes for those states."""
import os

import numpy as np
import pytest

from oracle import pyref
from spc2_langevin_integration_gb300 import observer as obs
from spc2_langevin_integration_gb300.host import build_host
from tests._helpers import golden_cases, load_golden, periodic_diff

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-9
RHS_TOL = 1e-12


def _run(g, mode, extra_env=None):
    n, L = int(g["n"]), float(g["L"])
    kw = dict(mode=mode, family=int(g["family"]), stepper=int(g["stepper"]),
              nsteps=int(g["nsteps"]), record_every=int(g["record_every"]),
              v0=float(g["v0"]), sigma=float(g["sigma"]), rho=float(g["rho"]),
              alpha=float(g["alpha"]), D_phi=float(g["D_phi"]), dt=float(g["dt"]),
              k_coef=float(g["k_coef"]), state=g["state0"], k_prev=g["k_prev"],
              k_next_init=g["k_next_init"])
    noise = g["noise"]
    if "omega" in g:
        noise = np.concatenate([g["omega"], noise])
    return pyref.run_reference(n, L, noise=noise, binary=build_host.build_driver(),
                               extra_env=extra_env, **kw)


def _runnable(name):
    g = load_golden(name)
    # the driver runs the vector classes and the vortex SRK-Ptr form
    return int(g["family"]) == 0 or (int(g["family"]) == 1 and int(g["stepper"]) == 1)


@pytest.mark.parametrize("name", [c for c in golden_cases() if _runnable(c)])
def test_dropin_engine_loop_matches_reference_golden(name, tmp_path):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    out = _run(g, 0, extra_env={"SPC_OUTPUT_DIR": str(tmp_path)})
    frames = out.reshape(-1, 3 * n)
    ref = np.asarray(g["trajectory"])
    assert frames.shape == ref.shape
    for got, want in zip(frames, ref):
        assert np.abs(periodic_diff(got, want, L)).max() <= TRAJ_TOL
    # observer files: one frame and one summary line after every step; the
    # recorded frames must be the float32 images of the driver's states
    bins = [f for f in os.listdir(tmp_path) if f.endswith(".bin")]
    txts = [f for f in os.listdir(tmp_path) if f.startswith("summary_statistics_")]
    assert len(bins) == 1 and len(txts) == 1
    saved = list(obs.read_frames(str(tmp_path / bins[0]), n))
    nsteps, every = int(g["nsteps"]), int(g["record_every"])
    assert len(saved) == nsteps
    lines = open(tmp_path / txts[0]).read().splitlines()
    assert len(lines) == nsteps
    recorded = [k for k in range(1, nsteps + 1) if (every > 0 and k % every == 0) or k == nsteps]
    t = 0.0
    for k in range(1, nsteps + 1):
        t += float(g["dt"])
        if k in recorded:
            st = frames[recorded.index(k)]
            tf, fr = saved[k - 1]
            assert tf == float(np.float32(t))
            assert np.array_equal(fr, st.astype(np.float32))
            assert lines[k - 1] + "\n" == obs.summary_line(t, st)


@pytest.mark.parametrize("name", [c for c in golden_cases() if load_golden(c)["family"] == 0])
def test_dropin_rhs_matches_reference_golden(name):
    g = load_golden(name)
    n = int(g["n"])
    kn = _run(g, 1)
    want = g["rhs_rk"]
    scale = np.maximum(np.abs(want), 1.0)
    assert np.all(np.abs(kn - want) <= RHS_TOL * scale * 10)
    out = _run(g, 2)
    d, a = out[:3 * n], out[3 * n:]
    assert np.all(np.abs(d - g["srk_derivative"]) <= RHS_TOL * np.maximum(np.abs(g["srk_derivative"]), 1.0) * 10)
    assert np.all(np.abs(a - g["srk_additional"]) <= RHS_TOL * np.maximum(np.abs(g["srk_additional"]), 1.0) * 10)
