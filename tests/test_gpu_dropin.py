"""The C++ drop-in (host/spc_dropin.hpp, host/spc_observer.hpp) as a
reference-style program uses it: the engine loops of SimulationEngine.cpp:149-161
and SimulationEnginePtr.cpp:106-115 written against the reference's class names
(host/dropin_driver.cpp) for the vector classes, the shared-window classes and
VortexArraysSystemPtr, fed the golden inputs, must reproduce the reference's
golden trajectories and right-hand sides; with SPC_OUTPUT_DIR set, its
observer files must be the bytes the reference's observer writes for those
states."""
import glob
import os

import numpy as np
import pytest

from oracle import pyref
from spc2_langevin_integration_gb300 import observer as obs
from spc2_langevin_integration_gb300.host import build_host
from tests._helpers import golden_cases, load_golden, periodic_diff, va_golden_cases, va_params

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-9
RHS_TOL = 1e-12
VA_RHS_TOL = 1e-11  # of each array's largest magnitude, as for the vortex-arrays C-ABI tests


def _run(g, mode, extra_env=None):
    n, L = int(g["n"]), float(g["L"])
    fam, stepper = int(g["family"]), int(g["stepper"])
    kw = dict(mode=mode, family=fam, stepper=stepper,
              nsteps=int(g["nsteps"]), record_every=int(g["record_every"]),
              D_phi=float(g["D_phi"]), rho=float(g["rho"]), dt=float(g["dt"]),
              k_coef=float(g["k_coef"]), state=g["state0"], k_prev=g["k_prev"],
              k_next_init=g["k_next_init"])
    noise = g["noise"]
    if fam == pyref.FAMILY_VA:
        vp = va_params(g)
        kw.update(v0=vp["velocity"], va=[vp[k] for k in ("mu_plus", "mu_minus", "xi_a", "xi_r", "kappa")])
        if stepper == pyref.STEP_SRK:
            noise = np.concatenate([np.zeros(n), noise])  # the unused frequency draw
    else:
        kw.update(v0=float(g["v0"]), sigma=float(g["sigma"]), alpha=float(g["alpha"]))
        if "omega" in g:
            noise = np.concatenate([g["omega"], noise])
    if mode != 0:
        noise = None  # one right-hand side draws no normals
    return pyref.run_reference(n, L, noise=noise, binary=build_host.build_driver(),
                               extra_env=extra_env, **kw)


def _trajectory(name, extra_env=None):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    frames = _run(g, 0, extra_env=extra_env).reshape(-1, 3 * n)
    ref = np.asarray(g["trajectory"])
    assert frames.shape == ref.shape
    for got, want in zip(frames, ref):
        assert np.abs(periodic_diff(got, want, L)).max() <= TRAJ_TOL
    return g, frames


@pytest.mark.parametrize("name", golden_cases())
def test_dropin_engine_loop_matches_reference_golden(name, tmp_path):
    g, frames = _trajectory(name, extra_env={"SPC_OUTPUT_DIR": str(tmp_path)})
    n = int(g["n"])
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


OBSERVER_CASES = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                               "observer", "*.npz")))


@pytest.mark.parametrize("path", OBSERVER_CASES, ids=[os.path.basename(c)[:-4] for c in OBSERVER_CASES])
def test_dropin_observer_files_are_the_reference_observers(path, tmp_path):
    # the engine loop of SimulationEngine.cpp:113-127 on the GPU path, with the
    # reference's injected normals: its observer files must be the bytes the
    # reference's BinaryObserver wrote for the reference's own run (frames at
    # float32, summary lines through operator<<), under the same names
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    n, L = int(g["n"]), float(g["L"])
    out = pyref.run_reference(n, L, mode=3, family=pyref.FAMILY_VECTOR, stepper=int(g["stepper"]),
                              nsteps=int(g["nsteps"]), t0=float(g["t0"]), dt=float(g["dt"]),
                              state=g["state0"], noise=g["noise"],
                              binary=build_host.build_driver(),
                              extra_env={"SPC_OUTPUT_DIR": str(tmp_path)},
                              **{k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi", "rho_0")})
    frames = out.reshape(-1, 3 * n)
    for got, want in zip(frames, g["trajectory"]):
        assert np.abs(periodic_diff(got, want, L)).max() <= TRAJ_TOL
    assert sorted(os.listdir(tmp_path)) == sorted([str(g["bin_name"]), str(g["txt_name"])])
    assert open(tmp_path / str(g["bin_name"]), "rb").read() == g["bin_bytes"].tobytes()
    assert open(tmp_path / str(g["txt_name"]), "rb").read() == g["txt_bytes"].tobytes()


@pytest.mark.parametrize("name", va_golden_cases())
def test_dropin_vortex_arrays_engine_loop_matches_reference_golden(name):
    # VortexArraysSystemPtr driven by StochasticEulerStepperPtr,
    # StochasticRungeKuttaStepperPtr and RungeKutta4StepperPtr
    _trajectory(name)


def _close(got, want, tol):
    return np.abs(got - want).max() <= tol * max(np.abs(want).max(), 1.0)


@pytest.mark.parametrize("name", [c for c in golden_cases() if load_golden(c)["family"] == 1]
                         + va_golden_cases())
def test_dropin_ptr_rhs_matches_reference_golden(name):
    # both EvaluateRhs forms of ChimeraSystemPtr / VortexArraysSystemPtr on a
    # raw state pointer
    g = load_golden(name)
    n = int(g["n"])
    tol = VA_RHS_TOL if int(g["family"]) == pyref.FAMILY_VA else RHS_TOL * 10
    assert _close(_run(g, 1), g["rhs_rk"], tol)
    out = _run(g, 2)
    d, a = out[:3 * n], out[3 * n:]
    assert _close(d, g["srk_derivative"], tol)
    assert _close(a[0::2], g["srk_additional"][0::2], tol)
    assert _close(a[1::2], g["srk_additional"][1::2], tol)


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


@pytest.mark.parametrize("name", golden_cases() + va_golden_cases())
def test_dropin_device_loop_matches_per_step_loop(name, tmp_path):
    # RunObserved (the engine loop on the device, spc_run) against one DoStep
    # per step: the same recorded states, bit for bit, and byte-identical
    # observer files; both within the golden tolerance of the reference
    g = load_golden(name)
    d_step, d_loop = tmp_path / "step", tmp_path / "loop"
    d_step.mkdir()
    d_loop.mkdir()
    per_step = _run(g, 0, extra_env={"SPC_OUTPUT_DIR": str(d_step)})
    loop = _run(g, 0, extra_env={"SPC_OUTPUT_DIR": str(d_loop), "SPC_DEVICE_LOOP": "1"})
    assert np.array_equal(per_step, loop)
    n, L = int(g["n"]), float(g["L"])
    for got, want in zip(loop.reshape(-1, 3 * n), np.asarray(g["trajectory"])):
        assert np.abs(periodic_diff(got, want, L)).max() <= TRAJ_TOL
    files = sorted(os.listdir(d_step))
    assert files == sorted(os.listdir(d_loop)) and len(files) == 2
    for f in files:
        assert open(d_step / f, "rb").read() == open(d_loop / f, "rb").read(), f
