"""Generate the golden vectors in this folder from the reference's own code.

Runs ``oracle/_ref/spc_ref`` (the reference's unmodified sources, built by
``oracle/build_oracle.py`` from the reference checkout) on seeded synthetic
inputs with injected normals, and stores inputs and outputs as .npz.  The
fixtures pin the C restatement (tests/test_oracle.py) and the GPU path
(tests/test_gpu_parity.py) without the reference being present.

    python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyref  # noqa: E402


def init_state(n, L, seed):
    """x, y ~ U[0, L), phi ~ U[-pi, pi) from numpy PCG64(seed)."""
    rng = np.random.default_rng(seed)
    s = np.empty(3 * n)
    s[0::3] = rng.uniform(0.0, L, n)
    s[1::3] = rng.uniform(0.0, L, n)
    s[2::3] = rng.uniform(-np.pi, np.pi, n)
    return s


# name: (n, L, params, family, stepper, nsteps, seed)
CASES = {
    # the Euler configuration: N=1024 in the unit square, rho = 0.1 (10x10 cells)
    "chimera_euler_n1024": (1024, 1.0, dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005),
                            pyref.FAMILY_VECTOR, pyref.STEP_EULER, 50, 0),
    # the vortex configuration at reduced size: alpha = 0, omega ~ N(0, 0.5^2), SRK with frequencies
    "vortex_srk_n512": (512, 1.5, dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01),
                        pyref.FAMILY_PTR, pyref.STEP_SRK, 50, 1),
    # plain SRK (vector classes)
    "chimera_srk_n512": (512, 1.2, dict(v0=0.02, sigma=1.0, rho=0.2, alpha=1.2, D_phi=0.01),
                         pyref.FAMILY_VECTOR, pyref.STEP_SRK, 30, 4),
    # the deterministic RK4 configuration at reduced size (rho = 0.25, D = 0)
    "chimera_rk4_n1024": (1024, 4.0, dict(v0=0.01, sigma=1.0, rho=0.25, alpha=1.45, D_phi=0.0),
                          pyref.FAMILY_VECTOR, pyref.STEP_RK4, 30, 0),
    # rho > L/4: the all-pairs path
    "chimera_allpairs_euler_n200": (200, 0.4, dict(v0=0.01, sigma=1.0, rho=0.12, alpha=1.3,
                                                   D_phi=0.01),
                                    pyref.FAMILY_VECTOR, pyref.STEP_EULER, 40, 5),
    # StochasticEulerStepperPtr (SRK-form right-hand side, phase noise sqrt(2D) sqrt(dt) xi)
    "chimera_eulerptr_n512": (512, 1.0, dict(v0=0.01, sigma=1.0, rho=0.125, alpha=1.45,
                                             D_phi=0.005),
                              pyref.FAMILY_PTR, pyref.STEP_EULER, 30, 6),
}


def make_case(name, n, L, prm, family, stepper, nsteps, seed, dt=0.01):
    rng = np.random.default_rng(1000 + seed)
    state0 = init_state(n, L, seed)
    m = {pyref.STEP_EULER: 1, pyref.STEP_SRK: 2, pyref.STEP_RK4: 0}[stepper]
    noise = rng.standard_normal(nsteps * n * m)
    omega = rng.normal(0.0, 0.5, n) if (family == pyref.FAMILY_PTR and stepper == pyref.STEP_SRK) \
        else None
    feed = noise if omega is None else np.concatenate([omega, noise])
    traj = pyref.run_reference(n, L, mode=pyref.MODE_RUN, family=family, stepper=stepper,
                               nsteps=nsteps, record_every=25, dt=dt, state=state0,
                               noise=feed if feed.size else None, **prm)
    traj = traj.reshape(-1, 3 * n)
    # right-hand sides at the initial state
    k_prev = rng.normal(0.0, 0.05, 3 * n)
    k_next_init = rng.normal(0.0, 1.0, 3 * n)
    rhs_rk = pyref.run_reference(n, L, mode=pyref.MODE_RHS_RK, family=pyref.FAMILY_VECTOR,
                                 dt=dt, k_coef=0.5, state=state0, k_prev=k_prev,
                                 k_next_init=k_next_init, **prm)
    srk = pyref.run_reference(n, L, mode=pyref.MODE_RHS_SRK, family=pyref.FAMILY_VECTOR, dt=dt,
                              state=state0, **prm)
    out = dict(n=n, L=L, dt=dt, family=family, stepper=stepper, nsteps=nsteps, record_every=25,
               state0=state0, noise=noise, trajectory=traj, k_prev=k_prev,
               k_next_init=k_next_init, k_coef=0.5, rhs_rk=rhs_rk,
               srk_derivative=srk[:3 * n], srk_additional=srk[3 * n:], **prm)
    if omega is not None:
        out["omega"] = omega
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return traj.shape


# VortexArraysSystemPtr: the reference's vortex-array configuration
# (SimulationEnginePtr.cpp:131-139) in a unit box: velocity 0.1, mu+- 100,
# xi_a 0.04, xi_r 0.02, D 0.01, kappa 20, rho 0.2
VA_PRM = dict(velocity=0.1, mu_plus=100.0, mu_minus=100.0, xi_a=0.04, xi_r=0.02, D_phi=0.01,
              kappa=20.0, rho=0.2)
# name: (n, L, stepper, nsteps, seed)
VA_CASES = {
    "va_srk_n1024": (1024, 1.0, pyref.STEP_SRK, 30, 7),
    "va_rk4_n512": (512, 1.0, pyref.STEP_RK4, 20, 8),
    "va_eulerptr_n512": (512, 1.0, pyref.STEP_EULER, 20, 9),
    "va_allpairs_srk_n150": (150, 0.6, pyref.STEP_SRK, 20, 10),  # rho > L/4
}


def make_va_case(name, n, L, stepper, nsteps, seed, dt=0.01):
    rng = np.random.default_rng(2000 + seed)
    state0 = init_state(n, L, seed)
    m = {pyref.STEP_EULER: 1, pyref.STEP_SRK: 2, pyref.STEP_RK4: 0}[stepper]
    noise = rng.standard_normal(nsteps * n * m)
    # the SRK-Ptr constructor draws N frequencies first (unused by this model)
    feed = np.concatenate([np.zeros(n), noise]) if stepper == pyref.STEP_SRK else noise
    va = [VA_PRM[k] for k in ("mu_plus", "mu_minus", "xi_a", "xi_r", "kappa")]
    common = dict(family=pyref.FAMILY_VA, v0=VA_PRM["velocity"], rho=VA_PRM["rho"],
                  D_phi=VA_PRM["D_phi"], dt=dt, va=va)
    traj = pyref.run_reference(n, L, mode=pyref.MODE_RUN, stepper=stepper, nsteps=nsteps,
                               record_every=10, state=state0,
                               noise=feed if feed.size else None, **common)
    traj = traj.reshape(-1, 3 * n)
    k_prev = rng.normal(0.0, 0.05, 3 * n)
    k_next_init = rng.normal(0.0, 1.0, 3 * n)
    rhs_rk = pyref.run_reference(n, L, mode=pyref.MODE_RHS_RK, k_coef=0.5, state=state0,
                                 k_prev=k_prev, k_next_init=k_next_init, **common)
    srk = pyref.run_reference(n, L, mode=pyref.MODE_RHS_SRK, state=state0, **common)
    out = dict(n=n, L=L, dt=dt, family=pyref.FAMILY_VA, stepper=stepper, nsteps=nsteps,
               record_every=10, state0=state0, noise=noise, trajectory=traj, k_prev=k_prev,
               k_next_init=k_next_init, k_coef=0.5, rhs_rk=rhs_rk, srk_derivative=srk[:3 * n],
               srk_additional=srk[3 * n:], **VA_PRM)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return traj.shape


# The reference's BinaryObserver (Observers/BinaryObserver.cpp) in the engine
# loop of SimulationEngine.cpp:113-127: its .bin frames and summary lines for
# a short run, written under the file names it builds from the parameters.
# name: (n, L, params, stepper, nsteps, seed, t0)
OBSERVER_CASES = {
    "observer_chimera_euler_n256": (256, 0.5, dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45,
                                                   D_phi=0.005, rho_0=1.0),
                                    pyref.STEP_EULER, 12, 11, 0.0),
    "observer_chimera_srk_n200": (200, 0.8, dict(v0=0.02, sigma=0.75, rho=0.15, alpha=0.3,
                                                 D_phi=0.0125, rho_0=0.5),
                                  pyref.STEP_SRK, 10, 12, 2.5),
}


def make_observer_case(name, n, L, prm, stepper, nsteps, seed, t0, dt=0.01):
    import tempfile
    rng = np.random.default_rng(3000 + seed)
    state0 = init_state(n, L, seed)
    m = {pyref.STEP_EULER: 1, pyref.STEP_SRK: 2, pyref.STEP_RK4: 0}[stepper]
    noise = rng.standard_normal(nsteps * n * m)
    with tempfile.TemporaryDirectory() as td:
        traj = pyref.run_reference(n, L, mode=pyref.MODE_OBSERVE, family=pyref.FAMILY_VECTOR,
                                   stepper=stepper, nsteps=nsteps, t0=t0, dt=dt, state=state0,
                                   noise=noise, extra_env={"SPC_REF_OUT_DIR": td}, **prm)
        files = sorted(os.listdir(td))
        assert len(files) == 2, files
        bin_name = [f for f in files if f.endswith(".bin")][0]
        txt_name = [f for f in files if f.endswith(".txt")][0]
        bin_bytes = np.frombuffer(open(os.path.join(td, bin_name), "rb").read(), np.uint8)
        txt_bytes = np.frombuffer(open(os.path.join(td, txt_name), "rb").read(), np.uint8)
    out = dict(n=n, L=L, dt=dt, t0=t0, stepper=stepper, nsteps=nsteps, state0=state0, noise=noise,
               trajectory=traj.reshape(-1, 3 * n), bin_name=bin_name, txt_name=txt_name,
               bin_bytes=bin_bytes, txt_bytes=txt_bytes, **prm)
    os.makedirs(os.path.join(HERE, "observer"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "observer", name + ".npz"), **out)
    return bin_name, bin_bytes.size, txt_bytes.size


def main():
    which = sys.argv[1:]
    for name, (n, L, prm, stepper, nsteps, seed, t0) in OBSERVER_CASES.items():
        if which and name not in which:
            continue
        print(name, make_observer_case(name, n, L, prm, stepper, nsteps, seed, t0))
    for name, (n, L, prm, family, stepper, nsteps, seed) in CASES.items():
        if which and name not in which:
            continue
        shape = make_case(name, n, L, prm, family, stepper, nsteps, seed)
        print(name, shape)
    for name, (n, L, stepper, nsteps, seed) in VA_CASES.items():
        if which and name not in which:
            continue
        shape = make_va_case(name, n, L, stepper, nsteps, seed)
        print(name, shape)


if __name__ == "__main__":
    main()
