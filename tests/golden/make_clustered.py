"""Make tests/golden/states/vortex_clustered_n65536.npz: a clustered input state.

The vortex workload (N = 65,536 in L = 8, v0 = 0.02, sigma = 2, rho = 0.25,
alpha = 0, D = 0.01, omega ~ N(0, 0.5^2), SRK dt = 0.005, initial state and
frequencies from numpy PCG64(1)) clusters as it runs: cells that start with
~64 particles hold several hundred after a few thousand steps, which sends
the neighbour kernels into their multi-round staging, FIFO-drain and
row-overflow paths.  This script runs the plain FP64 form for 4,000 steps
(library Philox noise, seed 1) on a GPU and stores the state and frequencies.
The fixture is an input: the dense-state parity tests compare the GPU path on
it against the oracle, so how the state was reached does not enter them.

    python tests/golden/make_clustered.py [out.npz]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from spc2_langevin_integration_gb300 import abi  # noqa: E402

N, L, STEPS, DT, SEED = 65536, 8.0, 4000, 0.005, 1
PRM = dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01)


def initial_state():
    rng = np.random.default_rng(SEED)
    st = np.empty(3 * N)
    st[0::3] = rng.uniform(0.0, L, N)
    st[1::3] = rng.uniform(0.0, L, N)
    st[2::3] = rng.uniform(-np.pi, np.pi, N)
    omega = rng.normal(0.0, 0.5, N)
    return st, omega


def main():
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "states", "vortex_clustered_n65536.npz")
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    st, omega = initial_state()
    p = abi.make_params(L=L, stepper=abi.STEPPER_SRK, model=abi.MODEL_VORTEX,
                        precision=abi.PRECISION_FP64, seed=SEED, **PRM)
    with abi.System(N, p) as s:
        s.upload_state(st)
        s.upload_omega(omega)
        for _ in range(STEPS // 100):
            s.step(DT, 100, graph=True)
        state = s.download_state()
    np.savez_compressed(out, n=N, L=L, steps=STEPS, dt=DT, seed=SEED, state=state, omega=omega,
                        **PRM)
    print(out)


if __name__ == "__main__":
    main()
