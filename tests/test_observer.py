"""Observer formats (CPU): frames, summary statistics and restart files as the
reference writes and reads them (Observers/BinaryObserver.cpp:186-234,
ControlEngines/SimulationEngine.cpp:52-73)."""
import math

import numpy as np

from spc2_langevin_integration_gb300 import observer as obs
from tests._helpers import init_state


def _reference_order_parameter(state):
    # the observer's arithmetic one term at a time with float32 scalars
    n = len(state) // 3
    re, im = np.float32(0.0), np.float32(0.0)
    for i in range(n):
        phi = float(state[3 * i + 2])
        re = np.float32(re + np.float32(math.cos(phi)))
        im = np.float32(im + np.float32(math.sin(phi)))
    re, im = np.float32(re / np.float32(n)), np.float32(im / np.float32(n))
    return np.float32(np.hypot(re, im)), np.float32(np.arctan2(im, re))


def test_frames_round_trip(tmp_path):
    st = init_state(300, 1.0, 3)
    o = obs.BinaryObserver(str(tmp_path), 0.01, 1.0, 0.1, 1.45, 0.005, 300, 1.0, trial=2,
                           state_every=2)
    for k in range(5):
        o.save_system_state(st + k, 0.01 * (k + 1))
    assert o.simulation_file.endswith("v0_0.01_sigma_1_rho_0.1_alpha_1.45_Dphi_0.005_N_300_rho0_1_0_2.bin")
    frames = list(obs.read_frames(o.simulation_file, 300))
    assert [t for t, _ in frames] == [float(np.float32(0.01 * k)) for k in (1, 3, 5)]
    for (t, fr), k in zip(frames, (0, 2, 4)):
        assert np.array_equal(fr, (st + k).astype(np.float32))
    raw = open(o.simulation_file, "rb").read()
    assert len(raw) == 3 * 4 * (1 + 900)


def test_summary_statistics_match_the_float_arithmetic(tmp_path):
    st = init_state(500, 1.0, 4)
    st[2::3] *= 0.3  # partly ordered phases
    r, psi = obs.order_parameter_f32(st)
    rr, pp = _reference_order_parameter(st)
    assert r == rr and psi == pp
    o = obs.BinaryObserver(str(tmp_path), 0.01, 1.0, 0.1, 1.45, 0.005, 500, 1.0)
    o.save_summary_statistics(st, 0.25)
    line = open(o.summary_file).read()
    assert line == "%g\t%g\t%g\n" % (0.25, float(rr), float(pp))
    assert len(line.strip().split("\t")) == 3


def test_restart_file(tmp_path):
    st = init_state(200, 2.0, 5)
    p = str(tmp_path / "restart.bin")
    obs.write_restart(p, st)
    back = obs.read_restart(p, 200)
    assert np.array_equal(back, st.astype(np.float32).astype(np.float64))
    # a frame file is not a restart file: its first value is the time
    o = obs.BinaryObserver(str(tmp_path), 0.01, 1.0, 0.1, 1.45, 0.005, 200, 1.0)
    o.save_system_state(st, 7.0)
    assert obs.read_restart(o.simulation_file, 200)[0] == 7.0
