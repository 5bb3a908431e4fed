"""Observer output pinned to the reference's own BinaryObserver (CPU).

tests/golden/observer/*.npz hold what the reference's Observers/BinaryObserver.cpp
wrote in the engine loop of ControlEngines/SimulationEngine.cpp:113-127 (made
by tests/golden/make_golden.py from the reference build): the file names it
builds from the parameters, the .bin frames (float32 t, then the 3N float32
state) and the summary lines (t, |R|, arg R through operator<< on float and
std::complex<float>), with the states of every step.  The drop-in's C++
observer (host/spc_observer.cpp, driven by tests/host/observer_replay.cpp) and
the Python observer (observer.py), fed the same states, must write the same
file names and the same bytes.
"""
import glob
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from spc2_langevin_integration_gb300 import observer as obs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "spc2_langevin_integration_gb300", "host")
CASES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "observer", "*.npz")))


def _load(path):
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    g["bin_name"], g["txt_name"] = str(g["bin_name"]), str(g["txt_name"])
    return g


@pytest.fixture(scope="module")
def replay_exe(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("obs") / "observer_replay")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-o", exe,
                    os.path.join(ROOT, "tests", "host", "observer_replay.cpp"),
                    os.path.join(ROOT, "tests", "host", "fake_spc.cpp"),
                    os.path.join(HOST, "spc_dropin.cpp"), os.path.join(HOST, "spc_observer.cpp"),
                    "-I", os.path.join(ROOT, "include")], check=True, timeout=300)
    return exe


def test_fixtures_present():
    assert len(CASES) == 2


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_cpp_observer_writes_the_reference_files(path, replay_exe, tmp_path):
    g = _load(path)
    n, nsteps = int(g["n"]), int(g["nsteps"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(struct.pack("<2i", nsteps, 0))
        f.write(struct.pack("<9d", float(g["L"]), float(g["t0"]), float(g["dt"]), float(g["v0"]),
                            float(g["sigma"]), float(g["rho"]), float(g["alpha"]), float(g["D_phi"]),
                            float(g["rho_0"])))
        f.write(np.ascontiguousarray(g["state0"], np.float64).tobytes())
        f.write(np.ascontiguousarray(g["trajectory"], np.float64).tobytes())
    out = tmp_path / "out"
    out.mkdir()
    env = dict(os.environ, SPC_N=str(n), SPC_OUTPUT_DIR=str(out))
    r = subprocess.run([replay_exe, str(inp)], capture_output=True, text=True, timeout=60, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sorted(os.listdir(out)) == sorted([g["bin_name"], g["txt_name"]])
    assert open(out / g["bin_name"], "rb").read() == g["bin_bytes"].tobytes()
    assert open(out / g["txt_name"], "rb").read() == g["txt_bytes"].tobytes()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_python_observer_writes_the_reference_files(path, tmp_path):
    g = _load(path)
    n, dt = int(g["n"]), float(g["dt"])
    o = obs.BinaryObserver(str(tmp_path), float(g["v0"]), float(g["sigma"]), float(g["rho"]),
                           float(g["alpha"]), float(g["D_phi"]), n, float(g["rho_0"]))
    t = float(g["t0"])
    o.save_system_state(g["state0"], t)
    for st in g["trajectory"]:
        t += dt
        o.save_system_state(st, t)
        o.save_summary_statistics(st, t)
    del o
    assert sorted(os.listdir(tmp_path)) == sorted([g["bin_name"], g["txt_name"]])
    assert open(tmp_path / g["bin_name"], "rb").read() == g["bin_bytes"].tobytes()
    assert open(tmp_path / g["txt_name"], "rb").read() == g["txt_bytes"].tobytes()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[:-4] for c in CASES])
def test_reference_files_decode(path):
    """The fixtures' frames are the float32 images of the recorded states (a
    check of the fixture itself, independent of either observer)."""
    g = _load(path)
    n = int(g["n"])
    raw = g["bin_bytes"].tobytes()
    frame = 4 * (1 + 3 * n)
    assert len(raw) == frame * (int(g["nsteps"]) + 1)
    states = [g["state0"]] + list(g["trajectory"])
    for k, st in enumerate(states):
        rec = np.frombuffer(raw[k * frame:(k + 1) * frame], np.float32)
        assert np.array_equal(rec[1:], st.astype(np.float32))
