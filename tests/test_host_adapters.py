"""The C++ drop-in adapters' host logic on the CPU: tests/host/adapter_test.cpp
drives ChimeraSystem / VortexArraysSystem and their steppers against a
host-memory stand-in of the C-ABI (tests/host/fake_spc.cpp) and checks which
state and frequencies reach which library handle, and that a failed step or a
throwing observer leaves the caller's state in charge of the next call; and
that the engine loop on the device (RunObserved) writes the observer files of
the reference's per-step loop byte for byte."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "spc2_langevin_integration_gb300", "host")


def test_adapters_against_a_host_stand_in(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "adapter_test")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-o", exe,
                    os.path.join(ROOT, "tests", "host", "adapter_test.cpp"),
                    os.path.join(ROOT, "tests", "host", "fake_spc.cpp"),
                    os.path.join(HOST, "spc_dropin.cpp"), os.path.join(HOST, "spc_observer.cpp"),
                    "-I", os.path.join(ROOT, "include")], check=True, timeout=300)
    env = dict(os.environ, SPC_OUTPUT_DIR=str(tmp_path))
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("ok ") == 5, out.stdout
