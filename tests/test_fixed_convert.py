"""The FP32X form's integer-only fixed-point -> double conversion
(csrc/spc_fixed.h, used on the device by the neighbour kernels) against the C
library's round-to-nearest conversion, bit for bit, on the CPU: every
magnitude, halfway cases, carries into the exponent, INT64_MIN, and the
fixed-point exponents 0..64 (the form uses 11..52)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fixed_to_double_is_round_to_nearest(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "fixed_convert")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-o", exe,
                    os.path.join(ROOT, "tests", "host", "fixed_convert.cpp"),
                    "-I", os.path.join(ROOT, "spc2_langevin_integration_gb300", "csrc")],
                   check=True, timeout=300)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok "), out.stdout
