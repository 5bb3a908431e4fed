"""The ctypes mirrors of the C-ABI's structs (abi.Params, abi.Tuning,
abi.BatchConfig) against the header, compiled here with the host C compiler:
every field's offset and each struct's size must agree, or a Python caller
would pass garbage through the boundary.  CPU only."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from spc2_langevin_integration_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "spc_params": abi.Params,
    "spc_tuning": abi.Tuning,
    "spc_batch_config": abi.BatchConfig,
}


def test_ctypes_structs_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "spc_gb300.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", exe], check=True, timeout=120)
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=60).stdout
    got = {}
    for line in out.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for name, cls in STRUCTS.items():
        assert got[(name, "size")] == C.sizeof(cls), name
        for field, _ in cls._fields_:
            assert got[(name, field)] == getattr(cls, field).offset, (name, field)
