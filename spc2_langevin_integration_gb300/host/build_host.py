"""Build recipe for the C++ drop-in adapters' driver (links the CUDA library)."""
from __future__ import annotations

import os
import subprocess

from .. import build as lib_build

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "spc_dropin_driver")
SOURCES = [os.path.join(HERE, f) for f in ("dropin_driver.cpp", "spc_dropin.cpp", "spc_observer.cpp")]


def build_driver(force: bool = False) -> str:
    lib = lib_build.build_library()
    deps = SOURCES + [os.path.join(HERE, "spc_dropin.hpp"), os.path.join(HERE, "spc_observer.hpp"),
                      lib, __file__]
    if not force and os.path.exists(OUT) and all(
            os.path.getmtime(d) <= os.path.getmtime(OUT) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    libdir = os.path.dirname(lib)
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-o", tmp, *SOURCES,
           "-I", os.path.join(lib_build.ROOT, "include"), "-L", libdir, "-lspc_gb300",
           "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT
