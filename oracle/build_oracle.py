"""Build recipe for the oracle (test infrastructure, never the product path).

* ``build_restatement()`` compiles the plain-C restatement ``spc_oracle.c``
  into ``oracle/_build/libspc_oracle.so`` with ``-ffp-contract=off`` so that
  no multiply-add is fused (the reference's arithmetic is unfused double).
* ``build_reference()`` compiles the reference's OWN sources, unmodified, in
  place under the reference checkout, together with the forced-include
  prelude and the single-rank MPI stub in ``oracle/ref`` and the driver
  ``oracle/ref/ref_driver.cpp``, into ``oracle/_ref/spc_ref``.  It is only
  possible where the reference checkout exists; its output is used to make the
  golden vectors in ``tests/golden``.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "libspc_oracle.so")
REF_BIN = os.path.join(REF_OUT, "spc_ref")
# The reference checkout: SPC_REFERENCE_ROOT, else a `reference` directory
# beside the repository's own.
REFERENCE_ROOT = (os.environ.get("SPC_REFERENCE_ROOT")
                  or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

# The reference translation units the particle-update path needs.
REF_SOURCES = [
    "Parallelization/Thread.cpp",
    "Parallelization/ThreadSharedMemory.cpp",
    "BoundaryConfiguration/PeriodicBoundaryConditions.cpp",
    "DynamicalSystems/ChimeraSystem.cpp",
    "DynamicalSystems/ChimeraSystemPtr.cpp",
    "Steppers/RungeKutta4Stepper.cpp",
    "Steppers/RungeKutta4StepperPtr.cpp",
    "DynamicalSystems/VortexArraysSystemPtr.cpp",
    "Observers/BinaryObserver.cpp",
]

FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math"]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_restatement(force: bool = False) -> str:
    src = os.path.join(HERE, "spc_oracle.c")
    hdr = os.path.join(HERE, "spc_oracle.h")
    os.makedirs(BUILD, exist_ok=True)
    if not force and _newer(LIB, [src, hdr, __file__]):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", *FP_FLAGS, "-fPIC", "-shared", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE_ROOT, s)) for s in REF_SOURCES)


def build_reference(force: bool = False) -> str | None:
    """Compile the reference path from its own sources; None if absent."""
    if not reference_available():
        return None
    srcs = [os.path.join(REFERENCE_ROOT, s) for s in REF_SOURCES]
    prelude = os.path.join(HERE, "ref", "ref_prelude.hpp")
    stub_dir = os.path.join(HERE, "ref", "stub")
    driver = os.path.join(HERE, "ref", "ref_driver.cpp")
    deps = srcs + [prelude, driver, os.path.join(stub_dir, "mpi.h"), __file__]
    os.makedirs(REF_OUT, exist_ok=True)
    if not force and _newer(REF_BIN, deps):
        return REF_BIN
    tmp = REF_BIN + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", *FP_FLAGS, "-w",
           "-include", prelude, "-I", stub_dir, "-I", REFERENCE_ROOT,
           "-o", tmp, driver, *srcs]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_BIN)
    return REF_BIN


if __name__ == "__main__":
    print(build_restatement(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
