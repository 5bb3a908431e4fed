"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every
function include/spc_gb300.h declares, and rejects bad parameters before it
touches a GPU."""
import ctypes as C
import shutil

import pytest

from spc2_langevin_integration_gb300 import abi, build

needs_nvcc = pytest.mark.skipif(shutil.which("nvcc") is None and not build.up_to_date(),
                                reason="no nvcc and no prebuilt library")


@needs_nvcc
def test_library_builds_and_loads():
    path = build.build_library()
    assert path.endswith("libspc_gb300.so")
    L = abi.lib()
    assert L.spc_abi_version() == 4


@needs_nvcc
def test_every_declared_function_is_exported():
    L = abi.lib()
    names = abi.header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


@needs_nvcc
@pytest.mark.parametrize("field,value", [
    ("L", 0.0), ("rho", -1.0), ("D_phi", -0.1), ("stepper", 9), ("model", 7),
    ("precision", 5), ("neighbour", 3),
])
def test_invalid_parameters_rejected_without_gpu(field, value):
    L = abi.lib()
    p = abi.make_params(L=1.0, v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
    setattr(p, field, value)
    h = C.c_void_p()
    rc = L.spc_create(C.byref(p), 16, C.byref(h))
    assert rc == -1
    assert not h.value
    assert L.spc_last_error(None)


@needs_nvcc
def test_vortex_rk4_and_nonpositive_n_rejected():
    L = abi.lib()
    h = C.c_void_p()
    # natural frequencies enter the Euler and SRK drifts only
    p = abi.make_params(L=1.0, v0=0.01, sigma=1.0, rho=0.1, alpha=0.0, D_phi=0.005,
                        model=abi.MODEL_VORTEX, stepper=abi.STEPPER_RK4)
    assert L.spc_create(C.byref(p), 16, C.byref(h)) == -1
    p = abi.make_params(L=1.0, v0=0.01, sigma=1.0, rho=0.1, alpha=0.0, D_phi=0.005)
    assert L.spc_create(C.byref(p), 0, C.byref(h)) == -1
    p = abi.make_params(L=1.0, v0=0.01, sigma=1.0, rho=0.1, alpha=0.0, D_phi=0.005,
                        neighbour=abi.NEIGHBOUR_VERLET, skin=0.0)
    assert L.spc_create(C.byref(p), 16, C.byref(h)) == -1


def test_header_declares_the_boundary():
    names = abi.header_functions()
    for required in ("spc_create", "spc_destroy", "spc_upload_state", "spc_download_state",
                     "spc_step", "spc_rhs_rk", "spc_rhs_srk", "spc_neighbours",
                     "spc_inject_noise", "spc_export_noise", "spc_order_params"):
        assert required in names
