"""The allocation-free right-hand side, spc_rhs_srk_noalloc.

Callers whose device memory belongs to another component's pool, or whose
loop must not stall on a cudaMalloc, take the SRK right-hand side from
spc_rhs_srk_noalloc: they pass device buffers in and out, and the library keeps
every intermediate in one static device array instead of allocating.  This
file calls it through the C-ABI twice in a row, with different inputs and box
sizes so the second call runs on scratch that still holds the first call's
data, and checks each result against the handle API's spc_rhs_srk with the
tolerance of the other right-hand-side tests.
"""
import ctypes as C

import numpy as np
import pytest

from tests._helpers import alignment_scale, init_state

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12


def _noalloc():
    from spc2_langevin_integration_gb300 import abi
    L = abi.lib()
    f = L.spc_rhs_srk_noalloc
    f.argtypes = [C.POINTER(abi.Params), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return abi, L, f


def _check(n, state, d, a, d_ref, a_ref, prm, L):
    from oracle import pyoracle as po
    o = po.OracleSystem(n, L, **prm)
    off, idx = o.neighbour_lists(state)
    scale, counts = alignment_scale(state, off, idx, prm["sigma"], prm["alpha"])
    d, d_ref = d.reshape(-1, 3), d_ref.reshape(-1, 3)
    assert np.all(np.abs(d[:, :2] - d_ref[:, :2]) <= RHS_TOL * abs(prm["v0"]))
    assert np.all(np.abs(d[:, 2] - d_ref[:, 2]) <= RHS_TOL * np.maximum(np.abs(d_ref[:, 2]), scale))
    # additional_derivative: both come from the same kernels; hold them to the
    # same relative rule against their own magnitude (plus the phase-rate scale)
    a, a_ref = a.reshape(-1, 2), a_ref.reshape(-1, 2)
    mag = np.maximum(np.abs(a_ref), (np.sqrt(2 * prm["D_phi"]) + prm["sigma"]) * 1e-3)
    assert np.all(np.abs(a - a_ref) <= RHS_TOL * mag)


def test_noalloc_rhs_matches_handle_rhs_on_two_calls():
    torch = pytest.importorskip("torch")
    abi, L, f = _noalloc()
    cases = [
        (1024, 1.0, dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005), 41),
        (2048, 2.0, dict(v0=0.02, sigma=2.0, rho=0.15, alpha=0.3, D_phi=0.01), 42),
    ]
    for n, Lbox, prm, seed in cases:
        p = abi.make_params(L=Lbox, stepper=abi.STEPPER_SRK, **prm)
        state = init_state(n, Lbox, seed)
        with abi.System(n, p) as s:
            s.upload_state(state)
            d_ref, a_ref = s.rhs_srk()
        dev_state = torch.tensor(state, dtype=torch.float64, device="cuda")
        dev_d = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
        dev_a = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = f(C.byref(p), n, dev_state.data_ptr(), dev_d.data_ptr(), dev_a.data_ptr(), None)
        assert rc == 0, L.spc_last_error(None)
        torch.cuda.synchronize()
        _check(n, state, dev_d.cpu().numpy(), dev_a.cpu().numpy(), d_ref, a_ref, prm, Lbox)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    abi, L, f = _noalloc()
    p = abi.make_params(L=10.0, v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005,
                        stepper=abi.STEPPER_SRK)
    # too many particles
    assert f(C.byref(p), 8193, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None) == -7
    assert b"8192" in L.spc_last_error(None)
    # too many cells: int(L/rho)^2 = 200^2
    p = abi.make_params(L=20.0, v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005,
                        stepper=abi.STEPPER_SRK)
    assert f(C.byref(p), 1024, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None) == -7
