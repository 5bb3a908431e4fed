"""The allocation-free right-hand side, spc_rhs_srk_noalloc.

Callers whose device memory belongs to another component's pool, or whose
loop must not stall on a cudaMalloc, take the SRK right-hand side from
spc_rhs_srk_noalloc: they pass device buffers in and out, and the library keeps
every intermediate in one static device array instead of allocating.

This file calls it through the C-ABI:
* against the reference's own SRK derivative and additional derivative (the
  golden vectors made from the reference build), every Chimera fixture in
  turn, so each call runs on scratch that still holds the previous call's
  data, with the tolerance of the other right-hand-side tests;
* against the handle API's spc_rhs_srk on the shapes the fixtures do not
  reach: the FP32C form, all pairs, more than 2,048 cells (a two-pass radix
  sort), sparse cells, and the vortex model, each twice in a row;
* with a vortex-arrays system and with sizes beyond its limits, which it must
  refuse.
"""
import ctypes as C

import numpy as np
import pytest

from tests._helpers import alignment_scale, golden_cases, init_state, load_golden

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
FP32C_TOL = 2e-6  # the FP32C right-hand-side bound of the parity tests


def _noalloc():
    from spc2_langevin_integration_gb300 import abi
    L = abi.lib()
    f = L.spc_rhs_srk_noalloc
    f.argtypes = [C.POINTER(abi.Params), C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    f.restype = C.c_int
    return abi, L, f


def _call(f, L, p, n, state):
    torch = pytest.importorskip("torch")
    dev_state = torch.tensor(state, dtype=torch.float64, device="cuda")
    dev_d = torch.full((3 * n,), float("nan"), dtype=torch.float64, device="cuda")
    dev_a = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = f(C.byref(p), n, dev_state.data_ptr(), dev_d.data_ptr(), dev_a.data_ptr(), None)
    assert rc == 0, L.spc_last_error(None)
    torch.cuda.synchronize()
    return dev_d.cpu().numpy(), dev_a.cpu().numpy()


def _scales(state, prm, n, L, d_ref):
    """Per-particle error scales of the phase rate and of both additional
    derivative components (as the golden right-hand-side test uses)."""
    from oracle import pyoracle as po
    o = po.OracleSystem(n, L, **prm)
    off, idx = o.neighbour_lists(state)
    scale, counts = alignment_scale(state, off, idx, prm["sigma"], prm["alpha"])
    phi = state[2::3]
    owner = np.repeat(np.arange(n), np.diff(off))
    c = np.abs(np.cos(phi[idx] - phi[owner] - prm["alpha"]))
    nn = np.maximum(counts, 1)
    rate = d_ref.reshape(-1, 3)[:, 2]
    s0 = np.sqrt(2 * prm["D_phi"]) * np.bincount(owner, c, n) / nn
    s1 = np.bincount(owner, np.abs(rate[idx] - rate[owner]) * c, n) / nn + \
        2 * prm["D_phi"] * np.abs(rate)
    return scale, s0, s1


def _check(d, a, d_ref, a_ref, scales, v0, tol):
    scale, s0, s1 = scales
    d, d_ref = d.reshape(-1, 3), d_ref.reshape(-1, 3)
    a, a_ref = a.reshape(-1, 2), a_ref.reshape(-1, 2)
    assert np.all(np.abs(d[:, :2] - d_ref[:, :2]) <= tol * abs(v0) + 1e-300)
    assert np.all(np.abs(d[:, 2] - d_ref[:, 2]) <= tol * np.maximum(np.abs(d_ref[:, 2]), scale) + 1e-300)
    assert np.all(np.abs(a[:, 0] - a_ref[:, 0]) <= tol * np.maximum(np.abs(a_ref[:, 0]), s0) + 1e-300)
    assert np.all(np.abs(a[:, 1] - a_ref[:, 1]) <= tol * np.maximum(np.abs(a_ref[:, 1]), s1) + 1e-300)


def test_noalloc_rhs_matches_reference_golden_vectors():
    abi, L, f = _noalloc()
    names = golden_cases()
    assert len(names) >= 2
    for name in names:  # consecutive calls, each on the previous call's scratch
        g = load_golden(name)
        n, Lbox = int(g["n"]), float(g["L"])
        prm = {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}
        # the right-hand side is the ChimeraSystem's (a vortex fixture's
        # frequencies enter only its stepper)
        p = abi.make_params(L=Lbox, stepper=abi.STEPPER_SRK, **prm)
        d, a = _call(f, L, p, n, g["state0"])
        _check(d, a, g["srk_derivative"], g["srk_additional"],
               _scales(g["state0"], prm, n, Lbox, g["srk_derivative"]), prm["v0"], RHS_TOL)


CASES = [
    # (name, n, L, params, precision, model)
    ("fp32c", 2048, 2.0, dict(v0=0.02, sigma=2.0, rho=0.15, alpha=0.3, D_phi=0.01), "fp32c", "chimera"),
    ("all_pairs", 300, 1.0, dict(v0=0.01, sigma=1.0, rho=0.3, alpha=1.45, D_phi=0.005), "fp64", "chimera"),
    ("cells_14400", 8192, 12.0, dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005), "fp64", "chimera"),
    ("sparse", 600, 6.0, dict(v0=0.01, sigma=1.0, rho=0.25, alpha=1.2, D_phi=0.01), "fp64", "chimera"),
    ("vortex", 4096, 4.0, dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01), "fp64", "vortex"),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_rhs_matches_handle_rhs_on_two_calls(case):
    abi, L, f = _noalloc()
    name, n, Lbox, prm, prec, model = case
    precision = abi.PRECISION_FP32C if prec == "fp32c" else abi.PRECISION_FP64
    mdl = abi.MODEL_VORTEX if model == "vortex" else abi.MODEL_CHIMERA
    p = abi.make_params(L=Lbox, stepper=abi.STEPPER_SRK, precision=precision, model=mdl, **prm)
    # two different states of the same shape, one call after the other
    for seed in (61, 62):
        state = init_state(n, Lbox, seed)
        with abi.System(n, p) as s:
            s.upload_state(state)
            if mdl == abi.MODEL_VORTEX:
                s.upload_omega(np.random.default_rng(seed).normal(0.0, 0.5, n))
            d_ref, a_ref = s.rhs_srk()
        d, a = _call(f, L, p, n, state)
        tol = FP32C_TOL if prec == "fp32c" else RHS_TOL
        _check(d, a, d_ref, a_ref, _scales(state, prm, n, Lbox, d_ref), prm["v0"], tol)


def test_noalloc_refuses_the_vortex_arrays_model():
    abi, L, f = _noalloc()
    p = abi.make_va_params(L=2.0, velocity=0.1, mu_plus=100.0, mu_minus=100.0, xi_a=0.04,
                           xi_r=0.02, D_phi=0.01, kappa=20.0, rho=0.2, stepper=abi.STEPPER_SRK)
    assert f(C.byref(p), 512, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), None) == -1
    assert b"vortex-arrays" in L.spc_last_error(None)


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
