"""GPU parity of the CUDA path (through the C-ABI) against the oracle and the
reference's golden vectors.

Tolerances (the plain FP64 form's contract):
* neighbour sets: bit-exact, same indices in the same visiting order;
* right-hand sides: |delta| <= 1e-12 * max(|value|, scale), where for a phase
  rate scale = (sigma / n_i) sum_j |sin(phi_j - phi_i - alpha)| (a sum that
  nearly cancels has no meaningful pure relative error; CUDA's and glibc's
  sin/cos differ in the last ulp);
* trajectories: |delta| <= 1e-9 after up to 100 steps (x, y by minimum image).
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from spc2_langevin_integration_gb300 import abi
from tests._helpers import alignment_scale, golden_cases, init_state, load_golden, periodic_diff
from tests.test_oracle import PHILOX_KAT

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
TRAJ_TOL = 1e-9
PRM0 = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)


# neighbour-pass kernels: cell-tile (one CTA per cell) and warp-per-cell;
# the value is the SPARSE_BELOW tuning that sends every system to that kernel
KERNELS = {"tile": 0.0, "warp": 1e9}


def gpu(n, L, prm, stepper, model=abi.MODEL_CHIMERA, precision=abi.PRECISION_FP64,
        neighbour=abi.NEIGHBOUR_CELL, flags=0, seed=0, kernel=None):
    p = abi.make_params(L=L, stepper=stepper, model=model, precision=precision,
                        neighbour=neighbour, flags=flags, seed=seed, **prm)
    s = abi.System(n, p)
    if kernel is not None:
        s.set_tuning(abi.TUNE_SPARSE_BELOW, KERNELS[kernel])
    return s


def golden_stepper(g):
    fam, stp = int(g["family"]), int(g["stepper"])
    if stp == 0:
        return abi.STEPPER_EULER if fam == 0 else abi.STEPPER_EULER_PTR
    return abi.STEPPER_SRK if stp == 1 else abi.STEPPER_RK4


def golden_params(g):
    return {k: float(g[k]) for k in ("v0", "sigma", "rho", "alpha", "D_phi")}


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_device_philox_known_answers(ctr, key, expect):
    assert abi.philox4x32_10(ctr, key) == expect


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", golden_cases())
def test_trajectory_matches_reference_golden(name, kernel):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    model = abi.MODEL_VORTEX if "omega" in g else abi.MODEL_CHIMERA
    with gpu(n, L, golden_params(g), golden_stepper(g), model=model, kernel=kernel) as s:
        s.upload_state(g["state0"])
        if "omega" in g:
            s.upload_omega(g["omega"])
        if s.noise_per_particle:
            s.inject_noise(g["noise"])
        every, nsteps = int(g["record_every"]), int(g["nsteps"])
        frames, done = [], 0
        while done < nsteps:
            k = min(every - done % every, nsteps - done)
            s.step(float(g["dt"]), k)
            done += k
            frames.append(s.download_state())
    for got, ref in zip(frames, g["trajectory"]):
        assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL


def _phase_rate_ok(got, ref, scale, v0):
    got, ref = got.reshape(-1, 3), ref.reshape(-1, 3)
    assert np.all(np.abs(got[:, :2] - ref[:, :2]) <= RHS_TOL * abs(v0) + 1e-300)
    tol = RHS_TOL * np.maximum(np.abs(ref[:, 2]), scale)
    bad = np.abs(got[:, 2] - ref[:, 2]) > tol
    assert not bad.any(), (np.flatnonzero(bad)[:5], got[bad][:3], ref[bad][:3])


@pytest.mark.parametrize("kernel", sorted(KERNELS))
@pytest.mark.parametrize("name", golden_cases())
def test_rhs_matches_reference_golden(name, kernel):
    g = load_golden(name)
    n, L = int(g["n"]), float(g["L"])
    prm = golden_params(g)
    o = po.OracleSystem(n, L, **prm)
    with gpu(n, L, prm, abi.STEPPER_RK4, kernel=kernel) as s:
        s.upload_state(g["state0"])
        kn = s.rhs_rk(g["k_prev"], float(g["k_coef"]), float(g["dt"]), g["k_next_init"])
        stage = g["state0"] + float(g["k_coef"]) * float(g["dt"]) * g["k_prev"]
        off, idx = o.neighbour_lists(stage)
        scale, counts = alignment_scale(stage, off, idx, prm["sigma"], prm["alpha"])
        _phase_rate_ok(kn, g["rhs_rk"], scale, prm["v0"])
        iso = counts == 0
        assert np.array_equal(kn[2::3][iso], g["k_next_init"][2::3][iso])
        d, a = s.rhs_srk()
    off, idx = o.neighbour_lists(g["state0"])
    scale, counts = alignment_scale(g["state0"], off, idx, prm["sigma"], prm["alpha"])
    _phase_rate_ok(d, g["srk_derivative"], scale, prm["v0"])
    a_ref = g["srk_additional"].reshape(-1, 2)
    a = a.reshape(-1, 2)
    d_ref = g["srk_derivative"][2::3]
    # scales: sqrt(2D) sum|cos|/n and sum |d_j - d_i||cos|/n + 2D|d_i|
    phi = g["state0"][2::3]
    owner = np.repeat(np.arange(n), np.diff(off))
    c = np.abs(np.cos(phi[idx] - phi[owner] - prm["alpha"]))
    nn = np.maximum(counts, 1)
    s0 = np.sqrt(2 * prm["D_phi"]) * np.bincount(owner, c, n) / nn
    s1 = np.bincount(owner, np.abs(d_ref[idx] - d_ref[owner]) * c, n) / nn + \
        2 * prm["D_phi"] * np.abs(d_ref)
    assert np.all(np.abs(a[:, 0] - a_ref[:, 0]) <= RHS_TOL * np.maximum(np.abs(a_ref[:, 0]), s0) + 1e-300)
    assert np.all(np.abs(a[:, 1] - a_ref[:, 1]) <= RHS_TOL * np.maximum(np.abs(a_ref[:, 1]), s1) + 1e-300)


def _lattice_ties(L=4.0, rho=0.25, m=12):
    # particles on a grid of pitch rho: every nearest pair sits exactly at dr^2 == rho^2
    xs = (np.arange(m) + 0.5) * rho
    X, Y = np.meshgrid(xs, xs)
    n = m * m
    st = np.zeros(3 * n)
    st[0::3], st[1::3] = X.ravel(), Y.ravel()
    st[2::3] = np.linspace(-3, 3, n)
    return n, L, st


def _neighbour_cases():
    yield "golden_euler", load_golden("chimera_euler_n1024")["state0"], 1024, 1.0, 0.1
    yield "random_n4096", init_state(4096, 2.0, 11), 4096, 2.0, 0.1
    n, L, st = _lattice_ties()
    yield "lattice_ties", st, n, L, 0.25
    st = init_state(512, 1.0, 12)
    st[0], st[3], st[4] = -1e-17, 1.0 - 2.0 ** -53, 1.0  # wraps to L, just below L, exactly L
    yield "edges", st, 512, 1.0, 0.1
    yield "allpairs", init_state(300, 0.5, 13), 300, 0.5, 0.2


@pytest.mark.parametrize("case", list(_neighbour_cases()), ids=lambda c: c[0])
def test_neighbour_sets_bit_exact(case):
    _, st, n, L, rho = case
    prm = dict(PRM0, rho=rho)
    o = po.OracleSystem(n, L, **prm)
    off_ref, idx_ref = o.neighbour_lists(st)
    for flags in (0, abi.FLAG_EXACT_ALL):
        for precision in (abi.PRECISION_FP64, abi.PRECISION_FP32C):
            with gpu(n, L, prm, abi.STEPPER_EULER, flags=flags, precision=precision) as s:
                s.upload_state(st)
                off, idx = s.neighbours()
            assert np.array_equal(off, off_ref)
            assert np.array_equal(idx, idx_ref)


def _oracle_run(n, L, prm, kind, state, dt, nsteps, noise=None, omega=None):
    o = po.OracleSystem(n, L, **prm)
    st = state.copy()
    o.run(kind, st, 0.0, dt, nsteps, noise, omega)
    return st


@pytest.mark.parametrize("stepper,n,L,prm,nsteps,dt", [
    (abi.STEPPER_EULER, 1024, 1.0, PRM0, 100, 0.01),
    (abi.STEPPER_EULER_PTR, 1024, 1.0, PRM0, 100, 0.01),
    (abi.STEPPER_SRK, 2048, 2.0, dict(v0=0.02, sigma=2.0, rho=0.25, alpha=0.0, D_phi=0.01), 100, 0.005),
    (abi.STEPPER_RK4, 4096, 4.0, dict(v0=0.01, sigma=1.0, rho=0.25, alpha=1.45, D_phi=0.0), 100, 0.01),
    (abi.STEPPER_EULER, 256, 0.5, dict(PRM0, rho=0.15), 100, 0.01),
])
@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_100_step_trajectory_with_philox_noise(stepper, n, L, prm, nsteps, dt, kernel):
    st0 = init_state(n, L, 21)
    vortex = stepper == abi.STEPPER_SRK
    omega = np.random.default_rng(22).normal(0, 0.5, n) if vortex else None
    with gpu(n, L, prm, stepper, model=abi.MODEL_VORTEX if vortex else abi.MODEL_CHIMERA,
             seed=1234, kernel=kernel) as s:
        s.upload_state(st0)
        if vortex:
            s.upload_omega(omega)
        s.step(dt, nsteps)
        got = s.download_state()
        noise = s.export_noise(0, nsteps) if s.noise_per_particle else None
    kind = {abi.STEPPER_EULER: po.EULER, abi.STEPPER_EULER_PTR: po.EULER_PTR,
            abi.STEPPER_SRK: po.SRK, abi.STEPPER_RK4: po.RK4}[stepper]
    ref = _oracle_run(n, L, prm, kind, st0, dt, nsteps, noise, omega)
    assert np.abs(periodic_diff(got, ref, L)).max() <= TRAJ_TOL


def test_graph_replay_and_resume_are_bitwise():
    n, L = 1024, 1.0
    st0 = init_state(n, L, 31)
    with gpu(n, L, PRM0, abi.STEPPER_EULER, seed=7) as a, \
            gpu(n, L, PRM0, abi.STEPPER_EULER, seed=7) as b, \
            gpu(n, L, PRM0, abi.STEPPER_EULER, seed=7) as c:
        a.upload_state(st0)
        b.upload_state(st0)
        a.step(0.01, 100)
        for _ in range(4):
            b.step(0.01, 25, graph=True)
        ra, rb = a.download_state(), b.download_state()
        assert np.array_equal(ra, rb)
        # exact resume: state + step counter
        a2 = gpu(n, L, PRM0, abi.STEPPER_EULER, seed=7)
        a2.upload_state(st0)
        a2.step(0.01, 50)
        mid = a2.download_state()
        c.upload_state(mid)
        c.step_counter = 50
        c.step(0.01, 50)
        assert np.array_equal(c.download_state(), ra)
        a2.close()


def test_rk4_buffers_resume_bitwise():
    n, L = 1024, 4.0
    prm = dict(v0=0.01, sigma=1.0, rho=0.25, alpha=1.45, D_phi=0.0)
    st0 = init_state(n, L, 32)
    with gpu(n, L, prm, abi.STEPPER_RK4) as a, gpu(n, L, prm, abi.STEPPER_RK4) as b:
        a.upload_state(st0)
        a.step(0.01, 10)
        b.upload_state(a.download_state())
        b.upload_rk4_buffers(a.download_rk4_buffers())
        a.step(0.01, 10)
        b.step(0.01, 10)
        assert np.array_equal(a.download_state(), b.download_state())


def test_injected_noise_exhaustion_is_an_error():
    n, L = 256, 1.0
    with gpu(n, L, PRM0, abi.STEPPER_EULER) as s:
        st0 = init_state(n, L, 33)
        s.upload_state(st0)
        s.inject_noise(np.zeros(n))
        with pytest.raises(abi.SpcError) as e:
            s.step(0.01, 2)
        assert e.value.code == -5
        assert np.array_equal(s.download_state(), st0)


def test_order_parameters_match_oracle():
    n, L = 2048, 2.0
    st = init_state(n, L, 34)
    st[2::3] = 0.3 * st[2::3]
    o = po.OracleSystem(n, L, **PRM0)
    ref = o.order_params(st)
    with gpu(n, L, PRM0, abi.STEPPER_EULER) as s:
        s.upload_state(st)
        got = s.order_params()
    for k in ("R", "psi", "R_local"):
        assert abs(got[k] - ref[k]) <= 1e-12


@pytest.mark.parametrize("kernel", sorted(KERNELS))
def test_fp32c_rhs_error_is_small(kernel):
    g = load_golden("chimera_euler_n1024")
    n, L = int(g["n"]), float(g["L"])
    prm = golden_params(g)
    o = po.OracleSystem(n, L, **prm)
    off, idx = o.neighbour_lists(g["state0"])
    scale, counts = alignment_scale(g["state0"], off, idx, prm["sigma"], prm["alpha"])
    with gpu(n, L, prm, abi.STEPPER_SRK, precision=abi.PRECISION_FP32C, kernel=kernel) as s:
        s.upload_state(g["state0"])
        d, _ = s.rhs_srk()
    err = np.abs(d[2::3] - g["srk_derivative"][2::3])
    assert np.all(err <= 2e-6 * np.maximum(scale, 1e-3))


@pytest.mark.parametrize("stepper", [abi.STEPPER_EULER, abi.STEPPER_SRK, abi.STEPPER_RK4])
def test_fp64_kernels_agree_bitwise(stepper):
    """Both neighbour kernels sum every particle's terms in the reference's
    visiting order with the same FP64 operations, so their FP64 trajectories
    are identical bit for bit (sparse and dense cells, ragged cell sizes)."""
    cases = [(3000, 1.7, dict(v0=0.02, sigma=1.3, rho=0.09, alpha=1.4, D_phi=0.01)),
             (6000, 1.0, dict(v0=0.01, sigma=0.8, rho=0.2, alpha=1.2, D_phi=0.005))]
    for n, L, prm in cases:
        st0 = init_state(n, L, 51)
        out = {}
        for kernel in KERNELS:
            with gpu(n, L, prm, stepper, seed=5, kernel=kernel) as s:
                s.upload_state(st0)
                s.step(0.01, 20)
                out[kernel] = s.download_state()
        assert np.array_equal(out["tile"], out["warp"])


def test_fp32c_kernels_agree_closely():
    """The FP32C form sums in a different order in the two kernels (blocked
    per-thread Kahan sums vs per-lane Kahan sums and a shuffle tree); after
    one SRK right-hand side the phase rates agree to float rounding."""
    n, L = 3000, 1.7
    prm = dict(v0=0.02, sigma=1.3, rho=0.09, alpha=1.4, D_phi=0.01)
    st0 = init_state(n, L, 52)
    out = {}
    for kernel in KERNELS:
        with gpu(n, L, prm, abi.STEPPER_SRK, precision=abi.PRECISION_FP32C, kernel=kernel) as s:
            s.upload_state(st0)
            out[kernel] = s.rhs_srk()
    d_t, a_t = out["tile"]
    d_w, a_w = out["warp"]
    assert np.array_equal(d_t[0::3], d_w[0::3]) and np.array_equal(d_t[1::3], d_w[1::3])
    assert np.abs(d_t[2::3] - d_w[2::3]).max() <= 1e-5 * prm["sigma"]
    assert np.abs(a_t - a_w).max() <= 1e-5


def test_tuning_knob_round_trip():
    with gpu(256, 1.0, PRM0, abi.STEPPER_EULER) as s:
        assert s.get_tuning(abi.TUNE_SPARSE_BELOW) == 24.0
        s.set_tuning(abi.TUNE_SPARSE_BELOW, 3.5)
        assert s.get_tuning(abi.TUNE_SPARSE_BELOW) == 3.5
        with pytest.raises(abi.SpcError):
            s.set_tuning(abi.TUNE_SPARSE_BELOW, -1.0)
        with pytest.raises(abi.SpcError):
            s.set_tuning(99, 1.0)


@pytest.mark.parametrize("stepper", [abi.STEPPER_SRK, abi.STEPPER_RK4])
def test_tile_split_fp64_is_bitwise_and_fp32c_within_float(stepper):
    # CTAs per cell of the cell-tile passes: each FP64 particle sum walks the
    # whole candidate list in order whatever the split, so FP64 results are
    # bitwise equal; FP32C splits the list into other parts (summation order)
    n, L, dt = 8192, 1.0, 0.005
    prm = dict(v0=0.02, sigma=2.0, rho=0.125, alpha=0.3, D_phi=0.01)  # ~128 per cell
    st0 = init_state(n, L, 53)
    for prec in (abi.PRECISION_FP64, abi.PRECISION_FP32C):
        got = {}
        for split in (1, 2, 4, 8):
            with gpu(n, L, prm, stepper, precision=prec, kernel="tile") as s:
                s.set_tuning(abi.TUNE_TILE_SPLIT, split)
                s.upload_state(st0)
                s.step(dt, 12)
                got[split] = s.download_state()
                assert s.get_tuning(abi.TUNE_TILE_SPLIT) == (split if split else 1)
        for split in (2, 4, 8):
            if prec == abi.PRECISION_FP64:
                assert np.array_equal(got[split], got[1]), split
            else:
                assert np.abs(periodic_diff(got[split], got[1], L)).max() <= 1e-5, split


def test_tile_split_rhs_matches_oracle():
    # the split passes' SRK-form right-hand side against the oracle, at the
    # plain form's tolerance (sparse cells: some particles are isolated)
    n, L = 3000, 1.3
    prm = dict(v0=0.01, sigma=1.0, rho=0.1, alpha=1.45, D_phi=0.005)
    st0 = init_state(n, L, 54)
    o = po.OracleSystem(n, L, **prm)
    d_ref, a_ref, _ = o.rhs_srk(st0.copy())
    for split in (1, 3):
        with gpu(n, L, prm, abi.STEPPER_SRK, kernel="tile") as s:
            s.set_tuning(abi.TUNE_TILE_SPLIT, split)
            s.upload_state(st0)
            d, a = s.rhs_srk()
        assert np.abs(d - d_ref).max() <= RHS_TOL * max(np.abs(d_ref).max(), 1.0), split
        assert np.abs(a - a_ref).max() <= RHS_TOL * max(np.abs(a_ref).max(), 1.0), split


def test_tile_split_knob_validation():
    with gpu(256, 1.0, PRM0, abi.STEPPER_EULER) as s:
        for bad in (-1.0, 9.0, 1.5):
            with pytest.raises(abi.SpcError):
                s.set_tuning(abi.TUNE_TILE_SPLIT, bad)
        s.set_tuning(abi.TUNE_TILE_SPLIT, 3)
        assert s.get_tuning(abi.TUNE_TILE_SPLIT) == 3.0


@pytest.mark.parametrize("n,L,rho", [(20000, 8.0, 0.1), (3000, 3.0, 0.05)])
def test_two_pass_sort_neighbour_lists_match_oracle(n, L, rho):
    # more than 2048 cells: the radix sort takes two 8-bit passes, each
    # scattered by several CTAs per sort tile (few tiles); the neighbour lists
    # in the reference's visiting order must come out exactly
    prm = dict(v0=0.01, sigma=1.0, rho=rho, alpha=1.45, D_phi=0.005)
    st = init_state(n, L, 55)
    assert abi.cells_of(L, rho) > 2048
    with gpu(n, L, prm, abi.STEPPER_EULER) as s:
        s.upload_state(st)
        off, idx = s.neighbours()
    o = po.OracleSystem(n, L, **prm)
    off_ref, idx_ref = o.neighbour_lists(st)
    assert np.array_equal(off, off_ref) and np.array_equal(idx, idx_ref)


def test_fp64_division_by_reciprocal_is_bitwise():
    # the FP64 kernels divide by reused divisors (n_i, pair distances, the
    # vortex-arrays constants) through a rounded reciprocal and one fused
    # multiply-add correction; it must give every bit of the correctly
    # rounded quotient
    rng = np.random.default_rng(56)
    m = 4_000_000
    mant = 1.0 + rng.random(m)
    a = np.ldexp(mant, rng.integers(-40, 40, m)) * rng.choice([-1.0, 1.0], m)
    b = np.concatenate([
        rng.integers(1, 5000, m // 4).astype(np.float64),              # neighbour counts
        rng.uniform(1e-6, 0.3, m // 4),                                 # pair distances
        np.ldexp(1.0 + rng.random(m // 4), rng.integers(-20, 20, m // 4)),
        # significands near all ones
        np.ldexp(2.0 - np.ldexp(rng.integers(1, 256, m // 4).astype(np.float64), -52),
                 rng.integers(-8, 8, m // 4)),
    ])
    assert abi.check_division(a, b) == 0
    assert abi.check_division(np.zeros(0), np.zeros(0)) == 0


def test_sincos_cosine_is_bitwise_the_cosine():
    # the FP64 Verlet SRK first pass keeps sincos's cosine of each accepted
    # pair for the second pass; it must be the cosine the second pass would
    # compute (test_row_overflow_fallback_is_bitwise_fp64 checks the passes)
    rng = np.random.default_rng(57)
    m = 2_000_000
    x = np.concatenate([rng.uniform(-7, 7, m), rng.uniform(-1e3, 1e3, m), rng.normal(0, 50, m),
                        np.ldexp(rng.random(m), rng.integers(-30, 30, m)) * rng.choice([-1.0, 1.0], m)])
    assert abi.check_sincos(x) == 0


def test_pair_at_the_lower_band_edge_is_counted():
    """A pair whose float prefilter offset lands exactly on the lower edge of
    the undecided band must still be decided (it is inside the cutoff).  For
    rho = 0.15 the rounded band centre makes |lo2 - mid| exceed the band
    half-width, so a test taken from d^2 < lo2 and |d^2 - mid| <= band
    separately leaves a float d^2 equal to lo2 in neither set and drops the
    pair.  Particles 0 and 1 sit in the cell at the origin, so their float
    offsets are their coordinates and the float d^2 is exactly lo2; the
    reference's FP64 test has them within rho.  Every kernel and precision
    must give the oracle's rates."""
    f = np.float32
    L, rho = 1.0, 0.15
    st = np.array([0.0078125, 0.0625, 0.3,
                   0.15781013667583466, 0.06268310546875, -1.1,
                   0.62, 0.58, 2.0,
                   0.81, 0.33, -0.4])
    n = st.size // 3
    # the geometry: float d^2 == lo2, inside the cutoff in FP64
    lo2, hi2 = f(rho * rho * (1 - 3e-5)), f(rho * rho * (1 + 3e-5))
    band, mid = f(f(0.5) * f(hi2 - lo2)), f(f(0.5) * f(hi2 + lo2))
    dx, dy = f(f(st[3]) - f(st[0])), f(f(st[4]) - f(st[1]))
    d2 = f(np.float64(dx) * np.float64(dx) + np.float64(f(dy * dy)))
    assert d2 == lo2 and not (d2 < lo2) and not (abs(f(d2 - mid)) <= band)
    assert (st[3] - st[0]) ** 2 + (st[4] - st[1]) ** 2 <= rho * rho
    prm = dict(v0=0.01, sigma=1.0, rho=rho, alpha=1.45, D_phi=0.005)
    o = po.OracleSystem(n, L, **prm)
    d_ref, _, counts = o.rhs_srk(st, with_counts=True)
    assert counts[0] == 1 and counts[1] == 1 and d_ref[2] != 0.0
    variants = [(abi.PRECISION_FP64, abi.NEIGHBOUR_CELL, k) for k in KERNELS] + \
        [(abi.PRECISION_FP64, abi.NEIGHBOUR_VERLET, None)] + \
        [(abi.PRECISION_FP32X, abi.NEIGHBOUR_CELL, k) for k in KERNELS] + \
        [(abi.PRECISION_FP32C, abi.NEIGHBOUR_CELL, k) for k in KERNELS] + \
        [(abi.PRECISION_FP32C, abi.NEIGHBOUR_VERLET, None)]
    for prec, nb, kernel in variants:
        p = abi.make_params(L=L, stepper=abi.STEPPER_SRK, precision=prec, neighbour=nb, skin=0.05,
                            **prm)
        with abi.System(n, p) as s:
            if kernel is not None:
                s.set_tuning(abi.TUNE_SPARSE_BELOW, KERNELS[kernel])
            s.upload_state(st)
            d, _ = s.rhs_srk()
        tol = 2e-6 if prec == abi.PRECISION_FP32C else RHS_TOL
        assert np.all(np.abs(d[2::3] - d_ref[2::3]) <= tol), (prec, nb, kernel, d[2::3], d_ref[2::3])
