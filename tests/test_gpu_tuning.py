"""The autotuner's candidates and in-place retuning.

* spc_autotune_ex offers every tuning dimension: the kernel choice (all
  cell-tile, the default split, all warp-per-cell), 1, 2 or 4 CTAs per cell,
  cell units and sub-cells (float forms), and Verlet skins where the
  precision and stencil allow them.
* Every kernel-choice candidate computes the same neighbour sets: FP64 and
  FP32X trajectories are bit for bit the same under each of them, and FP32C
  ones under every CTA split (with cell units off, on, and with sub-cells).
* spc_retune / spc_batch_retune leave the state and the step counters as they
  were, so a run that retunes midway equals one that does not, bit for bit.
"""
import numpy as np
import pytest

from spc2_langevin_integration_gb300 import abi
from tests._helpers import init_state
from tests.test_subcells_geometry import binning, within

pytestmark = pytest.mark.gpu

PRM = dict(v0=0.02, sigma=1.3, rho=0.12, alpha=1.4, D_phi=0.01)
N, L = 6000, 1.5


def _params(precision, stepper=abi.STEPPER_SRK):
    return abi.make_params(L=L, stepper=stepper, precision=precision, seed=31, **PRM)


def test_autotune_ex_offers_every_dimension():
    st = init_state(N, L, 90)
    cands, best = abi.autotune_ex(N, _params(abi.PRECISION_FP64), st, trial_steps=5)
    cell = [c for c in cands if c["neighbour"] == "cell"]
    assert {c["tile_split"] for c in cell} == {1, 2, 4}
    assert {c["sparse_below"] for c in cell} >= {0.0, 1e9}
    assert any(c["neighbour"] == "verlet" for c in cands)
    assert 0 <= best < len(cands) and all(c["ms_per_step"] > 0 for c in cands)
    assert {c["cell_units"] for c in cands} == {0}  # FP64 has no cell units
    assert {c["subcells"] for c in cands} == {0}  # nor sub-cells
    # FP32X runs the cell list only, with and without cell units
    cx, _ = abi.autotune_ex(N, _params(abi.PRECISION_FP32X), st, trial_steps=5)
    assert all(c["neighbour"] == "cell" for c in cx)
    assert len([c for c in cx if c["cell_units"] == 0]) == len(cell)
    assert {(c["sparse_below"], c["tile_split"]) for c in cx if c["cell_units"] == 1} == \
        {(0.0, 1), (0.0, 2), (24.0, 1), (24.0, 2)}
    # sub-cells (the cell-size dimension) run as units of half cells
    assert sorted((c["sparse_below"], c["tile_split"], c["cell_units"]) for c in cx if c["subcells"] == 1) == \
        [(0.0, 1, 1), (24.0, 1, 1)]


@pytest.mark.parametrize("precision,n,patch", [
    (abi.PRECISION_FP64, N, 0.45), (abi.PRECISION_FP32X, N, 0.45), (abi.PRECISION_FP32C, N, 0.45),
    (abi.PRECISION_FP32X, 9000, 0.2), (abi.PRECISION_FP32C, 9000, 0.2)])
def test_kernel_choices_give_identical_trajectories(precision, n, patch):
    """FP64 and FP32X: every kernel choice; FP32C: every CTA split of the
    cell-tile kernels, with cell units off and on (its cell-tile and
    warp-per-cell kernels, and cell units, sum in different orders).  The
    particles are clustered into a patch so that cells hold several particle
    groups and the splits really spread them.  6,000 in a 0.45 x 0.45 patch
    give cells of ~4,200 candidates, which cell units cut into units of 32
    particles x one staging round; 9,000 in a 0.2 x 0.2 patch share one
    stencil, more staging rounds than a cell may be cut into, so those cells
    stay whole groups with cell units on.  Sub-cells: FP32X gives the same
    bits again (the half stencils hold every pair within rho); FP32C sums
    in the half-cell order, the same under every split."""
    rng = np.random.default_rng(91)
    st = init_state(n, L, 91)
    st[0::3] = 0.2 + patch * rng.random(n)
    st[1::3] = 0.2 + patch * rng.random(n)
    choices = [((0.0, 1, 0, 0), (0.0, 2, 0, 0), (0.0, 4, 0, 0), (24.0, 1, 0, 0), (1e9, 1, 0, 0))]
    if precision == abi.PRECISION_FP32X:
        choices = [choices[0] + ((0.0, 1, 1, 0), (0.0, 2, 1, 0), (24.0, 1, 1, 0),
                                 (0.0, 1, 1, 1), (0.0, 2, 0, 1), (24.0, 1, 1, 1))]
    if precision == abi.PRECISION_FP32C:
        choices = [choices[0][:3], ((0.0, 1, 1, 0), (0.0, 2, 1, 0), (0.0, 4, 1, 0)),
                   ((0.0, 1, 1, 1), (0.0, 2, 1, 1), (0.0, 4, 0, 1))]
    for group in choices:
        out = []
        for sb, split, units, sub in group:
            with abi.System(n, _params(precision)) as s:
                s.set_tuning(abi.TUNE_SPARSE_BELOW, sb)
                s.set_tuning(abi.TUNE_TILE_SPLIT, split)
                s.set_tuning(abi.TUNE_CELL_UNITS, units)
                s.set_tuning(abi.TUNE_SUBCELLS, sub)
                s.upload_state(st)
                s.step(0.005, 30 if n == N else 10)
                out.append(s.download_state())
        for o in out[1:]:
            assert np.array_equal(o, out[0])


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_FP32X])
def test_retune_midway_leaves_the_run_unchanged(precision):
    st = init_state(N, L, 92)
    finals = []
    for retune in (False, True):
        with abi.System(N, _params(precision)) as s:
            s.upload_state(st)
            s.step(0.005, 20, graph=True)
            if retune:
                before, ctr = s.download_state(), s.step_counter
                cands, best = s.retune(0.005, trial_steps=5)
                nc = 7 if precision == abi.PRECISION_FP64 else 13
                assert len(cands) == nc and 0 <= best < nc
                assert np.array_equal(s.download_state(), before) and s.step_counter == ctr
                assert s.get_tuning(abi.TUNE_TILE_SPLIT) == cands[best]["tile_split"]
                assert s.get_tuning(abi.TUNE_CELL_UNITS) == cands[best]["cell_units"]
                assert s.get_tuning(abi.TUNE_SUBCELLS) == cands[best]["subcells"]
                s.prepare_graph(0.005, 20)  # captured, not run: state and counter unchanged
                assert s.graph_nodes() > 0
                assert np.array_equal(s.download_state(), before) and s.step_counter == ctr
            s.step(0.005, 20, graph=True)
            finals.append(s.download_state())
    assert np.array_equal(finals[0], finals[1])


def test_batch_retune_leaves_the_run_unchanged():
    systems = [(1500, 1.0, dict(PRM, rho=0.1)), (4000, 1.3, dict(PRM, rho=0.2)),
               (300, 0.6, dict(PRM, rho=0.16))]
    ntot = sum(n for n, _, _ in systems)
    ctot = sum(abi.cells_of(Lb, p["rho"]) for _, Lb, p in systems)
    finals = []
    for retune in (False, True):
        with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP32X, 3, ntot, ctot) as b:
            slots = [b.admit(n, abi.make_params(L=Lb, stepper=abi.STEPPER_EULER,
                                                precision=abi.PRECISION_FP32X, seed=4, system_id=k, **p),
                             init_state(n, Lb, 93 + k), steps=60)
                     for k, (n, Lb, p) in enumerate(systems)]
            b.step(0.01, 30)
            if retune:
                before = [b.download(s) for s in slots]
                status = [b.status(s) for s in slots]
                cands, best = b.retune(0.01, trial_steps=5)
                assert len(cands) == 13
                assert all(np.array_equal(b.download(s), x) for s, x in zip(slots, before))
                assert [b.status(s) for s in slots] == status
            b.step(0.01, 40)  # past the budgets: every system stops at 60 steps
            finals.append([b.download(s) for s in slots])
            assert all(b.status(s)[1] == 0 for s in slots)
    for x, y in zip(*finals):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP32X, abi.PRECISION_FP32C])
def test_cell_units_graph_equals_eager(precision):
    """With cell units the units kernel runs on a second stream beside the
    cell-tile kernel (parallel branches of the step graph): captured graph
    replays and eager steps give the same bits, and FP32X gives the bits of
    the run without cell units.  The same with sub-cells (units of half
    cells), switched on and off between calls of one handle."""
    rng = np.random.default_rng(94)
    st = init_state(N, L, 94)
    st[0::3] = 0.2 + 0.45 * rng.random(N)
    st[1::3] = 0.2 + 0.45 * rng.random(N)
    out = {}
    for units, sub, graph in ((1, 0, False), (1, 0, True), (0, 0, False), (0, 1, False), (0, 1, True)):
        with abi.System(N, _params(precision)) as s:
            s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
            s.set_tuning(abi.TUNE_CELL_UNITS, units)
            s.set_tuning(abi.TUNE_SUBCELLS, sub)
            assert s.get_tuning(abi.TUNE_CELL_UNITS) == units
            assert s.get_tuning(abi.TUNE_SUBCELLS) == sub
            s.upload_state(st)
            for _ in range(3):
                s.step(0.005, 10, graph=graph)
            out[(units, sub, graph)] = s.download_state()
    assert np.array_equal(out[(1, 0, False)], out[(1, 0, True)])
    assert np.array_equal(out[(0, 1, False)], out[(0, 1, True)])
    if precision == abi.PRECISION_FP32X:
        assert np.array_equal(out[(1, 0, False)], out[(0, 0, False)])
        assert np.array_equal(out[(0, 1, False)], out[(0, 0, False)])
    # toggled on one handle: sub-cells for the first call only
    with abi.System(N, _params(precision)) as s:
        s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
        s.upload_state(st)
        s.set_tuning(abi.TUNE_SUBCELLS, 1)
        s.step(0.005, 10, graph=True)
        mid = s.download_state()
        s.set_tuning(abi.TUNE_SUBCELLS, 0)
        s.step(0.005, 20, graph=True)
        toggled = s.download_state()
    with abi.System(N, _params(precision)) as s:
        s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
        s.set_tuning(abi.TUNE_SUBCELLS, 1)
        s.upload_state(st)
        s.step(0.005, 10, graph=True)
        assert np.array_equal(s.download_state(), mid)
        s.set_tuning(abi.TUNE_SUBCELLS, 0)
        s.step(0.005, 20)
        assert np.array_equal(s.download_state(), toggled)


def test_cell_units_refused_for_fp64():
    with abi.System(N, _params(abi.PRECISION_FP64)) as s:
        for key in (abi.TUNE_CELL_UNITS, abi.TUNE_SUBCELLS):
            with pytest.raises(abi.SpcError):
                s.set_tuning(key, 1)
            for bad in (-1.0, 2.0, 0.5):
                with pytest.raises(abi.SpcError):
                    s.set_tuning(key, bad)
            s.set_tuning(key, 0)
            assert s.get_tuning(key) == 0


def test_subcells_refused_for_verlet_rows():
    p = _params(abi.PRECISION_FP32C)
    p.neighbour = abi.NEIGHBOUR_VERLET
    p.skin = 0.2 * PRM["rho"]
    with abi.System(N, p) as s:
        with pytest.raises(abi.SpcError):
            s.set_tuning(abi.TUNE_SUBCELLS, 1)
        s.set_tuning(abi.TUNE_SUBCELLS, 0)


@pytest.mark.parametrize("stepper", [abi.STEPPER_SRK, abi.STEPPER_EULER])
def test_subcells_fp32x_on_half_lines_and_cutoff_ties_bitwise(stepper):
    """Lattices with pairs at exactly rho: off the half lines in the lower
    half of the box (the half stencils leave out the far halves), on them in
    the upper half (cells that keep their far cells whole); and pairs that
    straddle a half line a rounding step away from rho (the case the near
    flags keep whole).  FP32X with sub-cells gives the bits of whole cells.
    L = 2, rho = 0.125: the cell side is rho exactly."""
    Lb, rho = 2.0, 0.125
    rng = np.random.default_rng(98)
    g = np.arange(32) * (rho / 2)
    rows = np.concatenate([rho / 8 + np.arange(16) * (rho / 2),  # off the half lines
                           1.0 + np.arange(16) * (rho / 2)])     # on them and on the cell edges
    xs, ys = np.meshgrid(g, rows)
    x = list(xs.ravel())
    y = list(ys.ravel())
    n_lat = len(x)
    for k in range(64):  # straddling pairs at the same x
        cy = 0 if k < 32 else k % 15  # row 0: the reference's dy rounds to rho
        x0 = 0.03 + (k % 32) * (Lb / 32)
        x += [x0, x0]
        y += [np.nextafter(cy * rho + rho / 2, -1.0), (cy + 1) * rho + rho / 2]
    n = len(x)
    xa, ya = np.array(x), np.array(y)
    _, _, _, hh, _ = binning(xa, ya, Lb, rho)
    i = np.arange(n_lat, n, 2)
    assert np.all(hh[i] == 0) and np.all(hh[i + 1] == 1)
    assert within(xa, ya, Lb, rho, i, i + 1).sum() >= 32
    phi = rng.uniform(-np.pi, np.pi, n)
    st = np.empty(3 * n)
    st[0::3], st[1::3], st[2::3] = x, y, phi
    p = abi.make_params(L=Lb, stepper=stepper, precision=abi.PRECISION_FP32X, seed=7,
                        **dict(PRM, rho=rho))
    out = []
    for sub in (0, 1):
        with abi.System(n, p) as s:
            s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
            s.set_tuning(abi.TUNE_SUBCELLS, sub)
            s.upload_state(st)
            if stepper == abi.STEPPER_SRK:
                out.append(np.concatenate(s.rhs_srk()))
            s.step(0.001, 5)
            out.append(s.download_state())
    half = len(out) // 2
    for a, b in zip(out[:half], out[half:]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("stepper", [abi.STEPPER_RK4, abi.STEPPER_EULER])
def test_cell_units_fp32x_other_steppers_bitwise(stepper):
    """The units kernel serves every evaluation of a step (RK4's four, Euler's
    one): FP32X with cell units, or with sub-cells, gives the bits of the run
    without them."""
    rng = np.random.default_rng(95)
    st = init_state(N, L, 95)
    st[0::3] = 0.2 + 0.45 * rng.random(N)
    st[1::3] = 0.2 + 0.45 * rng.random(N)
    out = []
    for units, sub in ((0, 0), (1, 0), (0, 1)):
        with abi.System(N, _params(abi.PRECISION_FP32X, stepper)) as s:
            s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
            s.set_tuning(abi.TUNE_CELL_UNITS, units)
            s.set_tuning(abi.TUNE_SUBCELLS, sub)
            s.upload_state(st)
            s.step(0.005, 12, graph=True)
            out.append(s.download_state())
    assert np.array_equal(out[0], out[1])
    assert np.array_equal(out[0], out[2])


def test_cell_units_in_a_batch_with_admissions_equal_alone():
    """A served FP32X batch with cell units on (and, again, with sub-cells),
    whose layout changes between calls (a system released, another
    admitted): every system's state equals the same system run alone without
    cell units, bit for bit."""
    rng = np.random.default_rng(96)

    def clustered(n, Lb, seed):
        st = init_state(n, Lb, seed)
        st[0::3] = 0.1 * Lb + 0.4 * Lb * rng.random(n)
        st[1::3] = 0.1 * Lb + 0.4 * Lb * rng.random(n)
        return st

    systems = [(3000, 1.2, dict(PRM, rho=0.15)), (5000, 1.5, dict(PRM, rho=0.12)),
               (2000, 1.0, dict(PRM, rho=0.2))]
    states = [clustered(n, Lb, 97 + k) for k, (n, Lb, _) in enumerate(systems)]

    def params(k):
        n, Lb, p = systems[k]
        return abi.make_params(L=Lb, stepper=abi.STEPPER_SRK, precision=abi.PRECISION_FP32X, seed=5,
                               system_id=k, **p)

    ntot = sum(n for n, _, _ in systems)
    ctot = sum(abi.cells_of(Lb, p["rho"]) for _, Lb, p in systems)
    got = {}
    for key in (abi.TUNE_CELL_UNITS, abi.TUNE_SUBCELLS):
        with abi.Batch(abi.STEPPER_SRK, abi.PRECISION_FP32X, 3, ntot, ctot) as b:
            b.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
            b.set_tuning(key, 1)
            s0 = b.admit(systems[0][0], params(0), states[0])
            s1 = b.admit(systems[1][0], params(1), states[1])
            b.step(0.005, 10, graph=True)
            b.release(s0)
            s2 = b.admit(systems[2][0], params(2), states[2])
            b.step(0.005, 10, graph=True)
            got[key] = {1: b.download(s1), 2: b.download(s2)}
    for k, nsteps in ((1, 20), (2, 10)):
        with abi.System(systems[k][0], params(k)) as s:
            s.set_tuning(abi.TUNE_SPARSE_BELOW, 0.0)
            s.upload_state(states[k])
            s.step(0.005, nsteps)
            for key in got:
                assert np.array_equal(s.download_state(), got[key][k]), (key, k)


def test_subcells_with_sparse_systems_in_a_batch_bitwise():
    """Sub-cells sort every cell of the batch by half, the sparse systems'
    cells too (their warp-per-cell kernels find their own slot by position
    in the staged list, not by index order): an FP32X batch of dense
    (cell-tile) and sparse (warp-per-cell) systems gives the bits of the
    same batch without sub-cells."""
    systems = [(6000, 1.5, dict(PRM, rho=0.12)), (400, 1.6, dict(PRM, rho=0.1)),
               (900, 2.0, dict(PRM, rho=0.2))]
    ntot = sum(n for n, _, _ in systems)
    ctot = sum(abi.cells_of(Lb, p["rho"]) for _, Lb, p in systems)
    out = []
    for sub in (0, 1):
        with abi.Batch(abi.STEPPER_EULER, abi.PRECISION_FP32X, 3, ntot, ctot) as b:
            b.set_tuning(abi.TUNE_SUBCELLS, sub)
            assert b.get_tuning(abi.TUNE_SPARSE_BELOW) == 24.0
            slots = [b.admit(n, abi.make_params(L=Lb, stepper=abi.STEPPER_EULER,
                                                precision=abi.PRECISION_FP32X, seed=8, system_id=k, **p),
                             init_state(n, Lb, 120 + k))
                     for k, (n, Lb, p) in enumerate(systems)]
            b.step(0.01, 10)
            b.step(0.01, 10, graph=True)
            out.append([b.download(s) for s in slots])
    for x, y in zip(*out):
        assert np.array_equal(x, y)
