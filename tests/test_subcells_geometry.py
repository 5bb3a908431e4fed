"""Sub-cells (SPC_TUNE_SUBCELLS), restated on the CPU: the cell and half
bounds of the sorted keys (csrc/spc_sort.cuh half_bounds_at), the binning of
csrc/spc_kernels.cuh (cell_coord, row_offset: the half of each particle, the
near flag of each cell) and the half stencils of csrc/spc_tile.cuh
(stencil_of with half 0 / 1), checked against the reference's own cutoff test
(PeriodicBoundaryConditions.cpp:22-35 minimum image, ChimeraSystem.cpp:407-410
dr^2 <= rho^2) on every pair: each pair within rho lies in the stencil of its
particle's half.  Random states with the cell side equal to rho, lattices on
the half lines, and pairs built to straddle a half line at a distance that
rounds to rho.  The last show why the near flags exist: without them such a
pair is left out (a planted mistake in this restatement, not in the kernels)."""
import numpy as np

NEAR = 2.0 ** -20


def binning(x, y, L, rho):
    nc = max(1, int(L / rho))
    cell = L / nc
    pow2 = L > 0 and float(L).hex().startswith("0x1.0000000000000p")

    def coord(v):
        q = v * (1.0 / L) if pow2 else v / L
        return np.clip(np.trunc(q * nc).astype(np.int64), 0, nc - 1)

    cx, cy = coord(x), coord(y)
    u = y - cy.astype(np.float64) * cell  # row_offset
    half = (u >= 0.5 * cell).astype(np.int64)
    cellid = cy * nc + cx
    near = np.zeros(nc * nc, dtype=bool)
    near[cellid[np.abs(u - 0.5 * cell) < NEAR * cell]] = True
    return nc, cx, cy, half, near


def within(x, y, L, rho, i, j):
    rL = 1.0 / L

    def mi(d):
        return d - np.trunc((d * 2.0) * rL) * L

    dx = mi(x[j] - x[i])
    dy = mi(y[j] - y[i])
    return dx * dx + dy * dy <= rho * rho


def uncovered(x, y, L, rho, use_near=True):
    """Pairs within rho (reference test) outside the stencil of i's half."""
    nc, cx, cy, half, near = binning(x, y, L, rho)
    n = len(x)
    bad = []
    for i0 in range(0, n, 256):
        i = np.arange(i0, min(n, i0 + 256))[:, None]
        j = np.arange(n)[None, :]
        w = within(x, y, L, rho, i, j) & (i != j)
        ii, jj = np.nonzero(w)
        ii = ii + i0
        ox = (cx[jj] - cx[ii]) % nc
        oy = (cy[jj] - cy[ii]) % nc
        ox = np.where(ox == nc - 1, -1, ox)
        oy = np.where(oy == nc - 1, -1, oy)
        # the reference's own 3x3 stencil holds every pair it counts
        assert np.all(np.abs(ox) <= 1) and np.all(np.abs(oy) <= 1)
        far = oy == np.where(half[ii] == 0, 1, -1)
        whole = near[cy[ii] * nc + cx[ii]] & near[cy[jj] * nc + cx[jj]]
        if not use_near:
            whole = np.zeros_like(whole)
        left_out = far & ~whole & (half[jj] != half[ii])
        bad += list(zip(ii[left_out], jj[left_out]))
    return bad


def test_random_states_are_covered():
    rng = np.random.default_rng(5)
    for L, rho, n in ((8.0, 0.25, 3000), (8.0, 0.3, 2500), (10.0, 0.25, 3000), (4.0, 1.0, 600)):
        x = rng.uniform(0.0, L, n)
        y = rng.uniform(0.0, L, n)
        assert uncovered(x, y, L, rho) == []


def test_lattices_on_the_half_lines_are_covered():
    for L, rho in ((8.0, 0.25), (6.0, 0.25)):
        nc = int(L / rho)
        cell = L / nc
        for step in (cell / 2, cell / 4):
            g = np.arange(0.0, L, step)
            x, y = np.meshgrid(g[:40], g)
            x, y = x.ravel(), y.ravel()
            assert uncovered(x, y, L, rho) == []


def test_straddling_pairs_need_the_near_flags():
    # i just below the half line of row 0, j on the half line of row 1, at the
    # same x: the reference's dy rounds to 0.25 = rho, so it counts the pair
    L, rho = 8.0, 0.25
    base_i = 0.125 - 2.0 ** -56
    xs, ys = [], []
    for k, (dy_i, dy_j) in enumerate([(0.0, 0.0), (-2.0 ** -56, 0.0), (0.0, 2.0 ** -54)]):
        x0 = 0.5 + 0.75 * k  # pairs in different cells, far apart
        xs += [x0, x0]
        ys += [base_i + dy_i, 0.375 + dy_j]
    x, y = np.array(xs), np.array(ys)
    nc, cx, cy, half, near = binning(x, y, L, rho)
    assert list(half[0::2]) == [0, 0, 0] and list(half[1::2]) == [1, 1, 1]
    assert within(x, y, L, rho, 0, 1)  # the reference counts it
    assert uncovered(x, y, L, rho, use_near=False) != []  # without the flags it is lost
    assert uncovered(x, y, L, rho) == []
    # the flags are rare on a random state: about 2 * 2^-20 of the particles
    rng = np.random.default_rng(9)
    xr, yr = rng.uniform(0, L, 200000), rng.uniform(0, L, 200000)
    _, _, _, _, nr = binning(xr, yr, L, rho)
    assert nr.sum() <= 5


def test_half_stencils_hold_fewer_candidates():
    rng = np.random.default_rng(2)
    L, rho, n = 8.0, 0.25, 65536
    x, y = rng.uniform(0, L, n), rng.uniform(0, L, n)
    nc, cx, cy, half, near = binning(x, y, L, rho)
    cnt = np.zeros((nc, nc, 2), dtype=np.int64)
    np.add.at(cnt, (cy, cx, half), 1)
    whole = sum(np.roll(np.roll(cnt.sum(2), a, 0), b, 1) for a in (-1, 0, 1) for b in (-1, 0, 1))
    # lower half: rows cy-1 and cy whole, row cy+1 lower half (roll by -1 brings row cy+1 to cy)
    row = lambda arr, a: sum(np.roll(np.roll(arr, a, 0), b, 1) for b in (-1, 0, 1))
    lower = row(cnt.sum(2), 1) + row(cnt.sum(2), 0) + row(cnt[:, :, 0], -1)
    upper = row(cnt[:, :, 1], 1) + row(cnt.sum(2), 0) + row(cnt.sum(2), -1)
    tests_whole = (cnt.sum(2) * whole).sum()
    tests_half = (cnt[:, :, 0] * lower).sum() + (cnt[:, :, 1] * upper).sum()
    assert 0.80 < tests_half / tests_whole < 0.87  # 7.5 of 9 stencil cells


def half_bounds(skeys, ncell):
    """half_bounds_at (csrc/spc_sort.cuh) for every slot p in [0, n], with a
    count of the writes to each entry."""
    n = len(skeys)
    start = np.full(ncell + 1, -1)
    mid = np.full(ncell, -1)
    writes = np.zeros(2 * ncell + 1, dtype=int)
    for p in range(n + 1):
        lo = -1 if p == 0 else int(skeys[p - 1])
        hi = 2 * ncell if p == n else min(int(skeys[p]), 2 * ncell)
        for k in range(lo + 1, hi + 1):
            writes[k] += 1
            if k & 1:
                mid[k >> 1] = p
            else:
                start[k >> 1] = p
    return start, mid, writes


def test_half_bounds_against_searchsorted():
    rng = np.random.default_rng(3)
    for ncell, n in ((1, 0), (1, 5), (7, 40), (64, 300), (50, 3)):
        keys = np.sort(rng.integers(0, 2 * ncell, n)) if n else np.zeros(0, dtype=int)
        start, mid, writes = half_bounds(keys, ncell)
        assert np.all(writes == 1)  # every entry exactly once
        assert np.array_equal(start, np.searchsorted(keys, 2 * np.arange(ncell + 1), "left"))
        assert np.array_equal(mid, np.searchsorted(keys, 2 * np.arange(ncell) + 1, "left"))
        assert np.all(start[:-1] <= mid) and np.all(mid <= start[1:])
