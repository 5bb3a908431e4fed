"""The index arithmetic of the cell units (csrc/spc_tile.cuh: unit_cell,
k_list_units, k_units_fp32c / k_units_fp32x, split_point), restated on the
CPU and checked against the buffers it addresses: every (particle, staging
round) pair of a unit cell is covered by exactly one unit, the list fits the
capacity the engine allocates ((N / 32 + cells) x 8 entries), the per-round
sums stay inside the 8 x N round buffers, and the four warp parts of a round
tile it on word (32-candidate) boundaries."""
import numpy as np

WARP = 32
SPLIT_ROUNDS = 8


def split_point(rcnt, part, S):
    return rcnt if part >= S else ((rcnt * part // S) & ~31)


def unit_cell(n_c, total, cap):
    return n_c > 0 and total <= SPLIT_ROUNDS * cap


def list_units(occupancy, totals, cap):
    units = []
    for c, (n_c, total) in enumerate(zip(occupancy, totals)):
        if not unit_cell(n_c, total, cap):
            continue
        rounds = (total + cap - 1) // cap
        units += [(c, u) for u in range((n_c + WARP - 1) // WARP * rounds)]
    return units


def test_units_cover_every_particle_and_round_once():
    rng = np.random.default_rng(11)
    for cap in (1024, 768):  # FP32C and FP32X staging rounds
        for trial in range(20):
            ncell = int(rng.integers(1, 400))
            occupancy = rng.poisson(rng.uniform(1, 300), ncell)
            occupancy[rng.random(ncell) < 0.1] = 0
            # a cell's stencil holds at least the cell itself
            totals = occupancy + rng.integers(0, 9000, ncell)
            starts = np.concatenate([[0], np.cumsum(occupancy)])
            n_all = int(starts[-1])
            units = list_units(occupancy, totals, cap)
            assert len(units) <= ((n_all + WARP - 1) // WARP + ncell) * SPLIT_ROUNDS
            covered = {}
            for c, u in units:
                total = int(totals[c])
                rounds = (total + cap - 1) // cap
                k, r = divmod(u, rounds)
                c0, c1 = int(starts[c]), int(starts[c + 1])
                ig = c0 + k * WARP
                gi = min(WARP, c1 - ig)
                assert 0 < gi <= WARP and ig + gi <= c1 and r < rounds <= SPLIT_ROUNDS
                rlo = r * cap
                rcnt = min(cap, total - rlo)
                assert 0 < rcnt <= cap
                rpad = (rcnt + WARP - 1) & ~(WARP - 1)
                bounds = [split_point(rpad, w, 4) for w in range(5)]
                assert bounds[0] == 0 and bounds[-1] == rpad
                assert all(b % WARP == 0 for b in bounds) and bounds == sorted(bounds)
                for p in range(ig, ig + gi):
                    assert r * n_all + p < SPLIT_ROUNDS * n_all  # the round buffers
                    covered[(p, r)] = covered.get((p, r), 0) + 1
            for c in range(ncell):
                if unit_cell(int(occupancy[c]), int(totals[c]), cap):
                    rounds = (int(totals[c]) + cap - 1) // cap
                    for p in range(int(starts[c]), int(starts[c + 1])):
                        for r in range(rounds):
                            assert covered.pop((p, r)) == 1
            assert not covered  # nothing outside the unit cells


def list_units_halves(occupancy, mids, totals, half_totals, cap):
    """k_list_units with sub-cells: the units of each half, as (2c + h, u)."""
    units = []
    for c, (n_c, total) in enumerate(zip(occupancy, totals)):
        if not unit_cell(n_c, total, cap):
            continue
        for h in (0, 1):
            n_h = n_c - mids[c] if h else mids[c]
            if n_h == 0:
                continue
            rounds = (half_totals[c][h] + cap - 1) // cap
            units += [(2 * c + h, u) for u in range((n_h + WARP - 1) // WARP * rounds)]
    return units


def test_half_cell_units_cover_every_particle_and_round_once():
    rng = np.random.default_rng(12)
    for cap in (1024, 768):
        for trial in range(20):
            ncell = int(rng.integers(1, 300))
            occupancy = rng.poisson(rng.uniform(1, 300), ncell)
            occupancy[rng.random(ncell) < 0.1] = 0
            mids = np.array([rng.integers(0, n + 1) for n in occupancy])  # lower-half sizes
            totals = occupancy + rng.integers(0, 9000, ncell)
            # a half's stencil: its own cell whole, at most the whole stencil
            half_totals = [(int(rng.integers(n, t + 1)), int(rng.integers(n, t + 1)))
                           for n, t in zip(occupancy, totals)]
            starts = np.concatenate([[0], np.cumsum(occupancy)])
            n_all = int(starts[-1])
            units = list_units_halves(occupancy, mids, totals, half_totals, cap)
            assert len(units) <= ((n_all + WARP - 1) // WARP + 2 * ncell) * SPLIT_ROUNDS
            covered = {}
            for ex, u in units:
                c, half = ex >> 1, ex & 1
                c0 = int(starts[c])
                g0 = c0 + int(mids[c]) if half == 1 else c0
                g1 = c0 + int(mids[c]) if half == 0 else int(starts[c + 1])
                total = half_totals[c][half]
                rounds = (total + cap - 1) // cap
                k, r = divmod(u, rounds)
                ig = g0 + k * WARP
                gi = min(WARP, g1 - ig)
                assert 0 < gi <= WARP and ig + gi <= g1 and r < rounds <= SPLIT_ROUNDS
                assert 0 < min(cap, total - r * cap) <= cap
                # the own cell is stencil entry 4 whatever the half: i's staged
                # index stays inside the staged list
                for p in range(ig, ig + gi):
                    assert 0 <= p - c0 < occupancy[c] <= total
                    covered[(p, r)] = covered.get((p, r), 0) + 1
            for c in range(ncell):
                if unit_cell(int(occupancy[c]), int(totals[c]), cap):
                    for p in range(int(starts[c]), int(starts[c + 1])):
                        half = int(p - starts[c] >= mids[c])
                        rounds = (half_totals[c][half] + cap - 1) // cap
                        for r in range(rounds):
                            assert covered.pop((p, r)) == 1
            assert not covered
