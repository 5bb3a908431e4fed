"""Host-side helpers of bench.py's roofline, on the CPU: the candidate count
of the cell-list passes (3x3 stencil members per particle) against a direct
count, and the tuning a candidate sets on a handle."""
import numpy as np

import bench


def test_candidates_per_particle_matches_a_direct_count():
    w = dict(bench.WORKLOAD, n=2000, L=2.0, rho=0.25)
    rng = np.random.default_rng(3)
    st = np.empty(3 * w["n"])
    st[0::3] = rng.uniform(0.0, w["L"], w["n"])
    st[1::3] = rng.uniform(0.0, w["L"], w["n"])
    st[2::3] = 0.0
    nc = int(w["L"] / w["rho"])
    cx = np.minimum((st[0::3] / w["L"] * nc).astype(int), nc - 1)
    cy = np.minimum((st[1::3] / w["L"] * nc).astype(int), nc - 1)
    direct = []
    for i in range(w["n"]):
        dx = (cx - cx[i] + 1) % nc
        dy = (cy - cy[i] + 1) % nc
        direct.append(np.count_nonzero((dx <= 2) & (dy <= 2)))
    assert bench.candidates_per_particle(w, st) == np.mean(direct)


def test_apply_tuning_sets_every_knob():
    class Handle:
        def __init__(self):
            self.set = {}

        def set_tuning(self, key, value):
            self.set[key] = value

    class Abi:
        TUNE_SPARSE_BELOW, TUNE_TILE_SPLIT, TUNE_CELL_UNITS, TUNE_SUBCELLS = 1, 3, 4, 5

    h = Handle()
    bench.apply_tuning(Abi, h, {"sparse_below": 24.0, "tile_split": 2, "cell_units": 1, "subcells": 1})
    assert h.set == {1: 24.0, 3: 2, 4: 1, 5: 1}
    h = Handle()
    bench.apply_tuning(Abi, h, {"sparse_below": 0.0, "tile_split": 1})  # no cell-unit / sub-cell keys
    assert h.set == {1: 0.0, 3: 1, 4: 0, 5: 0}
