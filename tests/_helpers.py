"""Shared inputs and comparisons for the parity tests."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def init_state(n, L, seed):
    """x, y ~ U[0, L), phi ~ U[-pi, pi) from numpy PCG64(seed)."""
    rng = np.random.default_rng(seed)
    s = np.empty(3 * n)
    s[0::3] = rng.uniform(0.0, L, n)
    s[1::3] = rng.uniform(0.0, L, n)
    s[2::3] = rng.uniform(-np.pi, np.pi, n)
    return s


def golden_cases():
    """The ChimeraSystem fixtures (vector and shared-window classes)."""
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith("va_"))


def va_golden_cases():
    """The VortexArraysSystemPtr fixtures."""
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "va_*.npz")))


VA_KEYS = ("velocity", "mu_plus", "mu_minus", "xi_a", "xi_r", "D_phi", "kappa", "rho")


def va_params(g):
    return {k: float(g[k]) for k in VA_KEYS}


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def periodic_diff(a, b, L):
    """Element-wise difference of two AoS states, x/y by minimum image."""
    d = (a - b).reshape(-1, 3).copy()
    d[:, :2] -= L * np.round(d[:, :2] / L)
    return d


def alignment_scale(state, offsets, idx, sigma, alpha):
    """(sigma / n_i) sum_j |sin(phi_j - phi_i - alpha)|: the magnitude against
    which a phase rate's rounding error is measured (a near-cancelling sum has
    no meaningful pure relative error)."""
    n = state.size // 3
    phi = state[2::3]
    counts = np.diff(offsets)
    owner = np.repeat(np.arange(n), counts)
    terms = np.abs(np.sin(phi[idx] - phi[owner] - alpha))
    sums = np.bincount(owner, weights=terms, minlength=n)
    with np.errstate(divide="ignore", invalid="ignore"):
        scale = np.where(counts > 0, sigma * sums / np.maximum(counts, 1), 0.0)
    return scale, counts
