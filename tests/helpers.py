"""Shared inputs for the parity tests (seeded, sized for the oracle)."""
import numpy as np

from oracle.ns_ref import Grid


def random_state(grid: Grid, seed=0, kdecay=None, solenoidal=True):
    """Seeded random velocity spectrum of a real field inside the 2/3 set."""
    rng = np.random.default_rng(seed)
    shp = (3,) + grid.spec_shape
    uh = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp))
    if kdecay is None:
        kdecay = max(grid.N) / 4.0
    uh *= np.exp(-grid.K2 / (2 * kdecay ** 2 * (2 * np.pi / grid.L[0]) ** 2))
    u = np.fft.irfftn(uh, s=grid.N, axes=(1, 2, 3))
    uh = grid.forward(u) * grid.mask
    if solenoidal:
        P = sum(grid.K[i] * uh[i] for i in range(3))
        for i in range(3):
            uh[i] -= P * grid.K_over_K2[i]
    return uh.astype(grid.cdtype)


def relerr(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
