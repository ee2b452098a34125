"""energy_fourier of shenfun.fourier: sum over the full spectrum of |u_hat|^2
(the Hermitian half array counts the interior kz modes twice)."""
import numpy as np


def energy_fourier(u, T=None):
    u = np.asarray(u)
    w = np.full(u.shape[-1], 2.0)
    w[0] = 1.0
    n2 = None
    if T is not None and hasattr(T, "N"):
        n2 = int(T.N[-1])
    if n2 is None or n2 % 2 == 0:
        w[-1] = 1.0
    return float(np.sum((u.real.astype(np.float64) ** 2 + u.imag.astype(np.float64) ** 2) * w))
