"""Initial conditions of the benchmark flows (host side, run once).

* :func:`taylor_green` -- demo/TG.py:23-28 (u = sin x cos y cos z,
  v = -cos x sin y cos z, w = 0) on the physical mesh.
* :func:`isotropic_field` -- build-defined seeded solenoidal field with
  spectrum E(k) ~ k^4 exp(-2 (k/k0)^2), uniform random phases, zero mean,
  inside the dealiased set and scaled to a total kinetic energy
  1/2 sum|u_hat|^2.  The reference's own Rogallo initialisation
  (demo/Isotropic.py:29-76) is a different construction; this one is the
  spectrum the forced/decaying benchmark cases prescribe.
"""
from __future__ import annotations

import math

import numpy as np


def mesh(N, L):
    return [np.arange(N[i]) * (L[i] / N[i]) for i in range(3)]


def taylor_green(N, L=(2 * np.pi,) * 3, dtype=np.float64):
    x0, x1, x2 = mesh(N, L)
    x0 = x0[:, None, None]
    x1 = x1[None, :, None]
    x2 = x2[None, None, :]
    U = np.empty((3,) + tuple(N), dtype=dtype)
    U[0] = np.sin(x0) * np.cos(x1) * np.cos(x2)
    U[1] = -np.cos(x0) * np.sin(x1) * np.cos(x2)
    U[2] = 0
    return U


def dealias_cutoff(n, rule="2/3-rule"):
    if rule == "None":
        return n // 2 - 1
    kmax = 2.0 / 3.0 * (n // 2 + 1)
    kc = int(math.ceil(kmax)) - 1
    while kc + 1 < kmax:
        kc += 1
    while kc >= kmax:
        kc -= 1
    return kc


def isotropic_field(N, L=(2 * np.pi,) * 3, k0=4.0, energy=0.5, seed=0, dealias="2/3-rule",
                    dtype=np.complex64):
    """Seeded solenoidal spectrum (3, N0, N1, N2//2+1) with E(k) ~ k^4 exp(-2(k/k0)^2)."""
    N = tuple(int(n) for n in N)
    n0, n1, n2 = N
    kc = [dealias_cutoff(n, dealias) for n in N]
    # integer wave indices of the kept rows (FFT order) and their array positions
    j0 = np.concatenate([np.arange(0, kc[0] + 1), np.arange(-kc[0], 0)])
    j1 = np.concatenate([np.arange(0, kc[1] + 1), np.arange(-kc[1], 0)])
    j2 = np.arange(0, kc[2] + 1)
    p0 = np.mod(j0, n0)
    p1 = np.mod(j1, n1)
    s = [2 * np.pi / L[i] for i in range(3)]
    K = [(j0 * s[0]).astype(np.float32)[:, None, None], (j1 * s[1]).astype(np.float32)[None, :, None],
         (j2 * s[2]).astype(np.float32)[None, None, :]]
    K2 = K[0] ** 2 + K[1] ** 2 + K[2] ** 2
    kmag = np.sqrt(K2)
    with np.errstate(divide="ignore", invalid="ignore"):
        Ek = kmag ** 4 * np.exp(-2.0 * (kmag / k0) ** 2)
        amp = np.where(K2 > 0, np.sqrt(Ek / (4 * np.pi * np.where(K2 > 0, K2, 1))), 0).astype(np.float32)
    rng = np.random.default_rng(seed)
    shp = (3,) + K2.shape
    theta = rng.random(shp, dtype=np.float32) * np.float32(2 * np.pi)
    uc = (np.cos(theta) + 1j * np.sin(theta)).astype(np.complex64)
    del theta
    uc *= amp
    # project onto k . u = 0
    K2n = np.where(K2 > 0, K2, 1).astype(np.float32)
    P = (K[0] * uc[0] + K[1] * uc[1] + K[2] * uc[2]) / K2n
    for i in range(3):
        uc[i] -= P * K[i]
    del P
    # Hermitian symmetry of the kz = 0 plane (a real field)
    r0 = np.mod(-j0, 2 * kc[0] + 1)
    r1 = np.mod(-j1, 2 * kc[1] + 1)
    pl = uc[:, :, :, 0]
    uc[:, :, :, 0] = 0.5 * (pl + np.conj(pl[:, r0][:, :, r1]))
    uc[:, 0, 0, 0] = 0
    # energy with the Hermitian weights (kz = 0 once, kz > 0 twice), summed in FP64
    e = 0.0
    for i in range(3):
        a2 = uc[i].real ** 2 + uc[i].imag ** 2
        e += 2.0 * float(np.sum(a2, dtype=np.float64)) - float(np.sum(a2[..., 0], dtype=np.float64))
    del a2
    e *= 0.5
    uc *= np.float32(math.sqrt(energy / e)) if e > 0 else 0
    out = np.zeros((3, n0, n1, n2 // 2 + 1), dtype=dtype)
    out[:, p0[:, None], p1[None, :], :kc[2] + 1] = uc
    return out
