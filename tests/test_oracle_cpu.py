"""The oracle against the reference's own known answers and fixtures (CPU only)."""
import os
import sys

import numpy as np
import pytest

from oracle.ns_ref import Grid, dealias_cutoff, run_tg, taylor_green

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "short64.npz")
sys.path.insert(0, os.path.join(HERE, "golden"))


@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3), ((32, 32, 32), (2 * np.pi,) * 3),
                                 ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_tg_known_answers(N, L):
    """tests/TG.py:125-126 (7 digits, ntol default config.py:196)."""
    k, w, _ = run_tg(N, L=L)
    assert round(k - 0.124953117517, 7) == 0
    assert round(w - 0.375249930801, 7) == 0


def test_short_script_tg_state():
    """State after 10 RK4 steps equals the reference's spectralDNS3D_short.py (N=64)."""
    d = np.load(GOLD)
    N = int(d["N"])
    S = float(N ** 3)  # the short script's forward transform is unnormalised
    _, _, uh = run_tg((N, N, N))
    idx = tuple(d["tg_idx"].astype(int).T)
    assert np.max(np.abs(uh[idx] * S - d["tg_val"])) / np.max(np.abs(d["tg_val"])) < 1e-14
    mask = np.ones(uh.shape, bool)
    mask[idx] = False
    assert np.abs(uh[mask]).max() * S < 1e-9
    assert abs(float(d["tg_k"]) - 0.124953117517) < 5e-13


def test_short_script_compute_rhs():
    """ComputeRHS on a seeded random field equals the short script's (N=64)."""
    from make_golden import random_input
    d = np.load(GOLD)
    N = int(d["N"])
    S = float(N ** 3)
    g = Grid((N, N, N))
    rhs = g.compute_rhs(random_input(int(d["rhs_seed"]), N) / S) * S
    idx = tuple(d["rhs_idx"].astype(int).T)
    assert np.max(np.abs(rhs[idx] - d["rhs_val"])) / np.max(np.abs(d["rhs_val"])) < 1e-13


def test_dealias_cutoffs():
    # |k| < 2/3 (N/2+1)
    assert [dealias_cutoff(n) for n in (16, 32, 64, 128, 256, 512, 1024)] == [5, 11, 21, 43, 85, 171, 341]
    assert dealias_cutoff(32, "None") == 15


def test_parseval_and_divergence_free():
    g = Grid((32, 32, 32))
    uh = g.forward(taylor_green(g))
    assert abs(0.5 * g.energy_fourier(uh) - g.kinetic_energy(uh)) < 1e-14
    assert g.divergence_ms(uh) < 1e-28
    rhs = g.compute_rhs(uh)
    assert np.max(np.abs(sum(g.K[i] * (rhs[i] + g.nu * g.K2 * uh[i]) for i in range(3)))) < 1e-12


def test_forcing_injects_eps():
    from spectraldns_gb300.init import isotropic_field
    g = Grid((32, 32, 32), nu=0.0)
    uh = isotropic_field((32, 32, 32), k0=2.0, seed=3, dtype=np.complex128)
    src = g.forcing_source(uh, 0.1, 2.0)
    w = g.hermitian_weights()
    power = float(np.sum((np.conj(uh) * src).real * w))
    assert abs(power - 0.1) < 1e-12


def test_isotropic_field_properties():
    from spectraldns_gb300.init import isotropic_field
    g = Grid((64, 64, 64))
    uh = isotropic_field((64, 64, 64), k0=4.0, energy=0.5, seed=0, dtype=np.complex128)
    assert abs(0.5 * g.energy_fourier(uh) - 0.5) < 1e-6
    assert g.divergence_ms(uh) < 1e-12
    assert np.abs(uh * (~g.mask)).max() == 0
    assert np.abs(g.forward(g.backward(uh)) - uh).max() < 1e-12  # spectrum of a real field
    E = g.shell_spectrum(uh)
    assert 3 <= int(np.argmax(E)) <= 5  # k^4 exp(-2 (k/4)^2) peaks at k = 4


@pytest.mark.parametrize("method,ntol", [("ForwardEuler", 4), ("AB2", 4), ("BS5_fixed", 7), ("BS5_adaptive", 7)])
@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3), ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_integrators_known_answers(method, ntol, N, L):
    """tests/test_NSVV.py::test_integrators: TG to T = 0.1 meets tests/TG.py:125-126
    to ntol digits (4 for ForwardEuler/AB2, 7 otherwise)."""
    from oracle.ns_ref import Integrator
    g = Grid(N, L)
    uh = g.forward(taylor_green(g))
    it = Integrator(g, method, tol=1e-6)
    t, dt, tstep, T = 0.0, 0.01, 0, 0.1
    while t + dt <= T + 1e-12:
        uh, dt_next, took = it.step(uh, dt, tstep)
        t += took
        tstep += 1
        dt = dt_next
        if abs(t - T) < 1e-12:
            break
        if abs(t + dt - T) < 1e-12 or t + dt >= T + 1e-12:
            dt = T - t
    assert abs(t - T) < 1e-12
    assert round(g.kinetic_energy(uh) - 0.124953117517, ntol) == 0
    assert round(g.enstrophy(uh) - 0.375249930801, ntol) == 0


def test_bs5_tableau_consistent():
    """Row sums give the nodes; b and bhat are consistent (sum 1); FSAL: A[7] == b."""
    from oracle.ns_ref import bs5_tableau
    from spectraldns_gb300.integrators import _rows
    A, b, bhat = bs5_tableau()
    assert abs(b.sum() - 1) < 1e-15 and abs(bhat.sum() - 1) < 1e-15
    assert np.array_equal(A[7], b)
    c = A.sum(axis=1)
    assert np.allclose(c, [0, 1 / 6, 2 / 9, 3 / 7, 2 / 3, 3 / 4, 1, 1], atol=1e-15)
    # the GPU driver's tableau is the same table
    Ag, bg, bhg = _rows(np.float64)
    for i in range(8):
        assert np.allclose(A[i, :i], Ag[i], rtol=0, atol=0)
    assert np.allclose(b, bg, rtol=0, atol=0) and np.allclose(bhat, bhg, rtol=0, atol=0)


@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3), ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_vv_known_answers(N, L):
    """tests/test_NSVV.py runs the VV solver on TG (initialize2: W_hat = i K x U_hat) against
    tests/TG.py:125-126; the VV state stays the curl of the NS state."""
    g = Grid(N, L)
    uh = g.forward(taylor_green(g))
    wh = g.curl_hat(uh)
    for _ in range(10):
        wh = g.rk4_step(wh, 0.01, vv=True)
        uh = g.rk4_step(uh, 0.01)
    U = g.backward(g.velocity_of_vorticity(wh))
    assert round(0.5 * g.mean_square(U) - 0.124953117517, 7) == 0
    assert round(0.5 * g.mean_square(g.backward(wh)) - 0.375249930801, 7) == 0
    assert np.max(np.abs(wh - g.curl_hat(uh))) < 1e-13


@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3), ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_three_halves_rule_known_answers(N, L):
    """tests/test_NSVV.py::test_solvers reruns TG with dealias '3/2-rule' against tests/TG.py:125-126."""
    g = Grid(N, L, dealias="3/2-rule")
    uh = g.forward(taylor_green(g))
    for _ in range(10):
        uh = g.rk4_step(uh, 0.01)
    assert round(g.kinetic_energy(uh) - 0.124953117517, 7) == 0
    assert round(g.enstrophy(uh) - 0.375249930801, 7) == 0


def test_three_halves_rule_is_alias_free():
    """The padded product of two N-mode fields equals the exact product (formed on a 2N grid,
    where a quadratic term cannot alias), truncated to the N modes."""
    g = Grid((16, 16, 16), dealias="3/2-rule")
    rng = np.random.default_rng(0)
    a = g.forward(rng.standard_normal((3, 16, 16, 16))) * g.mask
    b = g.forward(rng.standard_normal((3, 16, 16, 16))) * g.mask
    nl = g._nonlinear(a, b)
    g2 = Grid((32, 32, 32))
    i0, t0, kz = np.r_[0:8, 9:16], np.r_[0:8, 25:32], np.arange(8)
    src = (slice(None), i0[:, None, None], i0[None, :, None], kz[None, None, :])
    dst = (slice(None), t0[:, None, None], t0[None, :, None], kz[None, None, :])

    def up(x):
        X = np.zeros((3, 32, 32, 17), complex)
        X[dst] = x[src]
        return X
    ex = g2.forward(g2.cross(g2.backward(up(a)), g2.backward(up(b))))
    exs = np.zeros_like(nl)
    exs[src] = ex[dst]
    assert np.abs(nl - exs).max() < 1e-14 * np.abs(exs).max()
    # the 2/3 rule on the same (unpadded) grid is a different, truncating approximation
    assert np.abs(Grid((16, 16, 16))._nonlinear(a, b) - exs).max() > 1e-3 * np.abs(exs).max()


def test_three_halves_rule_vv_is_curl_of_ns():
    """With the 3/2 rule as well, the velocity-vorticity trajectory of a zero-mean solenoidal field
    is the curl of the velocity trajectory (the padded nonlinear terms agree: i K x P(nl) = i K x nl)."""
    g = Grid((16, 16, 16), dealias="3/2-rule")
    uh = g.forward(taylor_green(g))
    rng = np.random.default_rng(3)
    pert = g.forward(rng.standard_normal((3,) + g.N)) * g.mask * 0.05
    P = sum(g.K[i] * pert[i] for i in range(3))
    for i in range(3):
        pert[i] -= P * g.K_over_K2[i]
    pert[:, 0, 0, 0] = 0  # the VV form carries no mean flow (i K x w / K^2 is 0 at K = 0)
    uh = uh + pert
    wh = g.curl_hat(uh)
    for _ in range(5):
        uh = g.rk4_step(uh, 0.01)
        wh = g.rk4_step(wh, 0.01, vv=True)
    assert np.max(np.abs(wh - g.curl_hat(uh))) < 1e-13 * np.max(np.abs(wh))
