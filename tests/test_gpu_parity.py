"""GPU parity tests: the CUDA library against the float64 oracle.

Tolerances: FP64 runs must agree to 1e-11 relative (rounding only); FP32
runs (FP32 transforms, FP64 RK4 accumulators) to 2e-5 relative on fields
and RHS and 1e-5 on energies.
"""
import numpy as np
import pytest

from oracle.ns_ref import Grid, taylor_green, RK4_A
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-11, "single": 2e-5}
GRIDS = [((16, 16, 16), (2 * np.pi,) * 3), ((32, 32, 32), (2 * np.pi,) * 3),
         ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi)), ((64, 64, 64), (2 * np.pi,) * 3)]


def ctx(N, L, prec, **kw):
    from spectraldns_gb300.gpu import Context
    return Context(N, L, nu=kw.pop("nu", 0.000625), precision=prec, **kw)


# 1024-point axes (the E = 32 line kernels of the 1024^3 case) in each direction
LONG = [((16, 16, 1024), (2 * np.pi,) * 3), ((1024, 16, 16), (2 * np.pi,) * 3), ((16, 1024, 16), (2 * np.pi,) * 3)]


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", GRIDS + [((128, 128, 128), (2 * np.pi,) * 3), ((256, 16, 32), (2 * np.pi,) * 3)] + LONG)
def test_transforms(built_lib, N, L, prec):
    g = Grid(N, L)
    c = ctx(N, L, prec)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((3,) + g.N)
    uh_ref = g.forward(u)
    uh = c.forward(u.astype(c.real))
    assert relerr(uh, uh_ref) < TOL[prec] * 5
    back = c.backward(uh_ref.astype(c.complex))
    assert relerr(back, g.backward(uh_ref)) < TOL[prec] * 5
    # single field
    s = c.backward(uh_ref[1].astype(c.complex))
    assert relerr(s, g.backward(uh_ref[1])) < TOL[prec] * 5


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", GRIDS + [((16, 16, 512), (2 * np.pi,) * 3), ((16, 32, 256), (2 * np.pi,) * 3),
                                          ((128, 16, 128), (2 * np.pi,) * 3)] + LONG)
def test_compute_rhs(built_lib, N, L, prec):
    g = Grid(N, L)
    uh = random_state(g, seed=3)
    ref = g.compute_rhs(uh)
    c = ctx(N, L, prec)
    rhs = c.compute_rhs(uh.astype(c.complex))
    assert relerr(rhs, ref) < TOL[prec]


def test_compute_rhs_outside_modes(built_lib):
    """Modes outside the 2/3 set get rhs = -nu K^2 u_hat (NS.py:215) and do not feed back."""
    N, L = (32, 32, 32), (2 * np.pi,) * 3
    g = Grid(N, L)
    rng = np.random.default_rng(7)
    uh = (rng.standard_normal((3,) + g.spec_shape) + 1j * rng.standard_normal((3,) + g.spec_shape)) * 1e-2
    u = g.backward(uh)
    uh = g.forward(u)
    ref = g.compute_rhs(uh)
    c = ctx(N, L, "double")
    assert relerr(c.compute_rhs(uh), ref) < 1e-11


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", GRIDS[:3] + LONG[:2])
def test_rk4_random(built_lib, N, L, prec):
    g = Grid(N, L, nu=0.01)
    uh = random_state(g, seed=5)
    c = ctx(N, L, prec, nu=0.01)
    c.set_state(uh.astype(c.complex))
    ref = uh.copy()
    for _ in range(3):
        ref = g.rk4_step(ref, 0.002)
    c.rk4(0.002, 3)
    out = c.get_state()
    assert relerr(out, ref) < (1e-11 if prec == "double" else 2e-5)
    d = c.diagnostics()
    assert abs(d["energy"] - g.kinetic_energy(ref)) < 1e-12 + 1e-6 * (prec == "single")
    assert abs(d["time"] - 0.006) < 1e-14


@pytest.mark.parametrize("N,L", [((32, 32, 32), (2 * np.pi,) * 3), ((16, 16, 16), (2 * np.pi,) * 3),
                                 ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_tg_known_answer(built_lib, N, L):
    """tests/TG.py:125-126: k and w after 10 steps of dt=0.01, 7 digits (FP64)."""
    g = Grid(N, L)
    c = ctx(N, L, "double")
    uh0 = c.forward(taylor_green(g))
    c.set_state(uh0)
    c.rk4(0.01, 10)
    U = c.velocity()
    W = c.curl()
    k = 0.5 * np.sum(U.astype(np.float64) ** 2) / np.prod(N)
    w = 0.5 * np.sum(W.astype(np.float64) ** 2) / np.prod(N)
    assert round(k - 0.124953117517, 7) == 0, k
    assert round(w - 0.375249930801, 7) == 0, w
    d = c.diagnostics()
    assert abs(d["energy"] - k) < 1e-13
    assert abs(d["enstrophy"] - w) < 1e-12


def test_tg_fp32_drift(built_lib):
    """FP32 run: TG energy within 1e-5 relative of the float64 oracle after 100 steps."""
    N = (32, 32, 32)
    g = Grid(N)
    ref = g.forward(taylor_green(g))
    c = ctx(N, (2 * np.pi,) * 3, "single")
    c.set_state(ref.astype(np.complex64))
    for _ in range(100):
        ref = g.rk4_step(ref, 0.01)
    c.rk4(0.01, 100)
    e = c.diagnostics()["energy"]
    assert abs(e - g.kinetic_energy(ref)) / g.kinetic_energy(ref) < 1e-5


def test_tg_config0_fp64_100_steps(built_lib):
    """The Taylor-Green case of the reference's CPU demo run (32^3, float64, nu = 0.000625,
    dt = 0.01, 100 RK4 steps, 2/3 rule): state against the float64 oracle to 1e-11 relative, and
    energy, enstrophy and dissipation every 10 steps to 1e-12 relative."""
    N = (32, 32, 32)
    g = Grid(N)
    ref = g.forward(taylor_green(g))
    c = ctx(N, (2 * np.pi,) * 3, "double")
    c.set_state(ref)
    for _ in range(10):
        for _ in range(10):
            ref = g.rk4_step(ref, 0.01)
        c.rk4(0.01, 10)
        d = c.diagnostics()
        k, w = g.kinetic_energy(ref), g.enstrophy(ref)
        assert abs(d["energy"] - k) < 1e-12 * k
        assert abs(d["enstrophy"] - w) < 1e-12 * w
        assert abs(d["dissipation"] - g.dissipation(ref)) < 1e-12 * g.dissipation(ref)
    assert relerr(c.get_state(), ref) < 1e-11
    assert abs(d["time"] - 1.0) < 1e-12


def test_diagnostics_and_spectrum(built_lib):
    N = (32, 32, 32)
    g = Grid(N)
    uh = random_state(g, seed=11)
    c = ctx(N, (2 * np.pi,) * 3, "double")
    c.set_state(uh)
    d = c.diagnostics()
    assert abs(d["energy"] - g.kinetic_energy(uh)) < 1e-13 * max(1, g.kinetic_energy(uh))
    assert abs(d["enstrophy"] - g.enstrophy(uh)) < 1e-12 * max(1, g.enstrophy(uh))
    assert abs(d["dissipation"] - g.dissipation(uh)) < 1e-12 * max(1, g.dissipation(uh))
    assert d["divergence"] < 1e-20
    Ek, _ = g.spectrum(uh)
    assert relerr(c.spectrum(len(Ek)), Ek) < 1e-12
    assert relerr(c.divergence(), g.backward(1j * sum(g.K[i] * uh[i] for i in range(3)))) < 1e-6 or \
        np.max(np.abs(c.divergence())) < 1e-12


@pytest.mark.parametrize("prec", ["double", "single"])
def test_forcing_and_cfl_step(built_lib, prec):
    """One RK4 step with constant-power forcing (Source from the step-start state) and the CFL
    time step dt = cfl / max(|u|/dx + |v|/dy + |w|/dz), against the oracle."""
    from spectraldns_gb300.init import isotropic_field
    N = (32, 32, 32)
    g = Grid(N, nu=0.01)
    uh = isotropic_field(N, k0=3.0, energy=0.5, seed=4, dtype=np.complex128)
    c = ctx(N, (2 * np.pi,) * 3, prec, nu=0.01)
    c.set_forcing(0.1, 2.0)
    c.set_cfl(0.5)
    c.set_state(uh.astype(c.complex))
    c.rk4(0.0, 1)
    rate = g.cfl_rate(uh)
    dt = 0.5 / rate
    ref = g.rk4_step(uh, dt, source=g.forcing_source(uh, 0.1, 2.0))
    d = c.diagnostics()
    tol = 1e-11 if prec == "double" else 2e-5
    assert abs(d["cfl_rate"] - rate) / rate < (1e-13 if prec == "double" else 1e-6)
    assert abs(d["last_dt"] - dt) / dt < (1e-13 if prec == "double" else 1e-6)
    assert relerr(c.get_state(), ref) < tol
    # the forcing injects eps at the step start: energy grows by ~eps*dt - dissipation*dt
    assert abs(d["time"] - dt) < 1e-12 + 1e-6 * dt


def test_source_term(built_lib):
    """ComputeRHS adds a user Source (NS.py:259), inside and outside the dealiased set."""
    N = (32, 32, 32)
    g = Grid(N)
    uh = random_state(g, seed=8)
    rng = np.random.default_rng(9)
    src = g.forward(rng.standard_normal((3,) + N)) * 0.1
    c = ctx(N, (2 * np.pi,) * 3, "double")
    c.set_source(src)
    assert relerr(c.compute_rhs(uh), g.compute_rhs(uh, source=src)) < 1e-11
    c.set_source(None)
    assert relerr(c.compute_rhs(uh), g.compute_rhs(uh)) < 1e-11
