"""GPU parity of the velocity-vorticity solver (spectralDNS solvers/VV.py) against
the oracle's restatement, and the reference's VV runs of tests/test_NSVV.py
through the driver API.

Tolerances as the NS parity tests: FP64 1e-11 relative, FP32 2e-5 (fields,
right-hand sides) and 1e-5 (energies).
"""
import numpy as np
import pytest

from oracle.ns_ref import Grid, taylor_green
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-11, "single": 2e-5}
GRIDS = [((16, 16, 16), (2 * np.pi,) * 3), ((32, 32, 32), (2 * np.pi,) * 3),
         ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi)), ((16, 16, 512), (2 * np.pi,) * 3),
         ((128, 64, 64), (2 * np.pi,) * 3)]


def vv_ctx(N, L, prec, nu=0.000625):
    from spectraldns_gb300.gpu import Context
    return Context(N, L, nu=nu, precision=prec, formulation="VV")


def vorticity(g, seed):
    return g.curl_hat(random_state(g, seed=seed))


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", GRIDS)
def test_vv_compute_rhs(built_lib, N, L, prec):
    g = Grid(N, L)
    wh = vorticity(g, 7)
    ref = g.compute_rhs_vv(wh)
    c = vv_ctx(N, L, prec)
    rhs = c.compute_rhs(wh.astype(c.complex))
    assert relerr(rhs, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["double", "single"])
def test_vv_rk4_and_diagnostics(built_lib, prec):
    N, L = (32, 32, 32), (2 * np.pi,) * 3
    g = Grid(N, L)
    wh = vorticity(g, 8) * 20
    c = vv_ctx(N, L, prec)
    c.set_state(wh.astype(c.complex))
    c.rk4(0.005, 4)
    ref = wh
    for _ in range(4):
        ref = g.rk4_step(ref, 0.005, vv=True)
    assert relerr(c.get_state(), ref) < (1e-11 if prec == "double" else 2e-5)
    d = c.diagnostics()
    uref = g.velocity_of_vorticity(ref)
    tol = 1e-11 if prec == "double" else 1e-5
    assert abs(d["energy"] - g.kinetic_energy(uref)) < tol * g.kinetic_energy(uref)
    enst = 0.5 * g.mean_square(g.backward(ref))
    assert abs(d["enstrophy"] - enst) < tol * enst
    assert abs(d["dissipation"] - 2 * g.nu * enst) < tol * 2 * g.nu * enst
    assert d["divergence"] < 1e-20
    # getters: the velocity of the state, and of a given vorticity vector
    assert relerr(c.velocity(), g.backward(uref)) < (1e-11 if prec == "double" else 2e-5)
    assert relerr(c.velocity_vv(ref.astype(c.complex)), g.backward(uref)) < (1e-11 if prec == "double" else 2e-5)
    assert np.max(np.abs(c.divergence())) < (1e-11 if prec == "double" else 1e-4) * np.max(np.abs(c.velocity()))
    # shell spectrum of the velocity
    ek_ref, _ = g.spectrum(uref)
    assert relerr(c.spectrum(len(ek_ref)), ek_ref) < (1e-11 if prec == "double" else 1e-5)


def test_vv_rejects_pressure_and_forcing(built_lib):
    from spectraldns_gb300._lib import SdnsError
    c = vv_ctx((16, 16, 16), (2 * np.pi,) * 3, "double")
    with pytest.raises(SdnsError):
        c.pressure()
    with pytest.raises(SdnsError):
        c.set_forcing(0.1, 2.0)


@pytest.mark.parametrize("integrator,ntol", [("RK4", 7), ("BS5_adaptive", 7), ("AB2", 4)])
@pytest.mark.parametrize("mesh", ["uniform", "nonuniform"])
def test_vv_solver_api(built_lib, mesh, integrator, ntol):
    """tests/test_NSVV.py 'VV/uniform' and 'VV/nonuniform': TG to T = 0.1 through the driver
    API, regression test of tests/TG.py:116-126 (velocity and curl from W_hat)."""
    from spectraldns_gb300 import config, get_solver, solve
    from tests.test_api_gpu import regression_test
    args = ["--M", "4", "4", "4", "--L", "2*pi", "2*pi", "2*pi"] if mesh == "uniform" else \
        ["--M", "6", "5", "4", "--L", "6*pi", "4*pi", "2*pi"]
    config.update({"nu": 0.000625, "dt": 0.01, "T": 0.1, "convection": "Vortex"})
    solver = get_solver(regression_test=regression_test, update=lambda c: None, parse_args=args + ["VV"])
    context = solver.get_context()
    assert "P_hat" not in context and context.u is context.W_hat
    config.params.integrator = integrator
    config.params.ntol = ntol
    # tests/TG.py initialize2: U from the TG formula, U_hat = F(U), W_hat = i K x U_hat
    U, X = context.U, context.X
    U[0] = np.sin(X[0]) * np.cos(X[1]) * np.cos(X[2])
    U[1] = -np.cos(X[0]) * np.sin(X[1]) * np.cos(X[2])
    U[2] = 0
    solver.set_velocity(**context)
    solver.cross2(context.W_hat, context.K, context.U_hat)
    config.params.t = 0.0
    config.params.tstep = 0
    solve(solver, context)
    div = solver.get_divergence(**context)
    assert np.max(np.abs(div)) < 1e-10


@pytest.mark.parametrize("prec", ["double", "single"])
def test_vv_cfl_step(built_lib, prec):
    """VV with the CFL time step: the z sweep's velocity fields are i K x w / K^2, so dt comes
    from the velocity of the vorticity state, as for NS."""
    N, L = (32, 32, 32), (2 * np.pi,) * 3
    g = Grid(N, L, nu=0.01)
    wh = vorticity(g, 12) * 20
    c = vv_ctx(N, L, prec, nu=0.01)
    c.set_state(wh.astype(c.complex))
    c.set_cfl(0.5)
    c.rk4(0.0, 1)
    d = c.diagnostics()
    rate = g.cfl_rate(g.velocity_of_vorticity(wh))
    dt = 0.5 / rate
    assert abs(d["last_dt"] - dt) < (1e-12 if prec == "double" else 1e-5) * dt
    ref = g.rk4_step(wh, dt, vv=True)
    assert relerr(c.get_state(), ref) < (1e-11 if prec == "double" else 2e-5)
