"""GPU parity of the 3/2-rule (padded) path: spectralDNS solvers/NS.py:29-31 with
padding_factor 1.5, and the VV solver on the same transforms, against the
oracle's restatement (Grid(dealias="3/2-rule")).

Tolerances: FP64 1e-11 relative, FP32 2e-5 (fields, right-hand sides).
"""
import numpy as np
import pytest

from oracle.ns_ref import Grid, taylor_green
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-11, "single": 2e-5}
GRIDS = [((16, 16, 16), (2 * np.pi,) * 3), ((32, 32, 32), (2 * np.pi,) * 3),
         ((64, 32, 16), (6 * np.pi, 4 * np.pi, 2 * np.pi)), ((32, 16, 64), (2 * np.pi,) * 3),
         ((128, 128, 128), (2 * np.pi,) * 3)]


def ctx(N, L, prec, formulation="NS", **kw):
    from spectraldns_gb300.gpu import Context
    return Context(N, L, precision=prec, dealias="3/2-rule", formulation=formulation, **kw)


def full_state(g, seed):
    """Seeded random spectrum using every mode but the Nyquist ones (solenoidal)."""
    rng = np.random.default_rng(seed)
    u = rng.standard_normal((3,) + g.N)
    uh = g.forward(u) * g.mask
    P = sum(g.K[i] * uh[i] for i in range(3))
    for i in range(3):
        uh[i] -= P * g.K_over_K2[i]
    return uh


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", GRIDS)
def test_pad32_compute_rhs(built_lib, N, L, prec):
    g = Grid(N, L, dealias="3/2-rule")
    uh = full_state(g, 3)
    c = ctx(N, L, prec, store_pressure=True)
    rhs = c.compute_rhs(uh.astype(c.complex))
    ref, parts = g.compute_rhs(uh, return_parts=True)
    assert relerr(rhs, ref) < TOL[prec]
    # the pressure of that evaluation
    Pref = g.backward(parts["P_hat"][None])[0]
    assert relerr(c.pressure(), Pref) < TOL[prec] * 10


@pytest.mark.parametrize("prec", ["double", "single"])
def test_pad32_vv_compute_rhs(built_lib, prec):
    N, L = (32, 32, 16), (2 * np.pi,) * 3
    g = Grid(N, L, dealias="3/2-rule")
    wh = g.curl_hat(full_state(g, 5))
    c = ctx(N, L, prec, formulation="VV")
    assert relerr(c.compute_rhs(wh.astype(c.complex)), g.compute_rhs_vv(wh)) < TOL[prec]


@pytest.mark.parametrize("prec", ["double", "single"])
def test_pad32_rk4_diagnostics_source(built_lib, prec):
    N, L = (32, 32, 32), (2 * np.pi,) * 3
    g = Grid(N, L, dealias="3/2-rule")
    uh = full_state(g, 6) * 0.05
    src = full_state(g, 7) * 0.01
    c = ctx(N, L, prec)
    c.set_state(uh.astype(c.complex))
    c.set_source(src.astype(c.complex))
    c.rk4(0.01, 3)
    ref = uh
    for _ in range(3):
        ref = g.rk4_step(ref, 0.01, source=src)
    assert relerr(c.get_state(), ref) < (1e-11 if prec == "double" else 2e-5)
    d = c.diagnostics()
    tol = 1e-11 if prec == "double" else 1e-5
    assert abs(d["energy"] - g.kinetic_energy(ref)) < tol * g.kinetic_energy(ref)
    assert abs(d["enstrophy"] - g.enstrophy(ref)) < tol * g.enstrophy(ref)
    assert abs(d["time"] - 0.03) < 1e-12
    ek, _ = g.spectrum(ref)
    assert relerr(c.spectrum(len(ek)), ek) < tol
    assert relerr(c.velocity(), g.backward(ref)) < (1e-11 if prec == "double" else 2e-5)


def test_pad32_rejects_cfl_and_forcing(built_lib):
    from spectraldns_gb300._lib import SdnsError
    c = ctx((16, 16, 16), (2 * np.pi,) * 3, "double")
    with pytest.raises(SdnsError):
        c.set_cfl(0.5)
    with pytest.raises(SdnsError):
        c.set_forcing(0.1, 2.0)


@pytest.mark.parametrize("solver_name", ["NS", "VV"])
@pytest.mark.parametrize("mesh", ["uniform", "nonuniform"])
def test_pad32_solver_api(built_lib, mesh, solver_name):
    """tests/test_NSVV.py::test_solvers with config.params.dealias = '3/2-rule': TG to T = 0.1,
    regression test of tests/TG.py:116-126 to 7 digits."""
    from spectraldns_gb300 import config, get_solver, solve
    from tests.test_api_gpu import regression_test
    args = ["--M", "4", "4", "4", "--L", "2*pi", "2*pi", "2*pi"] if mesh == "uniform" else \
        ["--M", "6", "5", "4", "--L", "6*pi", "4*pi", "2*pi"]
    config.update({"nu": 0.000625, "dt": 0.01, "T": 0.1, "convection": "Vortex"})
    solver = get_solver(regression_test=regression_test, update=lambda c: None,
                        parse_args=args + ["--dealias", "3/2-rule", solver_name])
    context = solver.get_context()
    U, X = context.U, context.X
    U[0] = np.sin(X[0]) * np.cos(X[1]) * np.cos(X[2])
    U[1] = -np.cos(X[0]) * np.sin(X[1]) * np.cos(X[2])
    U[2] = 0
    solver.set_velocity(**context)
    if solver_name == "VV":
        solver.cross2(context.W_hat, context.K, context.U_hat)
    config.params.t = 0.0
    config.params.tstep = 0
    solve(solver, context)
    assert abs(config.params.t - 0.1) < 1e-12


@pytest.mark.parametrize("method", ["BS5_adaptive", "AB2"])
def test_pad32_device_integrators(built_lib, method):
    """The host-driven integrators on a 3/2-rule context (every right-hand side padded)."""
    import torch
    from oracle.ns_ref import Integrator
    from spectraldns_gb300.integrators import DeviceIntegrator
    N, L = (16, 16, 32), (2 * np.pi,) * 3
    g = Grid(N, L, dealias="3/2-rule")
    uh0 = g.forward(taylor_green(g)) + 0.05 * full_state(g, 9)
    c = ctx(N, L, "double")
    it = DeviceIntegrator(c, method, tol=1e-6)
    it.u.copy_(torch.from_numpy(np.ascontiguousarray(uh0)))
    torch.cuda.synchronize()
    ref = Integrator(g, method, tol=1e-6)
    u, dt, dtg = uh0, 0.01, 0.01
    for ts in range(4):
        dtg, _ = it.step(dtg, ts)
        u, dt, _ = ref.step(u, dt, ts)
    assert abs(dtg - dt) <= 1e-9 * dt
    assert relerr(it.u.cpu().numpy(), u) < 1e-11


def test_pad32_vv_rk4(built_lib):
    N, L = (32, 16, 16), (4 * np.pi, 2 * np.pi, 2 * np.pi)
    g = Grid(N, L, nu=0.01, dealias="3/2-rule")
    wh = g.curl_hat(full_state(g, 10)) * 0.1
    c = ctx(N, L, "double", formulation="VV", nu=0.01)
    c.set_state(wh)
    c.rk4(0.01, 2)
    ref = wh
    for _ in range(2):
        ref = g.rk4_step(ref, 0.01, vv=True)
    assert relerr(c.get_state(), ref) < 1e-11
    d = c.diagnostics()
    assert abs(d["energy"] - g.kinetic_energy(g.velocity_of_vorticity(ref))) < 1e-11 * d["energy"]
