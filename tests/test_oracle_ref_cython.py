"""The oracle's pointwise arithmetic and integrator updates against the
reference's own compiled Cython kernels (spectralDNS/optimization/
cython_{maths,solvers,integrators}.in, built into oracle/_ref by
oracle/build_ref_cython.py from the reference tree).  CPU only; skipped where
the reference tree or Cython is absent (the GPU machine).

Tolerances: float64 agreement to 1e-14 relative (association-order rounding
only), float32 to 1e-6.
"""
import importlib
import os
import sys

import numpy as np
import pytest

from oracle.ns_ref import Grid, Integrator, taylor_green
from tests.helpers import random_state, relerr

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref")


@pytest.fixture(scope="module")
def cy():
    sys.path.insert(0, os.path.dirname(HERE))
    from oracle import build_ref_cython as b
    if not b.build():
        pytest.skip("reference tree or Cython not available: oracle/_ref not built")
    sys.path.insert(0, REF)
    try:
        yield {(p, m): importlib.import_module("cython_%s_%s" % (p, m))
               for p in ("single", "double") for m in ("maths", "solvers", "integrators")}
    finally:
        sys.path.remove(REF)


@pytest.mark.parametrize("prec", ["double", "single"])
def test_cross_products(cy, prec):
    """cross1 (u x w, maths/cross.py:13-25) and cross2 (i K x u_hat, :27-32)."""
    g = Grid((16, 32, 16), dtype=np.float64 if prec == "double" else np.float32)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((3,) + g.N).astype(g.dtype)
    w = rng.standard_normal((3,) + g.N).astype(g.dtype)
    c = np.empty_like(u)
    c = cy[(prec, "maths")].cross1(c, u, w)
    tol = 1e-14 if prec == "double" else 1e-6
    assert relerr(c, g.cross(u, w)) < tol
    uh = random_state(Grid(g.N), seed=1).astype(g.cdtype)
    ch = np.empty_like(uh)
    ch = cy[(prec, "maths")].cross2(ch, g.K, uh)
    assert relerr(ch, g.curl_hat(uh)) < tol


@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3), ((32, 16, 16), (4 * np.pi, 2 * np.pi, 2 * np.pi))])
def test_pressure_projection_and_diffusion(cy, N, L):
    """add_pressure_diffusion_NS (cython_solvers.in; NS.py:203-217) on the oracle's nonlinear term
    gives the oracle's right-hand side and P_hat."""
    g = Grid(N, L, nu=0.01)
    uh = random_state(g, seed=2)
    rhs, parts = g.compute_rhs(uh, return_parts=True)
    du = parts["nl"].copy()
    p_hat = np.zeros(g.spec_shape, dtype=np.complex128)
    KoK2 = np.ascontiguousarray(np.stack(np.broadcast_arrays(*g.K_over_K2)))
    K2 = np.ascontiguousarray(np.broadcast_to(g.K2, g.spec_shape))
    du = cy[("double", "solvers")].add_pressure_diffusion_NS(du, uh, float(g.nu), K2, g.K, p_hat, KoK2)
    assert relerr(du, rhs) < 1e-14
    assert relerr(p_hat, parts["P_hat"]) < 1e-14


class _Solver:
    """The solver-module surface the Cython integrators call (ComputeRHS writes into dU)."""

    def __init__(self, g):
        self.g = g

    def ComputeRHS(self, dU, U_hat, solver, **context):
        dU[:] = self.g.compute_rhs(U_hat)
        return dU


def test_integrators(cy):
    """Cython RK4 / ForwardEuler / AB2 (cython_integrators.in; integrators.py:149-175) driven
    by the oracle's ComputeRHS agree with the oracle's own steps."""
    g = Grid((16, 16, 16))
    uh0 = g.forward(taylor_green(g)) + 0.05 * random_state(g, seed=3)
    mod = cy[("double", "integrators")]
    s = _Solver(g)
    dt = 0.01
    # RK4
    U, U0, U1, dU = uh0.copy(), np.empty_like(uh0), np.empty_like(uh0), np.empty_like(uh0)
    a = np.array([1 / 6, 1 / 3, 1 / 3, 1 / 6])
    b = np.array([0.5, 0.5, 1.0])
    ref = uh0
    for _ in range(3):
        U, _, _ = mod.RK4(U, U0, U1, dU, a, b, dt, s, {})
        ref = g.rk4_step(ref, dt)
    assert relerr(U, ref) < 1e-14
    # ForwardEuler and AB2
    for name in ("ForwardEuler", "AB2"):
        U, U0, dU = uh0.copy(), np.zeros_like(uh0), np.empty_like(uh0)
        it = Integrator(g, name)
        ref = uh0
        for ts in range(3):
            if name == "ForwardEuler":
                U, _, _ = mod.ForwardEuler(U, U0, dU, dt, s, {})
            else:
                mod.AB2(U, U0, dU, dt, ts, s, {})
            ref, _, _ = it.step(ref, dt, ts)
        assert relerr(U, ref) < 1e-14, name
