"""Full-size decaying turbulence at 1024^3 FP32 on one GPU (the 1024^3 case:
k0 = 6 spectrum, no forcing, nu = 4e-4, RK4).

At this size no CPU oracle run fits a test, so the test checks properties
that hold for the exact semi-discrete system, with the FP64 reductions of the
library: the dealiased u x w term conserves energy, so the energy changes only
by dissipation, dE/dt = -nu <w.w> (the `dissipation` diagnostic); the field
stays solenoidal; the energy decays monotonically.  The trapezoid rule over
four CFL steps and the FP32 state bound the budget error by 1e-2 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_decaying_1024(built_lib):
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field
    N = (1024, 1024, 1024)
    nu = 4e-4
    uh = isotropic_field(N, k0=6.0, energy=0.5, seed=0, dtype=np.complex64)
    c = Context(N, nu=nu, precision="single")
    assert c.memory_bytes() < 80e9
    c.set_cfl(0.5)
    c.set_state(uh)
    del uh
    d = c.diagnostics()
    assert abs(d["energy"] - 0.5) < 1e-6
    E, D, T = [d["energy"]], [d["dissipation"]], [0.0]
    for _ in range(4):
        c.rk4(0.0, 1)
        d = c.diagnostics()
        E.append(d["energy"])
        D.append(d["dissipation"])
        T.append(d["time"])
        assert d["divergence"] < 1e-12 * d["energy"]
    assert all(E[i + 1] < E[i] for i in range(4))
    lost = E[0] - E[-1]
    budget = sum(0.5 * (D[i] + D[i + 1]) * (T[i + 1] - T[i]) for i in range(4))
    assert abs(lost - budget) < 1e-2 * budget, (lost, budget)
    assert T[-1] > 0


def test_tg256_fp32_against_fp64(built_lib):
    """Taylor-Green at 256^3, nu = 0.000625, dt = 0.005 (the 256^3 TG case): the FP64 GPU run
    matches the float64 oracle over the first two steps (1e-11), and over 200 steps the FP32
    run's energy and dissipation, taken every step, stay within 1e-5 and 1e-4 relative of
    the FP64 run's."""
    import os
    from oracle.ns_ref import Grid, taylor_green
    from spectraldns_gb300.gpu import Context
    from tests.helpers import relerr
    N = (256, 256, 256)
    nu, dt = 0.000625, 0.005
    g = Grid(N, nu=nu, workers=os.cpu_count() or 1)
    uh0 = g.forward(taylor_green(g))
    c64 = Context(N, nu=nu, precision="double")
    c32 = Context(N, nu=nu, precision="single")
    c64.set_state(uh0)
    c32.set_state(uh0.astype(np.complex64))
    ref = uh0
    for _ in range(2):
        ref = g.rk4_step(ref, dt)
    del uh0
    c64.rk4(dt, 2)
    assert relerr(c64.get_state(), ref) < 1e-11
    assert abs(c64.diagnostics()["energy"] - g.kinetic_energy(ref)) < 1e-13
    del ref
    c32.rk4(dt, 2)
    worst_e = worst_d = 0.0
    for _ in range(200):
        d64, d32 = c64.diagnostics(), c32.diagnostics()
        worst_e = max(worst_e, abs(d32["energy"] - d64["energy"]) / d64["energy"])
        worst_d = max(worst_d, abs(d32["dissipation"] - d64["dissipation"]) / d64["dissipation"])
        c64.rk4(dt, 1)
        c32.rk4(dt, 1)
    assert worst_e < 1e-5, worst_e
    assert worst_d < 1e-4, worst_d
    assert abs(c64.diagnostics()["time"] - 202 * dt) < 1e-12
