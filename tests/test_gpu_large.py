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
