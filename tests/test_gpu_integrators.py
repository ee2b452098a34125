"""GPU parity of the ForwardEuler, AB2 and BS5 integrators (spectralDNS
maths/integrators.py:15-147, 161-175) against the oracle's restatement, and
the reference's own integrator test (tests/test_NSVV.py::test_integrators)
through the driver API.

Tolerances: FP64 states agree with the float64 oracle to 1e-11 relative
(rounding only); adaptive time steps to 1e-9 relative; FP32 states to 2e-5.
"""
import numpy as np
import pytest

from oracle.ns_ref import Grid, Integrator, taylor_green
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu

METHODS = ["ForwardEuler", "AB2", "BS5_fixed", "BS5_adaptive"]


def _torch_vec(ctx, a):
    import torch
    t = ctx.empty_vec()
    t.copy_(torch.from_numpy(np.ascontiguousarray(a.astype(ctx.complex))))
    torch.cuda.synchronize()
    return t


@pytest.mark.parametrize("prec", ["double", "single"])
def test_lincomb_and_error_norm(built_lib, prec):
    from spectraldns_gb300.gpu import Context
    N = (16, 32, 16)
    c = Context(N, precision=prec)
    rng = np.random.default_rng(5)
    shp = c.spec_shape
    vs = [rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(9)]
    tv = [_torch_vec(c, v) for v in vs]
    coefs = list(rng.standard_normal(8))
    out = c.empty_vec()
    c.lincomb(out, tv[0], coefs, tv[1:])
    ref = vs[0] + sum(cf * v for cf, v in zip(coefs, vs[1:]))
    tol = 1e-14 if prec == "double" else 2e-6
    assert relerr(out.cpu().numpy(), ref) < tol
    # no base, aliasing out with a term
    c.lincomb(tv[1], None, [2.0, -1.0], [tv[1], tv[2]])
    assert relerr(tv[1].cpu().numpy(), 2 * vs[1].astype(c.complex) - vs[2].astype(c.complex)) < tol
    # zero terms: out = base
    c.lincomb(out, tv[3], [], [])
    assert np.array_equal(out.cpu().numpy(), vs[3].astype(c.complex))
    # error norm (integrators.py:87-92)
    e, a, b = (v.astype(c.complex) for v in vs[4:7])
    sums = c.error_norm(tv[4], tv[5], tv[6], 1e-3, 1e-2)
    sc = 1e-3 + np.maximum(np.abs(a.astype(np.complex128)), np.abs(b.astype(np.complex128))) * 1e-2
    want = [np.sum(np.abs(e[k].astype(np.complex128) / sc[k]) ** 2) for k in range(3)]
    assert np.allclose(sums, want, rtol=1e-12)
    with pytest.raises(ValueError):
        c.lincomb(out, None, [1.0] * 9, [tv[0]] * 9)


def _march(step, uh_or_none, T=0.1, dt=0.01):
    """The solve() loop of spectralDNS/__init__.py:69-123 with end_of_tstep (NS.py:112-122)."""
    t, tstep, states, dts = 0.0, 0, [], []
    while t + dt <= T + 1e-12:
        dt_next, took = step(dt, tstep)
        t += took
        tstep += 1
        states.append(uh_or_none())
        dts.append(took)
        dt = dt_next
        if abs(t - T) < 1e-12:
            break
        if abs(t + dt - T) < 1e-12 or t + dt >= T + 1e-12:
            dt = T - t
    return states, dts


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("N,L", [((16, 16, 16), (2 * np.pi,) * 3),
                                 ((32, 16, 16), (4 * np.pi, 2 * np.pi, 2 * np.pi))])
def test_integrator_parity_fp64(built_lib, method, N, L):
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.integrators import DeviceIntegrator
    g = Grid(N, L)
    uh0 = g.forward(taylor_green(g)) + 0.05 * random_state(g, seed=11)
    c = Context(N, L, precision="double")
    it = DeviceIntegrator(c, method, tol=1e-6)
    it.u.copy_(_torch_vec(c, uh0))
    gpu_states, gpu_dts = _march(lambda dt, ts: it.step(dt, ts), lambda: it.u.cpu().numpy())
    ref = Integrator(g, method, tol=1e-6)
    box = {"u": uh0}

    def rstep(dt, ts):
        box["u"], dtn, took = ref.step(box["u"], dt, ts)
        return dtn, took
    ref_states, ref_dts = _march(rstep, lambda: box["u"])
    assert len(gpu_states) == len(ref_states)
    assert np.allclose(gpu_dts, ref_dts, rtol=1e-9, atol=0)
    for a, b in zip(gpu_states, ref_states):
        assert relerr(a, b) < 1e-11
    if method == "BS5_adaptive":
        assert len(gpu_states) < 10  # the controller grows the step from dt = 0.01


def test_integrator_fp32_forward_euler(built_lib):
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.integrators import DeviceIntegrator
    N = (32, 32, 32)
    g = Grid(N)
    uh0 = random_state(g, seed=2)
    c = Context(N, precision="single")
    it = DeviceIntegrator(c, "ForwardEuler")
    it.u.copy_(_torch_vec(c, uh0))
    ref = Integrator(g, "ForwardEuler")
    u = uh0
    for ts in range(3):
        it.step(0.005, ts)
        u, _, _ = ref.step(u, 0.005, ts)
    assert relerr(it.u.cpu().numpy(), u) < 2e-5


def test_bs5_rejection_matches_oracle(built_lib):
    """A tolerance tight enough to reject the first attempts: same rejections, same steps."""
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.integrators import DeviceIntegrator
    N = (16, 16, 16)
    g = Grid(N, nu=0.01)
    uh0 = random_state(g, seed=4) * 100  # max |u| ~ 2: the first attempt (dt = 0.2) is rejected
    c = Context(N, nu=0.01, precision="double")
    it = DeviceIntegrator(c, "BS5_adaptive", tol=1e-8)
    it.u.copy_(_torch_vec(c, uh0))
    ref = Integrator(g, "BS5_adaptive", tol=1e-8)
    u, dt, dtg = uh0, 0.2, 0.2
    for ts in range(3):
        dtg, _ = it.step(dtg, ts)
        u, dt, _ = ref.step(u, dt, ts)
    assert ref.rejected > 0 and it.rejected == ref.rejected
    assert abs(dtg - dt) <= 1e-9 * dt
    assert relerr(it.u.cpu().numpy(), u) < 1e-11


@pytest.mark.parametrize("integrator,ntol", [("RK4", 7), ("ForwardEuler", 4), ("AB2", 4), ("BS5_adaptive", 7),
                                             ("BS5_fixed", 7)])
@pytest.mark.parametrize("mesh", ["uniform", "nonuniform"])
def test_integrators_api(built_lib, integrator, ntol, mesh):
    """tests/test_NSVV.py::test_integrators: TG to T = 0.1 with each integrator,
    regression test of tests/TG.py:116-126 to ntol digits."""
    from spectraldns_gb300 import config, get_solver, solve
    from tests.test_api_gpu import initialize, regression_test
    args = ["--M", "4", "4", "4", "--L", "2*pi", "2*pi", "2*pi"] if mesh == "uniform" else \
        ["--M", "6", "5", "4", "--L", "6*pi", "4*pi", "2*pi"]
    config.update({"nu": 0.000625, "dt": 0.01, "T": 0.1, "convection": "Vortex"})
    solver = get_solver(regression_test=regression_test, parse_args=args + ["NS"])
    context = solver.get_context()
    config.params.ntol = ntol
    config.params.integrator = integrator
    initialize(solver, context)
    solve(solver, context)
    assert abs(config.params.t - 0.1) < 1e-12
