"""The spectralDNS driver API on the GPU, in the manner of the reference's
tests/test_NSVV.py::test_solvers: Taylor-Green to T=0.1 with the known
answers of tests/TG.py:125-126 as the regression test."""
import numpy as np
import pytest

from oracle.ns_ref import Grid

pytestmark = pytest.mark.gpu

K_TG, W_TG = 0.124953117517, 0.375249930801


def initialize(solver, context):
    """Taylor-Green initial velocity (demo/TG.py:23-28) set through set_velocity."""
    from spectraldns_gb300 import config
    U, X = context.U, context.X
    U[0] = np.sin(X[0]) * np.cos(X[1]) * np.cos(X[2])
    U[1] = -np.cos(X[0]) * np.sin(X[1]) * np.cos(X[2])
    U[2] = 0
    solver.set_velocity(**context)
    config.params.t = 0.0
    config.params.tstep = 0


def regression_test(context):
    """Float64 mean-square energy and enstrophy to params.ntol digits (demo/TG.py:116-126)."""
    from spectraldns_gb300 import config
    params, solver = config.params, config.solver
    U = solver.get_velocity(**context)
    curl = solver.get_curl(**context)
    w = solver.comm.reduce(np.sum(curl.astype(np.float64) ** 2) / np.prod(params.N) / 2)
    k = solver.comm.reduce(np.sum(U.astype(np.float64) ** 2) / np.prod(params.N) / 2)
    assert round(float(w) - W_TG, params.ntol) == 0, w
    assert round(float(k) - K_TG, params.ntol) == 0, k


def _run(args, **extra):
    from spectraldns_gb300 import config, get_solver, solve
    config.update({"nu": 0.000625, "dt": 0.01, "T": 0.1, "convection": "Vortex"})
    solver = get_solver(regression_test=regression_test, parse_args=args)
    for k, v in extra.items():
        setattr(config.params, k, v)
    context = solver.get_context()
    initialize(solver, context)
    solve(solver, context)
    return solver, context


@pytest.mark.parametrize("mesh", ["uniform", "nonuniform"])
def test_solvers_tg(mesh):
    args = ["--M", "4", "4", "4", "--L", "2*pi", "2*pi", "2*pi"] if mesh == "uniform" else \
        ["--M", "6", "5", "4", "--L", "6*pi", "4*pi", "2*pi"]
    solver, context = _run(args + ["NS"])
    # the state after solve() is on the host and matches the oracle
    from spectraldns_gb300 import config
    g = Grid(tuple(config.params.N), tuple(config.params.L))
    assert round(g.kinetic_energy(context.U_hat) - K_TG, 7) == 0
    div = solver.get_divergence(**context)
    assert np.max(np.abs(div)) < 1e-10
    P = solver.get_pressure(**context)
    assert P.shape == tuple(config.params.N) and np.all(np.isfinite(P))


def test_solvers_single_precision_lazy_sync():
    """FP32 run, state kept on the GPU between steps; 5 digits (FP32 rounding ~3e-7)."""
    solver, context = _run(["--M", "5", "5", "5", "--precision", "single", "--gpu_sync", "lazy", "--ntol", "5",
                            "NS"])
    solver.sync_to_host(context)
    assert context.U_hat.dtype == np.complex64
    g = Grid((32, 32, 32))
    assert abs(g.kinetic_energy(context.U_hat.astype(np.complex128)) - K_TG) < 1e-6


def test_compute_rhs_through_module_api():
    from spectraldns_gb300 import config, get_solver
    solver = get_solver(parse_args=["--M", "5", "5", "5", "NS"])
    context = solver.get_context()
    initialize(solver, context)
    g = Grid((32, 32, 32))
    ref = g.compute_rhs(context.U_hat)
    rhs = solver.ComputeRHS(context.dU, context.U_hat, solver, **context)
    assert rhs is context.dU
    assert np.max(np.abs(rhs - ref)) / np.max(np.abs(ref)) < 1e-11


def test_checkpoints_written(tmp_path, monkeypatch):
    """write_result/checkpoint every 2 steps as in tests/test_NSVV.py:64-71."""
    monkeypatch.chdir(tmp_path)
    solver, context = _run(["--M", "4", "4", "4", "--write_result", "2", "--checkpoint", "2", "NS"])
    d = np.load(str(tmp_path / "NS_c.npz"))
    assert int(d["tstep"]) == 10
    assert np.allclose(d["U/3D/0"], context.U_hat)
    w = np.load(str(tmp_path / "NS_w_2.npz"))
    assert w["U/3D/2"].shape == (3, 16, 16, 16) and w["P/3D/2"].shape == (16, 16, 16)


@pytest.mark.parametrize("precision,integrator", [("double", "RK4"), ("single", "RK4"), ("double", "BS5_fixed"),
                                                  ("double", "ForwardEuler")])
def test_restart_from_checkpoint(tmp_path, monkeypatch, precision, integrator):
    """A run restarted from the checkpoint of step 5 ends where the uninterrupted run does (bit for bit)."""
    import shutil
    from spectraldns_gb300 import config, get_solver, solve
    from spectraldns_gb300.h5io import init_from_file
    monkeypatch.chdir(tmp_path)
    args = ["--M", "5", "5", "5", "--precision", precision, "--integrator", integrator, "NS"]

    def keep_step5(context):
        # update() runs before the file hook: at step 6 NS_c.npz still holds step 5
        if config.params.tstep == 6:
            shutil.copy("NS_c.npz", "NS5_c.npz")

    def run(restart=False):
        config.update({"nu": 0.000625, "dt": 0.01, "T": 0.1, "convection": "Vortex"})
        solver = get_solver(regression_test=lambda c: None, update=keep_step5, parse_args=args)
        config.params.checkpoint = 5
        context = solver.get_context()
        initialize(solver, context)
        if restart:
            init_from_file("NS5", solver, context)
            assert config.params.tstep == 5
        solve(solver, context)
        # 10 steps; in single precision dt is float32 (as the reference's Params return it) and
        # the time loop may end with one more, tiny step to land on T
        return context.U_hat.copy(), config.params.tstep

    full, nfull = run()
    assert int(np.load("NS5_c.npz")["tstep"]) == 5
    restarted, nrest = run(restart=True)
    assert nrest == nfull and nfull in (10, 11)
    assert np.array_equal(restarted, full)


def test_cross_helper():
    """NS.Cross (NS.py:131-136): the forward transform of a x b, on the GPU transform."""
    from spectraldns_gb300 import get_solver
    solver = get_solver(parse_args=["--M", "4", "4", "4", "NS"])
    context = solver.get_context()
    g = Grid((16, 16, 16))
    rng = np.random.default_rng(3)
    a = rng.standard_normal((3, 16, 16, 16))
    b = rng.standard_normal((3, 16, 16, 16))
    c = np.zeros(context.U_hat.shape, dtype=context.U_hat.dtype)
    c = solver.Cross(c, a, b, context.work, context.VT)
    ref = g.forward(g.cross(a, b))
    assert np.max(np.abs(c - ref)) < 1e-12 * np.max(np.abs(ref))
