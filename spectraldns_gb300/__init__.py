"""GB300 (sm_103a) backend of spectralDNS's triply periodic Navier-Stokes solver.

Driver API with the interface of spectralDNS/__init__.py:19-123:
``get_solver(update, regression_test, additional_callback, mesh, parse_args)``
returns the solver module selected by ``config.params.solver`` (``NS`` or ``VV``), and
``solve(solver, context)`` runs the time loop.  All compute runs in
``libsdns_gb300.so`` (see spectraldns_gb300.gpu).
"""
import importlib

from . import config

__version__ = "0.1.0"

_SOLVERS = {"NS": "spectraldns_gb300.solvers.NS", "VV": "spectraldns_gb300.solvers.VV"}


def get_solver(update=None, regression_test=None, additional_callback=None, mesh="triplyperiodic",
               parse_args=None):
    """Parse flags into config.params and return the solver module."""
    assert parse_args is None or isinstance(parse_args, list)
    if mesh != "triplyperiodic":
        raise ValueError("the GB300 backend provides the triply periodic NS solver only (mesh %r)" % mesh)
    args = getattr(config, mesh).parse_args(parse_args)
    config.params.update(vars(args))
    name = config.params.get("solver")
    if name not in _SOLVERS:
        raise AttributeError("Wrong solver! the GB300 backend provides %s, got %r" % (list(_SOLVERS), name))
    solver = importlib.import_module(_SOLVERS[name])
    if update:
        solver.update = update
    if regression_test:
        solver.regression_test = regression_test
    if additional_callback:
        solver.additional_callback = additional_callback
    config.solver = solver
    return solver


def solve(solver, context):
    """Time loop of spectralDNS/__init__.py:69-123 over the GPU integrator."""
    solver.timer = solver.Timer()
    params = solver.params
    solver.conv = solver.getConvection(params.convection)
    integrate = solver.getintegrator(context.dU, context.u, solver, context)
    dt_in = params.dt
    while params.t + params.dt <= params.T + 1e-12:
        u, params.dt, dt_took = integrate()
        params.t += dt_took
        params.tstep += 1
        solver.update(context)
        context.hdf5file.update(params, **context)
        solver.timer()
        if not solver.profiler.getstats() and params.make_profile:
            solver.profiler.enable()
        if solver.end_of_tstep(context):
            break
    params.dt = dt_in
    solver.timer.final(params.verbose)
    if params.make_profile:
        solver.results = solver.create_profile(solver.profiler)
    solver.regression_test(context)
    context.hdf5file.close()
