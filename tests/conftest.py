import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libsdns_gb300.so")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load the CUDA library; GPU tests fail loudly without it."""
    from spectraldns_gb300 import build, _lib
    build.build()
    return _lib.lib()


@pytest.fixture(autouse=True)
def _fresh_solver_hooks():
    """get_solver() installs hooks on the solver modules, which outlive a test (as in the
    reference); give every test the modules' default hooks."""
    yield
    import importlib
    for name in ("spectraldns_gb300.solvers.NS", "spectraldns_gb300.solvers.VV"):
        mod = sys.modules.get(name)
        if mod is None:
            continue
        for hook in ("update", "regression_test", "additional_callback"):
            default = getattr(sys.modules["spectraldns_gb300.solvers.NS"], "_default_" + hook, None)
            if default is not None:
                setattr(mod, hook, default)
