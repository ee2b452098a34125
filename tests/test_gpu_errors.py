"""Error statuses of the C ABI on the GPU: calls out of order, bad arguments and a
solution that is not finite are reported as status codes (nothing traps), and the
context stays usable afterwards."""
import ctypes as C

import numpy as np
import pytest

from oracle.ns_ref import Grid
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu


def test_status_codes_and_recovery(built_lib):
    from spectraldns_gb300 import _lib
    from spectraldns_gb300._lib import SdnsError
    from spectraldns_gb300.gpu import Context
    L = _lib.lib()
    N = (16, 16, 16)
    c = Context(N, precision="double")
    # out of order: no state yet
    assert L.sdns_rk4(c._h, C.c_double(0.01), 1) == _lib.SDNS_ESTATE
    out = (C.c_double * _lib.SDNS_DIAG_COUNT)()
    assert L.sdns_diagnostics(c._h, out) == _lib.SDNS_ESTATE
    assert b"no state" in L.sdns_last_error()
    # pressure was not requested at creation
    with pytest.raises(SdnsError) as e:
        c.pressure()
    assert e.value.code == _lib.SDNS_ESTATE
    g = Grid(N)
    uh = random_state(g, seed=5)
    c.set_state(uh)
    # bad arguments
    assert L.sdns_rk4(c._h, C.c_double(0.0), 1) == _lib.SDNS_EINVAL      # no CFL: dt must be > 0
    assert L.sdns_rk4(c._h, C.c_double(0.01), -1) == _lib.SDNS_EINVAL
    coef = (C.c_double * 9)(*([1.0] * 9))
    ptrs = (C.c_void_p * 9)()
    assert L.sdns_lincomb(c._h, C.c_void_p(1), None, 9, coef, ptrs) == _lib.SDNS_EINVAL
    assert L.sdns_set_state(c._h, None, _lib.SDNS_HOST) == _lib.SDNS_EINVAL
    # a non-finite solution is detected by the step's energy reduction
    bad = uh.copy()
    bad[0, 1, 1, 1] = np.nan
    c.set_state(bad)
    c.rk4(0.01, 1)
    with pytest.raises(SdnsError) as e:
        c.diagnostics()
    assert e.value.code == _lib.SDNS_ENONFINITE
    # the context is still usable: a finite state steps and matches the oracle
    c.set_state(uh)
    c.set_time(0.0)
    c.rk4(0.01, 2)
    ref = g.rk4_step(g.rk4_step(uh, 0.01), 0.01)
    assert relerr(c.get_state(), ref) < 1e-11
    d = c.diagnostics()
    assert np.isfinite(d["energy"]) and abs(d["time"] - 0.02) < 1e-15
    c.close()
