"""sdns_compute_rhs_noalloc: the right-hand side without any device allocation.

Some callers cannot allocate device memory (work recorded into a CUDA graph,
frameworks whose allocator owns the GPU, real-time loops).  This entry point
uses one static scratch array instead of a context.  These tests call it
through the C ABI on device buffers and compare each of two consecutive
calls with the context-based sdns_compute_rhs, within the parity tolerances
of the other GPU tests (1e-11 relative in FP64, 2e-5 in FP32).  The file is
named to be collected last so that a run stopping at the first failure has
run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.ns_ref import Grid
from tests.helpers import random_state, relerr

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-11, "single": 2e-5}


def _cfg(N, L, nu, prec):
    from spectraldns_gb300 import _lib
    cfg = _lib.sdns_config()
    cfg.n[:] = N
    cfg.L[:] = L
    cfg.nu = nu
    cfg.precision = _lib.SDNS_SINGLE if prec == "single" else _lib.SDNS_DOUBLE
    cfg.dealias = _lib.SDNS_DEALIAS_23
    cfg.device = 0
    return cfg


def _noalloc(lib, cfg, u_dev, r_dev):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.sdns_compute_rhs_noalloc(C.byref(cfg), C.c_void_p(u_dev.data_ptr()), C.c_void_p(r_dev.data_ptr()),
                                      C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("prec", ["double", "single"])
@pytest.mark.parametrize("N,L", [((32, 32, 32), (2 * np.pi,) * 3), ((16, 32, 64), (2 * np.pi, 4 * np.pi, 2 * np.pi))])
def test_noalloc_matches_context_rhs(built_lib, N, L, prec):
    import torch
    from spectraldns_gb300.gpu import Context
    g = Grid(N, L, nu=0.01)
    ctx = Context(N, L, nu=0.01, precision=prec)
    cfg = _cfg(N, L, 0.01, prec)
    tdt = torch.complex128 if prec == "double" else torch.complex64
    for seed in (3, 4):  # two calls in a row, different inputs
        uh = random_state(g, seed=seed).astype(ctx.complex)
        ref = ctx.compute_rhs(uh)
        u_dev = torch.from_numpy(uh).to("cuda:0")
        r_dev = torch.full(ctx.spec_shape, float("nan"), dtype=tdt, device="cuda:0")
        assert _noalloc(built_lib, cfg, u_dev, r_dev) == 0, built_lib.sdns_last_error()
        out = r_dev.cpu().numpy()
        assert relerr(out, ref) < TOL[prec]
    ctx.close()


def test_noalloc_rejects_oversize_grid(built_lib):
    import torch
    from spectraldns_gb300 import _lib
    N = (256, 256, 256)
    cfg = _cfg(N, (2 * np.pi,) * 3, 0.01, "double")
    small = torch.zeros(4, dtype=torch.complex128, device="cuda:0")
    rc = _noalloc(built_lib, cfg, small, small)
    assert rc == _lib.SDNS_EINVAL
    assert b"scratch" in built_lib.sdns_last_error()
