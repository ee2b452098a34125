"""Velocity-vorticity Navier-Stokes solver (Vortex form) on the GB300.

Module interface of spectralDNS/solvers/VV.py: the curl of the momentum
equation is advanced for W_hat = i K x U_hat, and the velocity needed by the
convective term is recovered as U_hat = i K x W_hat / K^2 (compute_velocity,
VV.py:52-67).  ComputeRHS (VV.py:112-146) is
``i K x F(u x w) - nu K^2 W_hat + Source`` with 2/3-rule dealiasing; it runs
inside libsdns_gb300.so (a context created with formulation SDNS_VV shares
every transform sweep with the NS solver and differs in the first sweep, which
forms the velocity from the vorticity, and in the pointwise update, which
takes the curl of the nonlinear term instead of projecting it).

Everything else (config, hooks, Space, getters of U, integrators, the time
loop) is the NS module's, as the reference's ``from .NS import *``.
"""
from __future__ import annotations

import numpy as np

from .NS import *  # noqa: F401,F403
from .NS import Field, _fresh, _push_source, get_context as NS_context, params  # noqa: F401
from ..h5io import HDF5File


def get_context():
    """Context of the VV solver (VV.py:23-38): NS's arrays without P, P_hat; W_hat is the state."""
    c = NS_context(formulation="VV")
    del c["P"], c["P_hat"]
    c.W_hat = Field(c.VT, True, c.complex)
    c.u = c.W_hat
    c.hdf5file = VVFile(params.solver, checkpoint={"space": c.VT, "data": {"0": {"curl": [c.W_hat]}}},
                        results={"space": c.VT, "data": {"U": [c.U], "curl": [c.curl]}})
    return c


class VVFile(HDF5File):
    """Checkpoint / results files of the VV solver (VV.py:40-50): W_hat as the checkpoint, U and curl as results."""

    def update_components(self, **context):
        get_velocity(**context)
        get_curl(**context)

    def refresh(self, **context):
        for fields in self.checkpoint.get("data", {}).values():
            for val in fields.values():
                _fresh(val[0], context.get("gpu"))


def compute_velocity(U, w_hat, work, VT, K_over_K2):
    """U = F^-1(i K x w_hat / K^2) (VV.py:52-67), on the GPU."""
    return VT.ctx.velocity_vv(w_hat, out=U)


def get_velocity(W_hat, U, work, VT, K_over_K2, **context):
    """Velocity of the vorticity W_hat (VV.py:69-72)."""
    return compute_velocity(U, _fresh(W_hat, VT.ctx), work, VT, K_over_K2)


def get_divergence(T, K, U_hat, W_hat, **context):
    """Divergence of the velocity (VV.py:74-78 evaluates div(i K x W_hat), which vanishes as well).

    With ``--gpu_sync step`` the host W_hat is the solution and is uploaded
    first; with ``lazy`` the GPU state is.
    """
    gpu = T.ctx
    if not getattr(gpu, "host_stale", False):
        gpu.set_state(W_hat)
    return gpu.divergence(None)


def get_curl(curl, W_hat, VT, **context):
    """The curl is the state itself: curl = F^-1(W_hat) (VV.py:80-83)."""
    return VT.backward(_fresh(W_hat, VT.ctx), curl)


def get_pressure(*args, **kwargs):
    raise NotImplementedError("the velocity-vorticity solver has no pressure (VV.py:27 deletes P and P_hat)")


def getConvection(convection):
    """The convection term (VV.py:85-103) is fused into ComputeRHS on the GPU (Vortex form only)."""
    if convection != "Vortex":
        raise NotImplementedError("the VV solver implements the Vortex convection form (VV.py:87-88)")

    def Conv(rhs, w_hat, work, Tp, VTp, K, K_over_K2, u_dealias):
        raise NotImplementedError("the GB300 backend evaluates the convection inside ComputeRHS")
    Conv.convection = convection
    return Conv


def add_linear(rhs, w_hat, nu, K2, Source):
    raise NotImplementedError("the GB300 backend evaluates diffusion and Source inside ComputeRHS")


def ComputeRHS(rhs, w_hat, solver, work=None, Tp=None, VT=None, VTp=None, K=None, K2=None, K_over_K2=None,
               Source=None, u_dealias=None, mask=None, **context):
    """Right-hand side of the velocity-vorticity equations (VV.py:112-146).
    ``w_hat``/``rhs`` are host arrays or CUDA tensors."""
    gpu = context["gpu"]
    _push_source(gpu, Source)
    return gpu.compute_rhs(w_hat, out=rhs)
