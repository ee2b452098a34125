"""Triply periodic Navier-Stokes solver (Vortex form) on the GB300.

Module interface of spectralDNS/solvers/NS.py: get_context (:12-72),
ComputeRHS (:219-261), getConvection (:164-201), the getters (:86-110),
end_of_tstep (:112-122), plus the hooks and globals the reference pulls in
from spectralinit.py (:19-62) and getintegrator (maths/integrators.py:177-191).

The context holds numpy arrays on the host exactly as the reference does
(U, U_hat, X, K, K2, K_over_K2, P, P_hat, curl, dU, Source ...); the
velocity state of the time loop lives on the GPU (``context.gpu``, a
spectraldns_gb300.gpu.Context) and every transform, right-hand side and RK4
step is computed by libsdns_gb300.so.  With ``--gpu_sync step`` (default)
U_hat is uploaded before and downloaded after every step, so hooks may read
and modify it like the reference's; ``--gpu_sync lazy`` keeps the state on
the GPU (hooks then use the getters, sync_to_host and sync_to_device).
"""
from __future__ import annotations

import cProfile
import os
import sys

import numpy as np

from .. import config
from ..config import AttributeDict
from ..gpu import Context
from ..h5io import HDF5File, init_from_file  # noqa: F401
from ..utilities import MemoryUsage, Timer, create_profile, reset_profile  # noqa: F401


class _Comm:
    """Single-rank stand-in for mpi4py's COMM_WORLD (one GPU, one process)."""

    def Get_size(self):
        return 1

    def Get_rank(self):
        return 0

    def reduce(self, x, op=None, root=0):
        return x

    def allreduce(self, x, op=None):
        return x

    def bcast(self, x, root=0):
        return x

    def barrier(self):
        return None


comm = _Comm()
num_processes = 1
rank = 0
params = config.params
profiler = cProfile.Profile()


def datatypes(precision):
    """Float and complex types of a precision (spectralinit.py:25-29)."""
    assert precision in ("single", "double")
    return {"single": (np.float32, np.complex64, None), "double": (np.float64, np.complex128, None)}[precision]


# ---------------------------------------------------------------- default hooks
def regression_test(context):
    pass


def update(context):
    pass


def additional_callback(context):
    pass


def solve_linear(context):
    pass


def conv(*args):
    raise NotImplementedError


_default_regression_test, _default_update, _default_additional_callback = regression_test, update, additional_callback


def set_source(Source, **context):
    Source[:] = 0
    return Source


def end_of_tstep(context):
    """Make the last step hit T exactly (NS.py:112-122)."""
    if abs(params.t - params.T) < 1e-12:
        return True
    if abs(params.t + params.dt - params.T) < 1e-12 or params.t + params.dt >= params.T + 1e-12:
        params.dt = params.T - params.t
    return False


# ---------------------------------------------------------------- spaces
class Space:
    """The transform object of a scalar (rank 1) or vector (rank 3) field.

    Provides the subset of shenfun's TensorProductSpace / VectorSpace the
    solver and the demos call; the transforms run on the GPU.
    """

    def __init__(self, ctx: Context, rank: int):
        self.ctx = ctx
        self.rank = rank
        self.N = ctx.N
        self.dtype = ctx.real

    def shape(self, spectral=False):
        n0, n1, n2 = self.N
        s = (n0, n1, n2 // 2 + 1) if spectral else (n0, n1, n2)
        return (3,) + s if self.rank == 3 else s

    def local_slice(self, spectral=False):
        return tuple(slice(0, n) for n in self.shape(spectral)[-3:])

    def forward(self, u, u_hat=None):
        return self.ctx.forward(u, out=u_hat)

    def backward(self, u_hat, u=None):
        return self.ctx.backward(u_hat, out=u)

    def get_mask_nyquist(self):
        n0, n1, n2 = self.N
        m0 = np.ones(n0, bool)
        m1 = np.ones(n1, bool)
        m2 = np.ones(n2 // 2 + 1, bool)
        m0[n0 // 2] = False
        m1[n1 // 2] = False
        m2[-1] = False
        return m0[:, None, None] & m1[None, :, None] & m2[None, None, :]

    def mask_nyquist(self, u_hat, mask=None):
        if mask is None:
            mask = self.get_mask_nyquist()
        u_hat *= mask
        return u_hat


class NSFile(HDF5File):
    """Checkpoint / results files of the NS solver (h5io/HDF5File.py; the
    reference's NS.py:66-70 stores U_hat as the checkpoint and U, P as results).

    With ``--gpu_sync lazy`` the checkpoint first pulls the state from the GPU.
    """

    def refresh(self, **context):
        for fields in self.checkpoint.get("data", {}).values():
            for val in fields.values():
                _fresh(val[0], context.get("gpu"))


class Field(np.ndarray):
    """A host array of the context that can transform itself, the part of shenfun's
    Array / Function the demos use (demo/TG.py:100 calls ``U.forward(U_hat)``): a physical
    field's ``forward`` and a spectral field's ``backward`` run on the GPU through its space."""

    def __new__(cls, space, spectral, dtype):
        obj = np.zeros(space.shape(spectral), dtype=dtype).view(cls)
        obj.space = space
        return obj

    def __array_finalize__(self, obj):
        self.space = getattr(obj, "space", None)

    def forward(self, output_array=None):
        return self.space.forward(np.asarray(self), output_array)

    def backward(self, output_array=None):
        return self.space.backward(np.asarray(self), output_array)


class _Work(dict):
    """Cached work arrays keyed like shenfun's CachedArrayDict: (array, index, zero)."""

    def __getitem__(self, key):
        a, i, fill = key[0], key[1], (key[2] if len(key) > 2 else True)
        k = (getattr(a, "shape", a), np.dtype(getattr(a, "dtype", np.float64)).str, i)
        if k not in self:
            dict.__setitem__(self, k, np.zeros(a.shape, dtype=a.dtype))
        arr = dict.__getitem__(self, k)
        if fill:
            arr.fill(0)
        return arr


# ---------------------------------------------------------------- context
def get_context(formulation="NS"):
    """Set up the GPU solver and the host arrays of NS.py:12-72.

    ``formulation="VV"`` makes the GPU context hold the vorticity (the
    velocity-vorticity solver, spectraldns_gb300.solvers.VV, builds on this).
    """
    float_, complex_, mpitype = datatypes(params.precision)
    if params.dealias == "None" and not params.mask_nyquist:
        raise ValueError("the GB300 backend masks the Nyquist modes when dealias is 'None'")
    if params.convection != "Vortex":
        raise ValueError("the GB300 backend implements the Vortex convection form")
    N = tuple(int(n) for n in params.N)
    L = tuple(float(x) for x in params.L)
    gpu = Context(N, L, nu=float(params.nu), precision=params.precision, dealias=params.dealias,
                  device=int(params.get("device", 0)), store_pressure=formulation == "NS",
                  formulation=formulation)
    T = Space(gpu, 1)
    VT = Space(gpu, 3)
    Tp, VTp = T, VT
    mask = T.get_mask_nyquist() if params.mask_nyquist else None
    x = [(np.arange(N[i]) * (L[i] / N[i])).astype(float_) for i in range(3)]
    X = [np.broadcast_to(x[0][:, None, None], N), np.broadcast_to(x[1][None, :, None], N),
         np.broadcast_to(x[2][None, None, :], N)]
    ki = [np.fft.fftfreq(N[0], 1.0 / N[0]), np.fft.fftfreq(N[1], 1.0 / N[1]), np.arange(N[2] // 2 + 1, dtype=float)]
    K = [(ki[0] * 2 * np.pi / L[0]).astype(float_)[:, None, None],
         (ki[1] * 2 * np.pi / L[1]).astype(float_)[None, :, None],
         (ki[2] * 2 * np.pi / L[2]).astype(float_)[None, None, :]]
    K2 = np.zeros(T.shape(True), dtype=float_)
    for i in range(3):
        K2 += K[i] * K[i]
    K_over_K2 = np.zeros(VT.shape(True), dtype=float_)
    K2n = np.where(K2 == 0, 1, K2)
    for i in range(3):
        K_over_K2[i] = K[i] / K2n
    del K2n, x, ki
    U = Field(VT, False, float_)
    U_hat = Field(VT, True, complex_)
    P = Field(T, False, float_)
    P_hat = Field(T, True, complex_)
    u_dealias = U
    u = U_hat
    dU = np.zeros(VT.shape(True), dtype=complex_)
    curl = Field(VT, False, float_)
    Source = np.zeros(VT.shape(True), dtype=complex_)
    work = _Work()
    hdf5file = NSFile(params.solver, checkpoint={"space": VT, "data": {"0": {"U": [U_hat]}}},
                      results={"space": VT, "data": {"U": [U], "P": [P]}})
    hdf5file.update_components = lambda **c: (get_velocity(**c), get_pressure(**c))
    return AttributeDict(
        float=float_, complex=complex_, mpitype=mpitype, N=N, L=L, gpu=gpu, T=T, VT=VT, Tp=Tp, VTp=VTp,
        mask=mask, X=X, K=K, K2=K2, K_over_K2=K_over_K2, U=U, U_hat=U_hat, P=P, P_hat=P_hat,
        u_dealias=u_dealias, u=u, dU=dU, curl=curl, Source=Source, work=work, hdf5file=hdf5file)


# ---------------------------------------------------------------- getters
def _fresh(U_hat, gpu):
    """With --gpu_sync lazy the host U_hat lags the GPU state: refresh it first."""
    if gpu is not None and getattr(gpu, "host_stale", False) and U_hat is getattr(gpu, "host_U_hat", None):
        gpu.get_state(out=U_hat)
        gpu.host_stale = False
    return U_hat


def get_curl(curl, U_hat, work, VT, K, **context):
    """curl = F^-1(i K x U_hat) (NS.py:86-89, 124-129)."""
    return compute_curl(curl, _fresh(U_hat, VT.ctx), work, VT, K)


def compute_curl(c, a, work, T, K):
    return T.ctx.curl(a, out=c)


def get_velocity(U, U_hat, VT, **context):
    """U = F^-1(U_hat) (NS.py:91-94)."""
    return VT.backward(_fresh(U_hat, VT.ctx), U)


def get_pressure(P, P_hat, T, **context):
    """Pressure of the last right-hand-side evaluation (NS.py:96-99)."""
    return T.ctx.pressure(out=P)


def set_velocity(U, U_hat, VT, **context):
    """U_hat = F(U) (NS.py:101-104)."""
    return VT.forward(U, U_hat)


def get_divergence(T, K, U_hat, mask, **context):
    """div u = F^-1(i K . U_hat) (NS.py:106-110)."""
    return T.ctx.divergence(_fresh(U_hat, T.ctx))


def sync_to_host(context):
    """Copy the GPU state into context.U_hat (for --gpu_sync lazy)."""
    context.gpu.get_state(out=context.U_hat)
    context.gpu.host_stale = False
    return context.U_hat


def sync_to_device(context):
    """Upload context.U_hat as the GPU state (after a hook changed it, --gpu_sync lazy)."""
    context.gpu.set_state(context.U_hat)


# ---------------------------------------------------------------- right-hand side
def cross1(c, a, b):
    """c = a x b for real fields (maths/cross.py:13-25); host utility for hook code."""
    c[0] = a[1] * b[2] - a[2] * b[1]
    c[1] = a[2] * b[0] - a[0] * b[2]
    c[2] = a[0] * b[1] - a[1] * b[0]
    return c


def cross2(c, a, b):
    """c = i (a x b) (maths/cross.py:27-32); host utility for hook code."""
    c = cross1(c, a, b)
    c *= 1j
    return c


def Cross(c, a, b, work, T):
    """c = F(a x b) for physical vectors a, b (NS.py:131-136); the transform runs on the GPU."""
    ab = work[(a, 0, False)] if isinstance(work, _Work) else np.empty_like(a)
    ab = cross1(ab, a, b)
    return T.forward(ab, c)


def standard_convection(rhs, u_dealias, U_hat, work, Tp, K):
    """The 'Standard' convection form (NS.py:138-145) is not provided by the GB300 backend."""
    raise NotImplementedError("the GB300 backend implements the Vortex convection form")


def divergence_convection(rhs, u_dealias, work, Tp, K, add=False):
    """The 'Divergence' convection form (NS.py:147-162) is not provided by the GB300 backend."""
    raise NotImplementedError("the GB300 backend implements the Vortex convection form")


def getConvection(convection):
    """The convection term is fused into ComputeRHS on the GPU (Vortex form only)."""
    if convection != "Vortex":
        raise ValueError("the GB300 backend implements the Vortex convection form")

    def Conv(rhs, u_hat, work, Tp, VTp, K, u_dealias):
        raise NotImplementedError("the GB300 backend evaluates the convection inside ComputeRHS")
    Conv.convection = convection
    return Conv


def add_pressure_diffusion(rhs, u_hat, nu, K2, K, P_hat, K_over_K2):
    raise NotImplementedError("the GB300 backend evaluates pressure and diffusion inside ComputeRHS")


def _push_source(gpu, Source):
    if Source is not None and np.any(Source):
        gpu.set_source(Source)
    else:
        gpu.set_source(None)


def ComputeRHS(rhs, u_hat, solver, work=None, Tp=None, VTp=None, P_hat=None, K=None, K2=None, u_dealias=None,
               K_over_K2=None, Source=None, mask=None, **context):
    """Right-hand side of NS in Vortex form, dealiased, projected, with diffusion and Source
    (NS.py:219-261).  ``u_hat``/``rhs`` are host arrays or CUDA tensors."""
    gpu = context["gpu"]
    _push_source(gpu, Source)
    return gpu.compute_rhs(u_hat, out=rhs)


# ---------------------------------------------------------------- integrator
def getintegrator(rhs, u0, solver, context):
    """The integrator closure of maths/integrators.py:177-239 on the GPU.

    RK4 (:149-159) runs as ``sdns_rk4`` on the library's compact state (one
    CUDA graph per step).  ForwardEuler, AB2, BS5_fixed and BS5_adaptive run
    as spectraldns_gb300.integrators.DeviceIntegrator, whose stage vectors
    stay on the GPU; after every step the library state is set to the new
    solution, so the getters and diagnostics see it.
    """
    gpu = context.gpu
    _push_source(gpu, context.get("Source"))
    lazy = params.get("gpu_sync", "step") == "lazy"
    state = {"uploaded": False}
    if params.integrator == "RK4":
        def func():
            if not lazy or not state["uploaded"]:
                gpu.set_state(u0)
                state["uploaded"] = True
            gpu.rk4(float(params.dt), 1)
            if not lazy:
                gpu.get_state(out=u0)
            else:
                gpu.host_U_hat = u0
                gpu.host_stale = True
            return u0, params.dt, params.dt
        func.__name__ = "RK4"
        return func

    import torch
    from ..integrators import DeviceIntegrator

    def callback(fu0):
        context.fu0 = fu0
        solver.additional_callback(context)

    integ = DeviceIntegrator(gpu, params.integrator, tol=params.get("TOL", 1e-6), callback=callback)
    context.integrator = integ

    def func():
        if not lazy or not state["uploaded"]:
            integ.u.copy_(torch.from_numpy(np.ascontiguousarray(u0)))
            torch.cuda.current_stream(integ.u.device).synchronize()
            state["uploaded"] = True
        dt, dt_took = integ.step(float(params.dt), int(params.tstep))
        gpu.set_state(integ.u)
        if not lazy:
            gpu.get_state(out=u0)
        else:
            gpu.host_U_hat = u0
            gpu.host_stale = True
        return u0, dt, dt_took
    func.__name__ = params.integrator
    return func
