"""Time integrators of spectralDNS/maths/integrators.py other than RK4, on the GPU.

RK4 runs inside the library (``sdns_rk4``: one CUDA graph per step on the
compact state).  ForwardEuler (integrators.py:161-165), AB2 (:167-175) and the
embedded Runge-Kutta step of :15-147 with the Bogacki-Shampine 5(4) pair
(``BS5_fixed``/``BS5_adaptive``, :193-233) keep their stage vectors on the
GPU and are driven from here exactly as the reference drives its numpy
arrays: every right-hand side is ``sdns_compute_rhs``, every update is one
fused ``sdns_lincomb`` and the error estimate is ``sdns_error_norm``.  No
arithmetic on the solution runs on the host.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

# Bogacki-Shampine 5(4) pair (P. Bogacki, L. F. Shampine, Comput. Math. Appl.
# 32 (1996) 15-28), the tableau of spectralDNS/maths/integrators.py:197-209:
# 8 stages, the last stage is the solution (first-same-as-last), embedded order 4.
BS5_A = (
    (),
    ("1/6",),
    ("2/27", "4/27"),
    ("183/1372", "-162/343", "1053/1372"),
    ("68/297", "-4/11", "42/143", "1960/3861"),
    ("597/22528", "81/352", "63099/585728", "58653/366080", "4617/20480"),
    ("174197/959244", "-30942/79937", "8152137/19744439", "666106/1039181", "-29421/29068", "482048/414219"),
    ("587/8064", "0", "4440339/15491840", "24353/124800", "387/44800", "2152/5985", "7267/94080"),
)
BS5_BHAT = ("2479/34992", "0", "123/416", "612941/3411720", "43/1440", "2272/6561", "79937/1113912", "3293/556956")
BS5_ERR_ORDER = 4

METHODS = ("ForwardEuler", "AB2", "BS5_fixed", "BS5_adaptive")


def _rows(real):
    """A, b, bhat rounded to the working float type (integrators.py:197-211 casts to context.float)."""
    A = [[float(real(float(Fraction(q)))) for q in row] for row in BS5_A]
    b = [float(real(float(Fraction(q)))) for q in BS5_A[7]] + [0.0]
    bhat = [float(real(float(Fraction(q)))) for q in BS5_BHAT]
    return A, b, bhat


class DeviceIntegrator:
    """One of ``METHODS`` advancing a device copy of the spectral state.

    ``step(dt, tstep)`` returns ``(dt_next, dt_taken)`` like the reference's
    integrator closures.  ``u`` is the current solution (a torch CUDA tensor
    in the layout of U_hat); ``step`` returns after the context stream has
    finished it, so torch may read it at once.  ``callback(fu0)`` is called
    with the first stage's right-hand side of every embedded-RK attempt (the
    reference sets ``context.fu0`` and calls ``additional_callback``, :73-75).
    """

    def __init__(self, ctx, method, tol=1e-6, callback=None):
        if method not in METHODS:
            raise ValueError("unknown integrator %r (GPU integrators: RK4, %s)" % (method, ", ".join(METHODS)))
        self.ctx = ctx
        self.method = method
        self.tol = float(tol)
        self.callback = callback
        self.u = ctx.empty_vec()
        self.rhs = ctx.empty_vec()
        self.rejected = 0
        self.last_est = None
        if method == "AB2":
            self.u1 = ctx.empty_vec()
        if method.startswith("BS5"):
            self.A, self.b, self.bhat = _rows(ctx.real)
            self.fY = [ctx.empty_vec() for _ in range(8)]
            self.unew = ctx.empty_vec()
            self.err = ctx.empty_vec()
            self.offset = 0
            # the reference reuses the FSAL stage whenever tstep > 0, which after a
            # restart (tstep > 0, fresh arrays) would use a stage never computed;
            # here stage 0 is recomputed until one step has produced it
            self.have_fsal = False

    def F(self, y, out):
        """ComputeRHS (NS.py:219-261, Source included) of device vector y into out."""
        return self.ctx.compute_rhs(y, out=out)

    def step(self, dt, tstep):
        c = self.ctx
        if self.method == "ForwardEuler":  # integrators.py:161-165
            self.F(self.u, self.rhs)
            c.lincomb(self.u, self.u, [dt], [self.rhs])
            out = (dt, dt)
        elif self.method == "AB2":  # integrators.py:167-175
            self.F(self.u, self.rhs)
            if tstep == 0:
                c.lincomb(self.u, self.u, [dt], [self.rhs])
            else:
                c.lincomb(self.u, self.u, [1.5 * dt, -0.5], [self.rhs, self.u1])
            c.lincomb(self.u1, None, [dt], [self.rhs])
            out = (dt, dt)
        else:
            out = self._embedded(dt, tstep, adaptive=self.method == "BS5_adaptive")
        c.synchronize()
        return out

    def _embedded(self, dt, tstep, adaptive):
        """adaptiveRK (integrators.py:15-147) with fsal=True, errnorm "2", aTOL = rTOL = TOL."""
        c, A, b, bhat, fY = self.ctx, self.A, self.b, self.bhat, self.fY
        s = 8
        facmax, fac, facmin = 2.0, 0.8, 0.01
        exponent = 1.0 / (BS5_ERR_ORDER + 1)
        nspec = math.sqrt(float(np.prod(c.spec_shape[1:])))  # the scalar space's shape, T.shape(True) (:96)
        while True:
            dt_prev = dt
            self.offset = (self.offset - 1) % s
            o = self.offset
            for i in range(s):
                if tstep == 0 or i != 0 or not self.have_fsal:
                    y = fY[(i + o) % s]
                    c.lincomb(y, self.u, [dt * A[i][j] for j in range(i)], [fY[(j + o) % s] for j in range(i)])
                    self.F(y, y)
                if i == 0 and self.callback is not None:
                    self.callback(fY[o % s])
            c.lincomb(self.unew, self.u, [dt * b[j] for j in range(s)], [fY[(j + o) % s] for j in range(s)])
            c.lincomb(self.err, None, [dt * (b[j] - bhat[j]) for j in range(s)], [fY[(j + o) % s] for j in range(s)])
            nsq = c.error_norm(self.err, self.u, self.unew, self.tol, self.tol)
            est = float(np.max(np.sqrt(nsq))) / nspec
            factor = min(facmax, max(facmin, fac * (1.0 / est) ** exponent)) if est > 0 else facmax
            if adaptive:
                dt = dt * factor
                if est > 1.0:
                    facmax = 1.0
                    self.rejected += 1
                    self.offset += 1
                    continue
            break
        self.last_est = est
        self.have_fsal = True
        self.u, self.unew = self.unew, self.u
        return dt, dt_prev
