"""CPU oracle for the triply-periodic pseudo-spectral Navier-Stokes RK4 step.

TEST INFRASTRUCTURE ONLY.  This module is the float64 (or float32) NumPy /
scipy.fft restatement of the spectralDNS NS "Vortex" path that the GPU
library is checked against.  Only the test-suite, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it; the product path
(``spectraldns_gb300``) never does.

What it restates (paths relative to the spectralDNS source tree):

* ``spectralDNS/solvers/NS.py:12-72``   get_context: wavenumbers ``K`` scaled by
  ``2*pi/L`` (:38-41), ``K2`` (:42-44), ``K_over_K2`` with ``K2==0 -> 1``
  (:46-48).
* ``spectralDNS/solvers/NS.py:124-136, 191-198``  Vortex convection:
  ``u = F^-1(u_hat)``, ``curl = F^-1(i K x u_hat)``, ``rhs = F(u x curl)``.
* ``spectralDNS/solvers/NS.py:203-217``  add_pressure_diffusion:
  ``P_hat = sum(rhs*K_over_K2)``; ``rhs -= P_hat*K``; ``rhs -= nu*K2*u_hat``.
* ``spectralDNS/solvers/NS.py:219-261``  ComputeRHS (``rhs += Source``, :259).
* ``spectralDNS/maths/integrators.py:149-159, 185-186``  classic RK4 with
  ``a=[1/6,1/3,1/3,1/6]``, ``b=[1/2,1/2,1]``.
* ``spectralDNS/solvers/VV.py:52-67, 85-146`` the velocity-vorticity form:
  ``u = F^-1(i K/K2 x w_hat)``, ``w = F^-1(w_hat)``,
  ``rhs = i K x F(u x w) - nu K2 w_hat + Source`` (``compute_rhs_vv``).
* ``spectralDNS/maths/integrators.py:15-147, 161-175, 193-233`` ForwardEuler,
  AB2 and the embedded Runge-Kutta step (FSAL, error norm "2", step-size
  controller) with the Bogacki-Shampine 5(4) tableau (``Integrator``).
* ``spectralDNS3D_short.py:36-46, 76-86`` and ``cpp/spectralDNS.cpp:122-129,
  217-236``  the explicit 2/3 rule: keep modes with ``|k_i| < (2/3)(N_i/2+1)``
  on every axis (integer wave index), applied to the nonlinear term on
  output; NS.py (``dealias_direct``) also truncates the transform input,
  which this oracle does as well (a no-op when the state is inside the set).
* Transform conventions of shenfun (third party, not vendored): forward
  R2C over the last axis, C2C over the others, normalised by 1/(N0 N1 N2);
  backward unnormalised.  In-tree evidence: ``demo/TG.py:98-109`` (Parseval
  check ``energy_fourier(U_hat)/2 - 1/2<U^2> ~ 0``) and
  ``demo/Isotropic.py:67-69``.
* ``spectralDNS/solvers/NS.py:29-31`` with ``padding_factor=1.5`` (the 3/2
  rule): every mode but the Nyquist ones is transformed on a grid of 3N/2
  points per axis (zero padded, unnormalised backward, forward scaled by
  1/prod(3N/2)), the nonlinear term is truncated back to the N modes and
  its Nyquist modes masked (``Grid(dealias="3/2-rule")``).  shenfun's own
  padding (its Nyquist split) is third party and absent: that detail is
  parity unpinned; the Nyquist modes are left out on input.
* Diagnostics: ``demo/TG.py:97-103, 116-126`` (float64 mean-square
  reductions), ``demo/Isotropic.py:88-147`` (shell spectrum).

Build-defined parts (not in the reference, mirrored by the GPU library):
the seeded ``k^4 exp(-2 (k/k0)^2)`` solenoidal initial field, the
constant-power low-wavenumber forcing (a ``Source`` recomputed at the start
of every RK4 step) and the CFL time step.

Parity pins: the Taylor-Green known answers ``k=0.124953117517`` and
``w=0.375249930801`` (``tests/TG.py:125-126``, ``spectralDNS3D_short.py:113``);
state fixtures produced by running ``spectralDNS3D_short.py`` itself
(``tests/golden/make_golden.py``); and the reference's own compiled Cython
kernels ``cross1``, ``cross2``, ``add_pressure_diffusion_NS``, ``RK4``,
``ForwardEuler`` and ``AB2`` (``oracle/build_ref_cython.py``,
``tests/test_oracle_ref_cython.py``).
"""
from __future__ import annotations

import math
import numpy as np

try:  # scipy.fft is threaded (workers=); numpy.fft is the fallback
    import scipy.fft as _fft
    _HAVE_SCIPY = True
except ImportError:  # pragma: no cover
    import numpy.fft as _fft
    _HAVE_SCIPY = False

RK4_A = (1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0)
RK4_B = (0.5, 0.5, 1.0)


def dealias_cutoff(n: int, rule: str = "2/3-rule") -> int:
    """Largest kept integer wave index |k| on an axis of n points.

    2/3 rule: keep |k| < (2/3)(n/2+1)  (spectralDNS3D_short.py:44-46).
    'None' (Nyquist masked): keep |k| <= n/2-1.
    """
    if rule == "2/3-rule":
        kmax = 2.0 / 3.0 * (n // 2 + 1)
        kc = int(math.ceil(kmax)) - 1
        while kc + 1 < kmax:
            kc += 1
        while kc >= kmax:
            kc -= 1
        return kc
    if rule in ("None", None, "3/2-rule"):
        return n // 2 - 1
    raise ValueError("unsupported dealias rule %r" % (rule,))


class Grid:
    """Spectral/physical grid of the triply periodic box (NS.py:12-48)."""

    def __init__(self, N, L=(2 * np.pi,) * 3, nu=0.000625, dealias="2/3-rule",
                 dtype=np.float64, workers=1):
        self.N = tuple(int(n) for n in N)
        self.L = tuple(float(l) for l in L)
        self.nu = float(nu)
        self.dealias = dealias
        self.dtype = np.dtype(dtype)
        self.cdtype = np.result_type(self.dtype, np.complex64)
        self.workers = workers
        n0, n1, n2 = self.N
        self.spec_shape = (n0, n1, n2 // 2 + 1)
        # integer wave indices in FFT order; R2C axis 0..n2/2
        self.ki = [np.fft.fftfreq(n0, 1.0 / n0).astype(np.int64),
                   np.fft.fftfreq(n1, 1.0 / n1).astype(np.int64),
                   np.arange(n2 // 2 + 1, dtype=np.int64)]
        # Nyquist index of the complex axes is -n/2 (fftfreq); the R2C
        # Nyquist +n2/2 is outside every kept set.
        scale = [2 * np.pi / l for l in self.L]
        # K cast to the working float type as NS.py:39-41 does
        k1d = [(self.ki[i].astype(np.float64) * scale[i]).astype(self.dtype) for i in range(3)]
        self.K = [k1d[0][:, None, None], k1d[1][None, :, None], k1d[2][None, None, :]]
        self.K2 = self.K[0] ** 2 + self.K[1] ** 2 + self.K[2] ** 2
        K2n = np.where(self.K2 == 0, self.dtype.type(1), self.K2)
        self.K_over_K2 = [self.K[i] / K2n for i in range(3)]
        self.nu = self.dtype.type(self.nu)
        self.kc = [dealias_cutoff(n, dealias) for n in self.N]
        m0 = np.abs(self.ki[0]) <= self.kc[0]
        m1 = np.abs(self.ki[1]) <= self.kc[1]
        m2 = np.abs(self.ki[2]) <= self.kc[2]
        self.mask = (m0[:, None, None] & m1[None, :, None] & m2[None, None, :])
        self.pad = dealias == "3/2-rule"
        self.M = tuple(3 * n // 2 for n in self.N)
        # the physical mesh (NS.py:37 via shenfun local_mesh)
        self.X = [(np.arange(self.N[i]) * self.L[i] / self.N[i]) for i in range(3)]

    # --- transforms (shenfun conventions) --------------------------------
    def forward(self, u):
        """R2C over the last axis, C2C over the others, scaled by 1/prod(N)."""
        kw = {"workers": self.workers} if _HAVE_SCIPY else {}
        out = _fft.rfftn(u, axes=(-3, -2, -1), **kw) / float(np.prod(self.N))
        return out.astype(self.cdtype, copy=False)

    def backward(self, uh):
        """Unnormalised inverse (C2C, C2C, C2R)."""
        kw = {"workers": self.workers} if _HAVE_SCIPY else {}
        out = _fft.irfftn(uh, s=self.N, axes=(-3, -2, -1), **kw) * float(np.prod(self.N))
        return out.astype(self.dtype, copy=False)

    def _pad_index(self):
        """(source, target) index arrays of the N modes (Nyquist left out) in the padded spectrum."""
        n0, n1, n2 = self.N
        M0, M1, _ = self.M
        i0 = np.r_[0:n0 // 2, n0 // 2 + 1:n0]
        t0 = np.r_[0:n0 // 2, M0 - n0 // 2 + 1:M0]
        i1 = np.r_[0:n1 // 2, n1 // 2 + 1:n1]
        t1 = np.r_[0:n1 // 2, M1 - n1 // 2 + 1:M1]
        i2 = np.arange(n2 // 2)
        return (i0[:, None, None], i1[None, :, None], i2[None, None, :]), \
            (t0[:, None, None], t1[None, :, None], i2[None, None, :])

    def padded_backward(self, uh):
        """Backward transform on the 3N/2 grid (zero padded spectrum, unnormalised)."""
        src, dst = self._pad_index()
        M0, M1, M2 = self.M
        U = np.zeros(uh.shape[:-3] + (M0, M1, M2 // 2 + 1), dtype=np.complex128)
        U[(Ellipsis,) + dst] = uh[(Ellipsis,) + src]
        kw = {"workers": self.workers} if _HAVE_SCIPY else {}
        out = _fft.irfftn(U, s=self.M, axes=(-3, -2, -1), **kw) * float(np.prod(self.M))
        return out.astype(self.dtype, copy=False)

    def padded_forward(self, u):
        """Forward transform on the 3N/2 grid (scaled by 1/prod(3N/2)), truncated to the N modes."""
        src, dst = self._pad_index()
        kw = {"workers": self.workers} if _HAVE_SCIPY else {}
        F = _fft.rfftn(u, axes=(-3, -2, -1), **kw) / float(np.prod(self.M))
        out = np.zeros(u.shape[:-3] + self.spec_shape, dtype=self.cdtype)
        out[(Ellipsis,) + src] = F[(Ellipsis,) + dst]
        return out

    def _nonlinear(self, a, b):
        """F(F^-1(a) x F^-1(b)), masked: dealiased by truncation (2/3) or by padding (3/2)."""
        m = self.mask
        if self.pad:
            return self.padded_forward(self.cross(self.padded_backward(a * m), self.padded_backward(b * m))) * m
        return self.forward(self.cross(self.backward(a * m), self.backward(b * m))) * m

    # --- pieces of ComputeRHS --------------------------------------------
    def curl_hat(self, uh):
        """cross2: i K x u_hat (maths/cross.py:27-32)."""
        K = self.K
        c = np.empty_like(uh)
        c[0] = 1j * (K[1] * uh[2] - K[2] * uh[1])
        c[1] = 1j * (K[2] * uh[0] - K[0] * uh[2])
        c[2] = 1j * (K[0] * uh[1] - K[1] * uh[0])
        return c

    @staticmethod
    def cross(a, b):
        """cross1: a x b for real fields (maths/cross.py:13-25)."""
        c = np.empty(a.shape, dtype=np.result_type(a, b))
        c[0] = a[1] * b[2] - a[2] * b[1]
        c[1] = a[2] * b[0] - a[0] * b[2]
        c[2] = a[0] * b[1] - a[1] * b[0]
        return c

    def compute_rhs(self, uh, source=None, return_parts=False):
        """ComputeRHS for the Vortex form (NS.py:219-261)."""
        m = self.mask
        uhm = uh * m
        if self.pad:
            u = self.padded_backward(uhm)
            w = self.padded_backward(self.curl_hat(uhm))
            nl = self.padded_forward(self.cross(u, w)) * m
        else:
            u = self.backward(uhm)
            w = self.backward(self.curl_hat(uhm))
            nl = self.forward(self.cross(u, w)) * m
        P = nl[0] * self.K_over_K2[0] + nl[1] * self.K_over_K2[1] + nl[2] * self.K_over_K2[2]
        rhs = np.empty_like(uh)
        nuK2 = self.nu * self.K2
        for i in range(3):
            rhs[i] = nl[i] - P * self.K[i] - nuK2 * uh[i]
        if source is not None:
            rhs += source
        if return_parts:
            return rhs, dict(u=u, curl=w, nl=nl, P_hat=P)
        return rhs

    def velocity_of_vorticity(self, wh):
        """compute_velocity's spectral part: i (K/K2) x w_hat (VV.py:52-67, cross2 with K_over_K2)."""
        Q = self.K_over_K2
        c = np.empty_like(wh)
        c[0] = 1j * (Q[1] * wh[2] - Q[2] * wh[1])
        c[1] = 1j * (Q[2] * wh[0] - Q[0] * wh[2])
        c[2] = 1j * (Q[0] * wh[1] - Q[1] * wh[0])
        return c

    def compute_rhs_vv(self, wh, source=None):
        """ComputeRHS of the velocity-vorticity form (VV.py:85-146), Vortex convection."""
        m = self.mask
        whm = wh * m
        v = self._nonlinear(self.velocity_of_vorticity(whm), whm)
        rhs = self.curl_hat(v) - (self.nu * self.K2) * wh
        if source is not None:
            rhs += source
        return rhs

    def rk4_step(self, uh, dt, source=None, vv=False):
        """One classic RK4 step (integrators.py:149-159) of the NS (or, vv, the VV) right-hand side."""
        u0 = uh.copy()
        u1 = uh.copy()
        u2 = uh.copy()
        dtc = np.asarray(dt, dtype=self.dtype)
        F = self.compute_rhs_vv if vv else self.compute_rhs
        for rk in range(4):
            rhs = F(u0, source)
            if rk < 3:
                u0 = u1 + np.asarray(RK4_B[rk], self.dtype) * dtc * rhs
            u2 += np.asarray(RK4_A[rk], self.dtype) * dtc * rhs
        return u2

    # --- diagnostics ------------------------------------------------------
    def hermitian_weights(self):
        n2 = self.N[2]
        w = np.full(self.spec_shape[2], 2.0)
        w[0] = 1.0
        if n2 % 2 == 0:
            w[-1] = 1.0
        return w

    def energy_fourier(self, uh):
        """sum over the full spectrum of |u_hat|^2 = <u.u> (shenfun energy_fourier)."""
        w = self.hermitian_weights()
        return float(np.sum((np.abs(uh.astype(np.complex128)) ** 2) * w))

    def mean_square(self, f):
        """sum(f*f)/prod(N) in float64 (demo/TG.py:97-98)."""
        f = f.astype(np.float64)
        return float(np.sum(f * f) / np.prod(self.N))

    def kinetic_energy(self, uh):
        return 0.5 * self.mean_square(self.backward(uh))

    def enstrophy(self, uh):
        return 0.5 * self.mean_square(self.backward(self.curl_hat(uh)))

    def divergence_ms(self, uh):
        K = self.K
        d = 1j * (K[0] * uh[0] + K[1] * uh[1] + K[2] * uh[2])
        return 0.5 * self.mean_square(self.backward(d)[None])

    def dissipation(self, uh):
        """nu * energy_fourier(i K x u_hat) (demo/Isotropic.py:241-249)."""
        return self.nu * self.energy_fourier(self.curl_hat(uh))

    def spectrum(self, uh):
        """Shell spectrum of demo/Isotropic.py:88-114 (bins at k+0.5)."""
        uiui = np.zeros(uh[0].shape)
        uiui[..., 1:-1] = 2 * np.sum((uh[..., 1:-1] * np.conj(uh[..., 1:-1])).real, axis=0)
        uiui[..., 0] = np.sum((uh[..., 0] * np.conj(uh[..., 0])).real, axis=0)
        uiui[..., -1] = np.sum((uh[..., -1] * np.conj(uh[..., -1])).real, axis=0)
        uiui *= (4.0 / 3.0 * np.pi)
        Nb = int(np.sqrt(np.sum((np.array(self.N) / 2) ** 2) / 3))
        bins = np.array(range(0, Nb)) + 0.5
        z = np.digitize(np.sqrt(self.K2), bins, right=True)
        Ek = np.zeros(Nb)
        ll = np.zeros(Nb)
        for i, k in enumerate(bins[1:]):
            k0 = bins[i]
            ii = np.where((z > k0) & (z <= k))
            ll[i] = len(ii[0])
            Ek[i] = (k ** 3 - k0 ** 3) * np.sum(uiui[ii])
        for i in range(Nb):
            if ll[i] != 0:
                Ek[i] = Ek[i] / ll[i]
        return Ek, bins

    def shell_spectrum(self, uh):
        """E(k) = 1/2 sum_{k-1/2 < |k| <= k+1/2} |u_hat|^2 (integer shells, full spectrum)."""
        w = self.hermitian_weights()
        e = 0.5 * np.sum(np.abs(uh.astype(np.complex128)) ** 2, axis=0) * w
        kmag = np.sqrt(self.K2) * (self.L[0] / (2 * np.pi))
        idx = np.floor(kmag + 0.5).astype(np.int64)
        nb = int(idx.max()) + 1
        return np.bincount(idx.ravel(), weights=e.ravel(), minlength=nb)

    def cfl_rate(self, uh):
        """max over points of |u|/dx + |v|/dy + |w|/dz of the dealiased field."""
        u = self.backward(uh * self.mask)
        dx = [self.L[i] / self.N[i] for i in range(3)]
        return float(np.max(np.abs(u[0]) / dx[0] + np.abs(u[1]) / dx[1] + np.abs(u[2]) / dx[2]))

    # --- build-defined forcing ------------------------------------------
    def forcing_source(self, uh, eps, kf):
        """Constant-power forcing on 0 < |k| <= kf as a Source term.

        Source = eps / (2 E_f) * u_hat on the shell, with E_f the kinetic
        energy of the shell (full-spectrum sum).  The injected power
        Re<Source, u_hat> equals eps at the start of the step.
        """
        shell = (self.K2 <= kf * kf + 1e-12) & (self.K2 > 0)
        w = self.hermitian_weights()
        Ef = 0.5 * float(np.sum((np.abs(uh.astype(np.complex128)) ** 2) * w * shell))
        src = np.zeros_like(uh)
        if Ef > 0:
            src[:] = (eps / (2.0 * Ef)) * uh * shell
        return src


# Bogacki-Shampine 5(4) pair (P. Bogacki, L. F. Shampine, Comput. Math. Appl.
# 32 (1996) 15-28), as tabulated at spectralDNS/maths/integrators.py:197-209:
# 8 stages, first-same-as-last, embedded order 4.
_BS5_ROWS = (
    (),
    ("1/6",),
    ("2/27", "4/27"),
    ("183/1372", "-162/343", "1053/1372"),
    ("68/297", "-4/11", "42/143", "1960/3861"),
    ("597/22528", "81/352", "63099/585728", "58653/366080", "4617/20480"),
    ("174197/959244", "-30942/79937", "8152137/19744439", "666106/1039181", "-29421/29068", "482048/414219"),
    ("587/8064", "0", "4440339/15491840", "24353/124800", "387/44800", "2152/5985", "7267/94080"),
)
_BS5_BHAT = ("2479/34992", "0", "123/416", "612941/3411720", "43/1440", "2272/6561", "79937/1113912", "3293/556956")


def bs5_tableau(dtype=np.float64):
    """(A, b, bhat) of the BS5 pair in ``dtype`` (integrators.py:197-211)."""
    from fractions import Fraction
    A = np.zeros((8, 8))
    for i, row in enumerate(_BS5_ROWS):
        for j, q in enumerate(row):
            A[i, j] = float(Fraction(q))
    b = A[7].copy()  # the last stage is the solution (FSAL)
    bhat = np.array([float(Fraction(q)) for q in _BS5_BHAT])
    return A.astype(dtype), b.astype(dtype), bhat.astype(dtype)


class Integrator:
    """The non-RK4 integrators of spectralDNS/maths/integrators.py on the oracle grid.

    ``step(uh, dt, tstep)`` returns ``(uh_new, dt_next, dt_taken)`` like the
    reference's integrator closures (getintegrator :177-239):

    * ``ForwardEuler`` (:161-165): ``u += dt F(u)``.
    * ``AB2`` (:167-175): ``u += dt F(u)`` on the first step, then
      ``u += 1.5 dt F(u) - 0.5 (dt F)_previous``.
    * ``BS5_fixed`` / ``BS5_adaptive`` (:15-147 with aTOL = rTOL = TOL):
      FSAL stage reuse through the rotating ``offset``, error norm "2"
      ``max_k sqrt(sum |err_k/sc_k|^2) / sqrt(prod(spectral shape))`` and, when
      adaptive, the step-size controller ``fac=0.8, facmin=0.01, facmax=2``
      (1 after a rejection) with exponent 1/(err_order+1).
    """

    def __init__(self, grid: Grid, name: str, tol: float = 1e-6, source=None):
        self.g = grid
        self.name = name
        self.tol = tol
        self.source = source
        self.prev = None  # AB2: dt F of the previous step
        if name.startswith("BS5"):
            self.A, self.b, self.bhat = bs5_tableau(grid.dtype)
            self.fY = np.zeros((8, 3) + grid.spec_shape, dtype=grid.cdtype)
            self.offset = 0
        elif name not in ("ForwardEuler", "AB2"):
            raise ValueError(name)
        self.rejected = 0

    def F(self, u):
        return self.g.compute_rhs(u, self.source)

    def step(self, uh, dt, tstep):
        dtype = self.g.dtype
        if self.name == "ForwardEuler":
            return uh + self.F(uh) * dtype.type(dt), dt, dt
        if self.name == "AB2":
            rhs = self.F(uh)
            if tstep == 0:
                new = uh + rhs * dtype.type(dt)
            else:
                new = uh + (dtype.type(1.5) * rhs * dtype.type(dt) - dtype.type(0.5) * self.prev)
            self.prev = rhs * dtype.type(dt)
            return new, dt, dt
        return self._adaptive(uh, dt, tstep, adaptive=self.name == "BS5_adaptive")

    def _adaptive(self, u0, dt, tstep, adaptive):
        A, b, bhat, fY = self.A, self.b, self.bhat, self.fY
        s = 8
        facmax, fac, facmin = 2.0, 0.8, 0.01
        exponent = 1.0 / (4 + 1)
        while True:
            dt_prev = dt
            self.offset = (self.offset - 1) % s
            o = self.offset
            for i in range(s):
                if tstep == 0 or i != 0:
                    y = u0.copy()
                    for j in range(i):
                        y += dt * A[i, j] * fY[(j + o) % s]
                    fY[(i + o) % s] = self.F(y)
            u_new = u0.copy()
            err = np.zeros_like(u0)
            for j in range(s):
                u_new += dt * b[j] * fY[(j + o) % s]
                err += dt * (b[j] - bhat[j]) * fY[(j + o) % s]
            sc = self.tol + np.maximum(np.abs(u0), np.abs(u_new)) * self.tol
            nsq = [np.sum(np.abs(err[k].astype(np.complex128) / sc[k]) ** 2) for k in range(3)]
            est = float(np.max(np.sqrt(nsq))) / math.sqrt(float(np.prod(self.g.spec_shape)))
            factor = min(facmax, max(facmin, fac * (1.0 / est) ** exponent))
            if adaptive:
                dt = dt * factor
                if est > 1.0:
                    facmax = 1.0
                    self.rejected += 1
                    self.offset += 1
                    continue
            self.last_est = est
            return u_new, dt, dt_prev


def taylor_green(grid: Grid):
    """TG initial velocity (demo/TG.py:23-28) in physical space."""
    x0 = grid.X[0][:, None, None]
    x1 = grid.X[1][None, :, None]
    x2 = grid.X[2][None, None, :]
    U = np.empty((3,) + grid.N, dtype=grid.dtype)
    U[0] = np.sin(x0) * np.cos(x1) * np.cos(x2)
    U[1] = -np.cos(x0) * np.sin(x1) * np.cos(x2)
    U[2] = 0
    return U


def run_tg(N, steps=10, dt=0.01, nu=0.000625, L=(2 * np.pi,) * 3, dtype=np.float64):
    """TG run as in demo/TG.py; returns (k, w, u_hat)."""
    g = Grid(N, L, nu, dtype=dtype)
    uh = g.forward(taylor_green(g))
    for _ in range(steps):
        uh = g.rk4_step(uh, dt)
    return g.kinetic_energy(uh), g.enstrophy(uh), uh
