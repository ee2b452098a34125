"""Python handle of one GPU solver context (one grid, one CUDA stream).

Arrays crossing the boundary use the reference's single-rank numpy layouts:
spectral vectors ``(3, N0, N1, N2//2+1)`` complex, physical vectors
``(3, N0, N1, N2)`` real.  They may be numpy arrays / torch CPU tensors
(host; pinned torch tensors transfer fastest) or torch CUDA tensors on the
context's device (no host copy).  Everything is computed by
``libsdns_gb300.so``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

try:  # torch is optional plumbing for device buffers and pinned host memory
    import torch
except ImportError:  # pragma: no cover
    torch = None


def _is_torch(a):
    return torch is not None and isinstance(a, torch.Tensor)


class Context:
    """GPU state of the NS solver (spectralDNS solvers/NS.py:12-72 get_context)."""

    def __init__(self, N, L=(2 * np.pi,) * 3, nu=0.000625, precision="double", dealias="2/3-rule",
                 device=0, store_pressure=False, formulation="NS"):
        self.N = tuple(int(n) for n in N)
        self.L = tuple(float(x) for x in L)
        self.nu = float(nu)
        if precision not in ("single", "double"):
            raise ValueError("precision must be 'single' or 'double'")
        if dealias not in ("2/3-rule", "3/2-rule", "None"):
            raise ValueError("dealias %r is not supported by the GPU backend (2/3-rule, 3/2-rule or None)"
                             % (dealias,))
        if formulation not in ("NS", "VV"):
            raise ValueError("formulation must be 'NS' (velocity) or 'VV' (velocity-vorticity)")
        self.precision = precision
        self.dealias = dealias
        self.formulation = formulation
        self.device = int(device)
        self.real = np.float32 if precision == "single" else np.float64
        self.complex = np.complex64 if precision == "single" else np.complex128
        n0, n1, n2 = self.N
        self.spec_shape = (3, n0, n1, n2 // 2 + 1)
        self.phys_shape = (3, n0, n1, n2)
        cfg = _lib.sdns_config()
        cfg.n[:] = self.N
        cfg.L[:] = self.L
        cfg.nu = self.nu
        cfg.precision = _lib.SDNS_SINGLE if precision == "single" else _lib.SDNS_DOUBLE
        cfg.dealias = {"2/3-rule": _lib.SDNS_DEALIAS_23, "3/2-rule": _lib.SDNS_DEALIAS_32,
                       "None": _lib.SDNS_DEALIAS_NONE}[dealias]
        cfg.device = self.device
        cfg.store_pressure = 1 if store_pressure and formulation == "NS" else 0
        cfg.formulation = _lib.SDNS_VV if formulation == "VV" else _lib.SDNS_NS
        self._L = _lib.lib()
        h = C.c_void_p()
        check(self._L.sdns_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = []
        # ordered = True: the caller launches everything that produces or reads the device
        # tensors it passes on the context stream (e.g. under torch.cuda.stream of
        # torch.cuda.ExternalStream(stream_handle())), so calls skip the host synchronisations
        # that otherwise order torch's stream and the context stream around them
        self.ordered = False

    # -- plumbing -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.sdns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arg_in(self, a, dtype, shape):
        """(pointer, where, keepalive) of an input array."""
        if _is_torch(a):
            if a.is_cuda:
                if a.device.index != self.device:
                    raise ValueError("tensor on cuda:%s, context on cuda:%d" % (a.device.index, self.device))
                t = a.contiguous()
                if t.dtype != _torch_dtype(dtype):
                    t = t.to(_torch_dtype(dtype))
                if tuple(t.shape) != tuple(shape):
                    t = t.reshape(shape)
                if not self.ordered:
                    torch.cuda.current_stream(t.device).synchronize()
                return t.data_ptr(), _lib.SDNS_DEVICE, t
            a = a.numpy()
        arr = np.ascontiguousarray(a, dtype=dtype)
        if arr.size != int(np.prod(shape)):
            raise ValueError("array of size %d, expected shape %s" % (arr.size, shape))
        return arr.ctypes.data, _lib.SDNS_HOST, arr

    def _arg_out(self, out, dtype, shape):
        """(pointer, where, array, writeback) of an output array."""
        if out is None:
            arr = np.empty(shape, dtype=dtype)
            return arr.ctypes.data, _lib.SDNS_HOST, arr, None
        if _is_torch(out):
            if out.is_cuda:
                if not out.is_contiguous() or out.dtype != _torch_dtype(dtype):
                    raise ValueError("device output must be a contiguous %s tensor" % dtype)
                if not self.ordered:
                    torch.cuda.current_stream(out.device).synchronize()
                return out.data_ptr(), _lib.SDNS_DEVICE, out, None
            if out.is_contiguous() and out.dtype == _torch_dtype(dtype):
                return out.data_ptr(), _lib.SDNS_HOST, out, None
            tmp = np.empty(shape, dtype=dtype)
            return tmp.ctypes.data, _lib.SDNS_HOST, tmp, out
        if out.flags.c_contiguous and out.dtype == dtype and out.size == int(np.prod(shape)):
            return out.ctypes.data, _lib.SDNS_HOST, out, None
        tmp = np.empty(shape, dtype=dtype)
        return tmp.ctypes.data, _lib.SDNS_HOST, tmp, out

    def _finish(self, arr, writeback, where):
        if where == _lib.SDNS_DEVICE and not self.ordered:
            check(self._L.sdns_synchronize(self._h))
        if writeback is not None:
            if _is_torch(writeback):
                writeback.copy_(torch.from_numpy(arr))
            else:
                writeback[...] = arr.reshape(writeback.shape)
            return writeback
        return arr

    # -- state ----------------------------------------------------------------
    def set_state(self, u_hat):
        p, w, keep = self._arg_in(u_hat, self.complex, self.spec_shape)
        check(self._L.sdns_set_state(self._h, C.c_void_p(p), w))
        del keep

    def get_state(self, out=None):
        p, w, arr, wb = self._arg_out(out, self.complex, self.spec_shape)
        check(self._L.sdns_get_state(self._h, C.c_void_p(p), w))
        return self._finish(arr, wb, w)

    def set_source(self, source):
        if source is None:
            check(self._L.sdns_set_source(self._h, None, _lib.SDNS_HOST))
            return
        p, w, keep = self._arg_in(source, self.complex, self.spec_shape)
        check(self._L.sdns_set_source(self._h, C.c_void_p(p), w))

    def set_forcing(self, eps, kf):
        check(self._L.sdns_set_forcing(self._h, float(eps), float(kf)))

    def set_cfl(self, cfl):
        check(self._L.sdns_set_cfl(self._h, float(cfl)))

    def set_time(self, t):
        check(self._L.sdns_set_time(self._h, float(t)))

    # -- compute ----------------------------------------------------------------
    def compute_rhs(self, u_hat, out=None):
        """ComputeRHS (spectralDNS solvers/NS.py:219-261), Vortex form."""
        p, w, keep = self._arg_in(u_hat, self.complex, self.spec_shape)
        if w == _lib.SDNS_DEVICE and out is None:
            out = torch.empty(self.spec_shape, dtype=_torch_dtype(self.complex), device=keep.device)
        q, w2, arr, wb = self._arg_out(out, self.complex, self.spec_shape)
        if w2 != w:
            raise ValueError("u_hat and rhs must both be host or both be device arrays")
        check(self._L.sdns_compute_rhs(self._h, C.c_void_p(p), C.c_void_p(q), w))
        return self._finish(arr, wb, w)

    def rk4(self, dt, nsteps=1):
        """nsteps RK4 steps (spectralDNS maths/integrators.py:149-159)."""
        check(self._L.sdns_rk4(self._h, float(dt), int(nsteps)))

    def synchronize(self):
        check(self._L.sdns_synchronize(self._h))

    def stream_handle(self):
        """Raw cudaStream_t of the context (wrap with torch.cuda.ExternalStream)."""
        s = C.c_void_p()
        check(self._L.sdns_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def _transform(self, fn, a, out, in_dtype, out_dtype, in_tail, out_tail):
        shp = tuple(np.shape(a)) if not _is_torch(a) else tuple(a.shape)
        nf = 1 if len(shp) == 3 else shp[0]
        ishape = (nf,) + in_tail if len(shp) == 4 else in_tail
        oshape = (nf,) + out_tail if len(shp) == 4 else out_tail
        p, w, keep = self._arg_in(a, in_dtype, ishape)
        if w == _lib.SDNS_DEVICE and out is None:
            out = torch.empty(oshape, dtype=_torch_dtype(out_dtype), device=keep.device)
        q, w2, arr, wb = self._arg_out(out, out_dtype, oshape)
        if w2 != w:
            raise ValueError("input and output must both be host or both be device arrays")
        check(fn(self._h, C.c_void_p(p), C.c_void_p(q), nf, w))
        return self._finish(arr, wb, w)

    def forward(self, u, out=None):
        """shenfun VT.forward / T.forward: R2C(z) C2C(y) C2C(x), scaled 1/(N0 N1 N2)."""
        n0, n1, n2 = self.N
        return self._transform(self._L.sdns_forward, u, out, self.real, self.complex,
                               (n0, n1, n2), (n0, n1, n2 // 2 + 1))

    def backward(self, u_hat, out=None):
        """shenfun VT.backward / T.backward (unnormalised)."""
        n0, n1, n2 = self.N
        return self._transform(self._L.sdns_backward, u_hat, out, self.complex, self.real,
                               (n0, n1, n2 // 2 + 1), (n0, n1, n2))

    def _phys(self, fn, out, nf):
        shape = self.phys_shape if nf == 3 else self.phys_shape[1:]
        p, w, arr, wb = self._arg_out(out, self.real, shape)
        check(fn(self._h, C.c_void_p(p), w))
        return self._finish(arr, wb, w)

    def velocity(self, out=None):
        """Velocity of the context state (for a VV context: of the vorticity state)."""
        return self._phys(self._L.sdns_velocity, out, 3)

    def velocity_vv(self, w_hat=None, out=None):
        """F^-1(i K x w_hat / K^2): the velocity of a vorticity spectral vector (None: the state)."""
        return self._phys_of(self._L.sdns_velocity_vv, w_hat, out, 3)

    def _phys_of(self, fn, u_hat, out, nf):
        """fn(ctx, u_hat or NULL, out, where) for the spectral vector u_hat (None: the state)."""
        shape = self.phys_shape if nf == 3 else self.phys_shape[1:]
        if u_hat is None:
            p, w, arr, wb = self._arg_out(out, self.real, shape)
            check(fn(self._h, None, C.c_void_p(p), w))
            return self._finish(arr, wb, w)
        q, w1, keep = self._arg_in(u_hat, self.complex, self.spec_shape)
        if w1 == _lib.SDNS_DEVICE and out is None:
            out = torch.empty(shape, dtype=_torch_dtype(self.real), device=keep.device)
        p, w, arr, wb = self._arg_out(out, self.real, shape)
        if w != w1:
            raise ValueError("input and output must both be host or both be device arrays")
        check(fn(self._h, C.c_void_p(q), C.c_void_p(p), w))
        return self._finish(arr, wb, w)

    def curl(self, u_hat=None, out=None):
        """F^-1(i K x u_hat); u_hat None: of the context state."""
        return self._phys_of(self._L.sdns_curl, u_hat, out, 3)

    def pressure(self, out=None):
        return self._phys(self._L.sdns_pressure, out, 1)

    def divergence(self, u_hat=None, out=None):
        """F^-1(i K . u_hat); u_hat None: of the context state."""
        return self._phys_of(self._L.sdns_divergence, u_hat, out, 1)

    def diagnostics(self):
        buf = (C.c_double * _lib.SDNS_DIAG_COUNT)()
        check(self._L.sdns_diagnostics(self._h, buf))
        return {k: buf[i] for i, k in enumerate(_lib.DIAG_NAMES)}

    def spectrum(self, nbins=None):
        if nbins is None:
            nbins = int(np.sqrt(np.sum((np.array(self.N) / 2) ** 2) / 3))
        buf = (C.c_double * nbins)()
        check(self._L.sdns_spectrum(self._h, buf, nbins))
        return np.array(buf[:])

    # -- integrator building blocks (device spectral vectors) ---------------------
    def _dev_vec(self, t, name):
        if not (_is_torch(t) and t.is_cuda):
            raise ValueError("%s must be a CUDA tensor" % name)
        if t.device.index != self.device or not t.is_contiguous() or t.dtype != _torch_dtype(self.complex) \
                or tuple(t.shape) != self.spec_shape:
            raise ValueError("%s must be a contiguous %s tensor of shape %s on cuda:%d"
                             % (name, np.dtype(self.complex).name, self.spec_shape, self.device))
        return t.data_ptr()

    def lincomb(self, out, base, coefs, terms):
        """out = base + sum_k coefs[k] * terms[k] on device spectral vectors (base None: 0).

        Enqueued on the context stream after the work pending on torch's
        current stream (which may still be writing the operands), like every
        other call of the context that takes device tensors.
        """
        n = len(terms)
        if not self.ordered:
            torch.cuda.current_stream(out.device).synchronize()
        if n != len(coefs) or n > _lib.SDNS_LINCOMB_MAX:
            raise ValueError("at most %d terms, one coefficient each" % _lib.SDNS_LINCOMB_MAX)
        po = self._dev_vec(out, "out")
        pb = self._dev_vec(base, "base") if base is not None else None
        ptrs = (C.c_void_p * max(n, 1))(*[self._dev_vec(t, "term") for t in terms])
        cf = (C.c_double * max(n, 1))(*[float(c) for c in coefs])
        check(self._L.sdns_lincomb(self._h, C.c_void_p(po), C.c_void_p(pb) if pb else None, n, cf, ptrs))
        return out

    def error_norm(self, err, u0, u1, atol, rtol):
        """float64 [sum_k |err/sc|^2 for k = 0, 1, 2], sc = atol + max(|u0|, |u1|) rtol."""
        sums = (C.c_double * 3)()
        if not self.ordered:
            torch.cuda.current_stream(err.device).synchronize()
        check(self._L.sdns_error_norm(self._h, C.c_void_p(self._dev_vec(err, "err")),
                                      C.c_void_p(self._dev_vec(u0, "u0")), C.c_void_p(self._dev_vec(u1, "u1")),
                                      float(atol), float(rtol), sums))
        return np.array(sums[:])

    def empty_vec(self):
        """Uninitialised device spectral vector of the context precision (a torch CUDA tensor)."""
        return torch.empty(self.spec_shape, dtype=_torch_dtype(self.complex), device="cuda:%d" % self.device)

    def memory_bytes(self):
        b = C.c_int64()
        check(self._L.sdns_memory_bytes(self._h, C.byref(b)))
        return b.value

    def set_timing(self, on=True):
        check(self._L.sdns_set_timing(self._h, 1 if on else 0))

    def get_timing(self):
        ms = (C.c_double * 8)()
        n = (C.c_int32 * 8)()
        check(self._L.sdns_get_timing(self._h, ms, n))
        return list(ms), list(n)


def _torch_dtype(np_dtype):
    return {np.float32: torch.float32, np.float64: torch.float64,
            np.complex64: torch.complex64, np.complex128: torch.complex128}[np.dtype(np_dtype).type]
