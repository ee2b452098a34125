"""ctypes binding of ``libsdns_gb300.so`` (declarations in include/sdns_gb300.h).

The library is the only compute path: if it is missing or cannot be loaded,
:func:`lib` raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

SDNS_OK, SDNS_EINVAL, SDNS_ECUDA, SDNS_ENOMEM, SDNS_ESTATE, SDNS_ENONFINITE = range(6)
SDNS_SINGLE, SDNS_DOUBLE = 0, 1
SDNS_DEALIAS_23, SDNS_DEALIAS_NONE, SDNS_DEALIAS_32 = 0, 1, 2
SDNS_HOST, SDNS_DEVICE = 0, 1
SDNS_NS, SDNS_VV = 0, 1
DIAG_NAMES = ("energy", "enstrophy", "dissipation", "divergence", "cfl_rate", "time", "last_dt")
SDNS_DIAG_COUNT = 8
SDNS_LINCOMB_MAX = 8


class sdns_config(C.Structure):
    _fields_ = [
        ("n", C.c_int32 * 3),
        ("L", C.c_double * 3),
        ("nu", C.c_double),
        ("precision", C.c_int32),
        ("dealias", C.c_int32),
        ("device", C.c_int32),
        ("store_pressure", C.c_int32),
        ("formulation", C.c_int32),
        ("reserved", C.c_int32 * 3),
    ]


class SdnsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("sdns error %d: %s" % (code, msg))
        self.code = code


_P = C.c_void_p
_CTX = C.c_void_p
# name -> (restype, argtypes); every symbol of include/sdns_gb300.h
SIGNATURES = {
    "sdns_abi_version": (C.c_int, []),
    "sdns_last_error": (C.c_char_p, []),
    "sdns_create": (C.c_int, [C.POINTER(sdns_config), C.POINTER(_CTX)]),
    "sdns_destroy": (C.c_int, [_CTX]),
    "sdns_synchronize": (C.c_int, [_CTX]),
    "sdns_get_stream": (C.c_int, [_CTX, C.POINTER(C.c_void_p)]),
    "sdns_memory_bytes": (C.c_int, [_CTX, C.POINTER(C.c_int64)]),
    "sdns_set_state": (C.c_int, [_CTX, _P, C.c_int]),
    "sdns_get_state": (C.c_int, [_CTX, _P, C.c_int]),
    "sdns_set_source": (C.c_int, [_CTX, _P, C.c_int]),
    "sdns_compute_rhs": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "sdns_set_forcing": (C.c_int, [_CTX, C.c_double, C.c_double]),
    "sdns_set_cfl": (C.c_int, [_CTX, C.c_double]),
    "sdns_rk4": (C.c_int, [_CTX, C.c_double, C.c_int32]),
    "sdns_set_time": (C.c_int, [_CTX, C.c_double]),
    "sdns_forward": (C.c_int, [_CTX, _P, _P, C.c_int32, C.c_int]),
    "sdns_backward": (C.c_int, [_CTX, _P, _P, C.c_int32, C.c_int]),
    "sdns_velocity": (C.c_int, [_CTX, _P, C.c_int]),
    "sdns_curl": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "sdns_velocity_vv": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "sdns_pressure": (C.c_int, [_CTX, _P, C.c_int]),
    "sdns_divergence": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "sdns_diagnostics": (C.c_int, [_CTX, C.POINTER(C.c_double)]),
    "sdns_spectrum": (C.c_int, [_CTX, C.POINTER(C.c_double), C.c_int32]),
    "sdns_set_timing": (C.c_int, [_CTX, C.c_int32]),
    "sdns_get_timing": (C.c_int, [_CTX, C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "sdns_lincomb": (C.c_int, [_CTX, _P, _P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_void_p)]),
    "sdns_error_norm": (C.c_int, [_CTX, _P, _P, _P, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "sdns_compute_rhs_noalloc": (C.c_int, [C.POINTER(sdns_config), _P, _P, _P]),
    # learned-closure LES
    "sdns_les_box_filter": (C.c_int, [_P, C.c_int32, _P, C.c_int32, _P, _P, _P]),
    "sdns_les_grad_hat": (C.c_int, [_P, _P, C.c_int32, _P, _P, _P]),
    "sdns_les_sgs_force": (C.c_int, [_P, _P, C.c_int32, _P, _P, C.c_double, _P]),
    "sdns_les_pack": (C.c_int, [_P, C.c_int32, C.c_int64, C.c_int32, _P, _P, _P, _P]),
    "sdns_les_unpack": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int64, _P, _P, _P, _P]),
    "sdns_conv3d_fwd": (C.c_int, [_P, _P, _P, _P, _P, _P, C.c_int32, C.c_int32, C.c_int32, _P]),
    "sdns_conv3d_bwd_data": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.c_int32, _P]),
    "sdns_conv3d_bwd_weight": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32, C.c_int32, _P]),
    "sdns_relu_bwd": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int32, _P]),
    "sdns_mse_grad": (C.c_int, [_P, C.c_int32, C.c_int32, _P, C.c_int64, _P, _P, _P]),
    "sdns_adam_step": (C.c_int, [_P, _P, _P, _P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32,
                                 _P, _P]),
    "sdns_to_bf16": (C.c_int, [_P, _P, C.c_int64, _P]),
}

_lib = None


def lib_path() -> str:
    return _build.lib_path()


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError("libsdns_gb300.so is not built (%s); run `python -m spectraldns_gb300.build` "
                           "or __graft_entry__.build()" % path)
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code):
    if code != SDNS_OK:
        msg = lib().sdns_last_error()
        raise SdnsError(code, msg.decode() if msg else "")
    return code
