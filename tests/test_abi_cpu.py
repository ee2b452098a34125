"""CPU checks of the C ABI: the library loads without a GPU and exports every
function include/sdns_gb300.h declares; the ctypes table matches the header."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sdns_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\*?\s+\**(sdns_[a-z_0-9]+)\s*\(", src, flags=re.M)))


def test_header_parses():
    fns = header_functions()
    assert "sdns_create" in fns and "sdns_rk4" in fns and "sdns_compute_rhs" in fns
    assert len(fns) >= 20


def test_library_exports_header_symbols():
    from spectraldns_gb300 import build, _lib
    build.build()
    L = _lib.lib()  # loads on a machine without a GPU (static CUDA runtime)
    missing = [f for f in header_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    from spectraldns_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(header_functions())


def test_abi_version_and_error_without_gpu():
    from spectraldns_gb300 import _lib
    L = _lib.lib()
    assert L.sdns_abi_version() == 1
    import ctypes as C
    cfg = _lib.sdns_config()
    cfg.n[:] = (17, 16, 16)  # not a power of two: rejected before any CUDA call
    cfg.L[:] = (1.0, 1.0, 1.0)
    h = C.c_void_p()
    assert L.sdns_create(C.byref(cfg), C.byref(h)) == _lib.SDNS_EINVAL
    assert b"powers of two" in L.sdns_last_error()


def test_noalloc_rejects_unsupported_configs_without_gpu():
    """The allocation-free entry point checks its configuration before any CUDA call: the
    3/2 rule and the velocity-vorticity formulation are rejected."""
    import ctypes as C
    from spectraldns_gb300 import _lib
    L = _lib.lib()
    for dealias, form in ((_lib.SDNS_DEALIAS_32, _lib.SDNS_NS), (_lib.SDNS_DEALIAS_23, _lib.SDNS_VV)):
        cfg = _lib.sdns_config()
        cfg.n[:] = (16, 16, 16)
        cfg.L[:] = (1.0, 1.0, 1.0)
        cfg.dealias = dealias
        cfg.formulation = form
        buf = (C.c_byte * 16)()
        assert L.sdns_compute_rhs_noalloc(C.byref(cfg), buf, buf, None) == _lib.SDNS_EINVAL


def test_header_is_c99_and_links():
    """include/sdns_gb300.h is plain C: a C99 program compiles against it with -Wall -Werror,
    links with libsdns_gb300.so and makes the calls that need no GPU (tests/c/abi_c99.c)."""
    import shutil
    import subprocess
    import tempfile
    from spectraldns_gb300 import build
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    lib = build.build()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "abi_c99")
        cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "c", "abi_c99.c"), "-o", exe, "-L", os.path.dirname(lib),
               "-l:" + os.path.basename(lib), "-Wl,-rpath," + os.path.dirname(lib)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
        assert "c99 caller ok" in r.stdout
