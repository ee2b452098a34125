"""Build recipe: the reference's own Cython kernels, compiled from its sources.

TEST INFRASTRUCTURE ONLY.  spectralDNS ships its optimised CPU kernels as
Cython templates (``spectralDNS/optimization/cython_{maths,solvers,integrators}.in``)
from which its ``optimization/setup.py:38-53`` writes one single- and one
double-precision ``.pyx`` per module by substituting the precision's
``ctypedef`` block into the template.  This recipe does the same substitution,
reading the templates where they lie in the reference tree (never copying
them into this repository), and compiles the six modules with Cython 3
(language level 2, as the templates use ``xrange``) into ``oracle/_ref/``,
which git ignores.  The CPU tests import them to pin the oracle's pointwise
arithmetic (``cross1``, ``cross2``, ``add_pressure_diffusion_NS``) and its
RK4 / ForwardEuler / AB2 updates to the reference's compiled code.

Usage: ``python oracle/build_ref_cython.py [reference root]``; the reference
root defaults to ``$SPECTRALDNS_REF`` or ``/root/reference``.  Without the
reference tree or without Cython it does nothing and says so.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MODULES = ("maths", "solvers", "integrators")
# the precision blocks substituted for "{0}" in the templates (optimization/setup.py:26-37)
PRECISION = {
    "single": "\nctypedef np.complex64_t complex_t\nctypedef np.float32_t real_t\nctypedef np.int64_t int_t\n",
    "double": "\nctypedef np.complex128_t complex_t\nctypedef np.float64_t real_t\nctypedef np.int64_t int_t\n",
}


def reference_root(argv=None):
    if argv and len(argv) > 1:
        return argv[1]
    return os.environ.get("SPECTRALDNS_REF", "/root/reference")


def built():
    """True when every module of the recipe is importable from oracle/_ref."""
    if not os.path.isdir(OUT):
        return False
    names = os.listdir(OUT)
    return all(any(n.startswith("cython_%s_%s." % (p, m)) and n.endswith(".so") for n in names)
               for p in PRECISION for m in MODULES)


def build(root=None, verbose=False):
    root = root or reference_root()
    opt = os.path.join(root, "spectralDNS", "optimization")
    if not os.path.isdir(opt):
        if verbose:
            print("reference tree not found at %s: nothing to build" % root)
        return False
    try:
        import numpy
        from Cython.Build import cythonize
        from setuptools import Extension
        from setuptools.dist import Distribution
    except ImportError as e:
        if verbose:
            print("Cython/setuptools not available (%s): nothing to build" % e)
        return False
    if built():
        return True
    os.makedirs(OUT, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="sdns_ref_cython_")
    try:
        exts = []
        for m in MODULES:
            with open(os.path.join(opt, "cython_%s.in" % m)) as f:
                template = f.read()
            for p, block in PRECISION.items():
                name = "cython_%s_%s" % (p, m)
                pyx = os.path.join(tmp, name + ".pyx")
                with open(pyx, "w") as f:
                    f.write(template.format(block))
                exts.append(Extension(name, [pyx], include_dirs=[numpy.get_include()],
                                      extra_compile_args=["-O2", "-w"]))
        ext_modules = cythonize(exts, compiler_directives={"language_level": 2}, build_dir=tmp, quiet=not verbose,
                                nthreads=min(6, os.cpu_count() or 1))
        dist = Distribution({"ext_modules": ext_modules})
        cmd = dist.get_command_obj("build_ext")
        cmd.build_lib = OUT
        cmd.build_temp = os.path.join(tmp, "build")
        cmd.parallel = min(6, os.cpu_count() or 1)
        cmd.ensure_finalized()
        cmd.run()
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return built()


if __name__ == "__main__":
    ok = build(reference_root(sys.argv), verbose=True)
    print("oracle/_ref:", "built" if ok else "not built")
