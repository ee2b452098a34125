"""Parameters and command-line flags of the GB300 backend.

Mirrors the interface of spectralDNS/config.py: ``params`` is an attribute
dictionary (spectralDNS/config.py:96-148) that casts ``nu`` and ``dt`` to the
working float type (:123-127) and derives ``N = 2**M`` (:110-121); the
argparse parsers ``parser`` / ``triplyperiodic`` carry the same flags
(:164-237) and ``update(dict, mesh)`` sets their defaults (:307-314).  Only
the triply periodic ``NS`` solver is provided by this backend; the GPU adds
``--device`` and ``--gpu_sync``.
"""
from __future__ import annotations

import argparse
import ast
import json
import operator
from collections import defaultdict
from collections.abc import MutableMapping

import numpy as np


class AttributeDict(MutableMapping, dict):
    """Dictionary whose values are also attributes (p.M is p['M'])."""

    def __init__(self, *args, **kwargs):
        dict.__init__(self, *args, **kwargs)
        self.__dict__ = self

    def __getattribute__(self, key):
        return dict.__getattribute__(self, key)

    def __setattr__(self, key, val):
        dict.__setattr__(self, key, val)

    def __getitem__(self, key):
        return dict.__getitem__(self, key)

    def __setitem__(self, key, val):
        dict.__setitem__(self, key, val)

    def __delitem__(self, key):
        dict.__delitem__(self, key)

    def __iter__(self):
        return dict.__iter__(self)

    def __len__(self):
        return dict.__len__(self)

    def __contains__(self, x):
        return dict.__contains__(self, x)


_OPS = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow, ast.USub: operator.neg, ast.UAdd: operator.pos}


def _length(expr) -> float:
    """Evaluate a box-length expression such as '2*pi' (numbers, pi, + - * / **)."""
    if isinstance(expr, (int, float, np.floating, np.integer)):
        return float(expr)

    def ev(node):
        if isinstance(node, ast.Expression):
            return ev(node.body)
        if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
            return float(node.value)
        if isinstance(node, ast.Name) and node.id == "pi":
            return float(np.pi)
        if isinstance(node, ast.BinOp) and type(node.op) in _OPS:
            return _OPS[type(node.op)](ev(node.left), ev(node.right))
        if isinstance(node, ast.UnaryOp) and type(node.op) in _OPS:
            return _OPS[type(node.op)](ev(node.operand))
        raise ValueError("unsupported length expression %r" % (expr,))
    return ev(ast.parse(str(expr), mode="eval"))


class Params(AttributeDict):
    """Solver parameters (spectralDNS/config.py:96-148 interface)."""

    def __getattr__(self, key):
        if key == "dx":
            return self.L / self.N
        if key == "N":
            if "M" not in self:
                raise KeyError("N")
            return 2 ** self.M
        raise KeyError(key)

    def __getattribute__(self, key):
        if key in ("nu", "dt"):
            fl = np.float32 if dict.get(self, "precision") == "single" else np.float64
            return fl(dict.__getattribute__(self, key))
        return dict.__getattribute__(self, key)

    def __setattr__(self, key, val):
        if key in ("N", "M", "L"):
            self.__setitem__(key, val)
        else:
            dict.__setattr__(self, key, val)

    def __setitem__(self, key, val):
        if key in ("M", "N"):
            val = np.array([int(str(f)) for f in val], dtype=int)
            val.flags.writeable = False
        elif key == "L":
            val = np.array([_length(f) for f in val], dtype=float)
            val.flags.writeable = False
        dict.__setitem__(self, key, val)


fft_plans = defaultdict(lambda: "FFTW_MEASURE", {"dct": "FFTW_MEASURE"})


class PlanAction(argparse.Action):
    """--planner_effort JSON (accepted for interface compatibility; the GPU plans nothing)."""

    def __call__(self, parser, namespace, values, option_string=None):
        fft_plans.update(json.loads(values))
        setattr(namespace, self.dest, fft_plans)


params = Params()

parser = argparse.ArgumentParser(prog="spectralDNS", add_help=False)
parser.add_argument("--precision", default="double", choices=("single", "double"))
parser.add_argument("--optimization", default="", choices=("", "cython", "weave", "numba", "pythran"),
                    help="accepted for compatibility; every kernel runs on the GPU")
parser.add_argument("--make_profile", default=0, type=int, help="Enable cProfile profiler")
parser.add_argument("--dt", default=0.01, type=float, help="Time step size")
parser.add_argument("--T", default=0.1, type=float, help="End time")
parser.add_argument("--write_result", default=int(1e8), type=int, help="Write results every tstep")
parser.add_argument("--checkpoint", default=int(1e8), type=int, help="Save a checkpoint every tstep")
parser.add_argument("--nu", default=0.000625, type=float, help="Viscosity")
parser.add_argument("--t", default=0.0, type=float, help="Time")
parser.add_argument("--tstep", default=0, type=int, help="Time step")
parser.add_argument("--filemode", default="w", choices=("w", "r", "a"))
parser.add_argument("--dealias", default="2/3-rule", choices=("2/3-rule", "3/2-rule", "None"))
parser.add_argument("--decomposition", default="slab", choices=("slab", "pencil"))
parser.add_argument("--ntol", default=7, type=int, help="Tolerance - number of accurate digits")
parser.add_argument("--threads", default=1, type=int)
parser.add_argument("--planner_effort", action=PlanAction, default=fft_plans)
parser.add_argument("--h5filename", default="results", type=str)
parser.add_argument("--verbose", dest="verbose", action="store_true")
parser.add_argument("--no-verbose", dest="verbose", action="store_false")
parser.set_defaults(verbose=True)
parser.add_argument("--mask_nyquist", dest="mask_nyquist", action="store_true")
parser.add_argument("--no-mask_nyquist", dest="mask_nyquist", action="store_false")
parser.set_defaults(mask_nyquist=True)
# GB300 backend
parser.add_argument("--device", default=0, type=int, help="CUDA device of the solver")
parser.add_argument("--gpu_sync", default="step", choices=("step", "lazy"),
                    help="step: U_hat is copied to/from the GPU every time step (drop-in); lazy: the state "
                         "stays on the GPU and hooks read it through the getters")

triplyperiodic = argparse.ArgumentParser(parents=[parser])
triplyperiodic.add_argument("--convection", default="Vortex", choices=("Standard", "Divergence", "Skewed", "Vortex"))
triplyperiodic.add_argument("--L", default=[2 * np.pi, 2 * np.pi, 2 * np.pi], nargs=3, metavar=("Lx", "Ly", "Lz"))
triplyperiodic.add_argument("--M", default=[6, 6, 6], nargs=3, metavar=("Mx", "My", "Mz"))
triplyperiodic.add_argument("--TOL", type=float, default=1e-6)
triplyperiodic.add_argument("--integrator", default="RK4",
                            choices=("RK4", "ForwardEuler", "AB2", "BS5_adaptive", "BS5_fixed"))
_sub = triplyperiodic.add_subparsers(dest="solver")
parser_NS = _sub.add_parser("NS", help="Navier-Stokes solver (Vortex form) on the GB300")
parser_VV = _sub.add_parser("VV", help="Velocity-vorticity Navier-Stokes solver (Vortex form) on the GB300")

solver = None  # set by get_solver


def update(new, mesh="triplyperiodic"):
    """Set parser defaults (spectralDNS/config.py:307-314)."""
    assert isinstance(new, dict)
    if "planner_effort" in new:
        fft_plans.update(new["planner_effort"])
        new["planner_effort"] = fft_plans
    if mesh != "triplyperiodic":
        raise ValueError("the GB300 backend provides the triply periodic mesh only (got %r)" % mesh)
    globals()[mesh].set_defaults(**new)
