"""Checkpoint and results files of the time loop (spectralDNS/h5io/HDF5File.py).

h5py is not available to this backend, so the files are NumPy ``.npz``
archives whose member names are the HDF5 dataset paths the reference's
ShenfunFile writes, e.g. ``U/3D/0`` for time level 0 of the checkpointed
vector ``U`` (read back by ``init_from_file`` as demo/Isotropic.py:267-282
reads ``f["U/3D/0"]``):

* checkpoint ``<filename>_c.npz``: every array of ``checkpoint['data']``
  (``{level: {name: [array]}}``) as ``<name>/3D/<level>``, plus ``tstep`` and
  ``t`` (the HDF5 attributes of HDF5File.py:67-69, 84-88).  It is written
  to a temporary file and renamed, so a crash while writing leaves the
  previous checkpoint intact.
* results ``<filename>_w_<tstep>.npz``: every array of ``results['data']``
  (``{name: [array]}``) as ``<name>/3D/<tstep>``, plus ``t`` (HDF5File.py:76-78).

A file named ``killspectraldns`` in the working directory makes the next
``update`` write a checkpoint and exit with status 1 (HDF5File.py:80-92,
107-120).
"""
from __future__ import annotations

import os
import sys

import numpy as np

__all__ = ["HDF5File", "read_checkpoint", "init_from_file"]


class HDF5File:
    """Stores checkpoint and results data of a run (HDF5File.py:12-105)."""

    def __init__(self, filename, checkpoint=None, results=None):
        self.filename = filename
        self.checkpoint = checkpoint if checkpoint is not None else {"data": {}}
        self.results = results if results is not None else {"data": {}}

    # hooks ---------------------------------------------------------------
    def update_components(self, **kw):
        """Transform the results arrays to physical space before they are stored."""

    def refresh(self, **kw):
        """Make the checkpoint arrays current (the GPU solver's lazy mode keeps the state on the device)."""

    # files ---------------------------------------------------------------
    def checkpoint_path(self):
        return self.filename + "_c.npz"

    def write_checkpoint(self, params, **kw):
        self.refresh(**kw)
        arrays = {"tstep": np.int64(params.tstep), "t": np.float64(params.t)}
        for level, fields in self.checkpoint.get("data", {}).items():
            for name, val in fields.items():
                arrays["%s/3D/%s" % (name, level)] = np.asarray(val[0])
        path = self.checkpoint_path()
        tmp = path + ".tmp.npz"
        np.savez(tmp, **arrays)
        os.replace(tmp, path)

    def write_results(self, params, **kw):
        self.update_components(**kw)
        arrays = {"t": np.float64(params.t)}
        for name, val in self.results.get("data", {}).items():
            arrays["%s/3D/%d" % (name, params.tstep)] = np.asarray(val[0])
        np.savez(self.filename + "_w_%d.npz" % params.tstep, **arrays)

    def update(self, params, **kw):
        """Called after every time step by solve() (spectralDNS/__init__.py:69-123)."""
        if params.tstep % params.write_result == 0:
            self.write_results(params, **kw)
        kill = self.check_if_kill()
        if params.tstep % params.checkpoint == 0 or kill:
            self.write_checkpoint(params, **kw)
            if kill:
                sys.exit(1)

    def open(self):
        pass

    def close(self):
        pass

    @staticmethod
    def check_if_kill():
        """True (and the file removed) if ``killspectraldns`` is in the working directory."""
        if os.path.exists("killspectraldns"):
            os.remove("killspectraldns")
            print("killspectraldns Found! Stopping simulations cleanly by checkpointing...")
            return True
        return False


def read_checkpoint(filename):
    """Arrays and attributes of a checkpoint (``<filename>_c.npz`` or the path itself)."""
    path = filename if filename.endswith(".npz") else filename + "_c.npz"
    with np.load(path) as f:
        return {k: f[k] for k in f.files}


def init_from_file(filename, solver, context, level="0", name="U"):
    """Restart from a checkpoint: U_hat, t and tstep (demo/Isotropic.py:267-282).

    The arrays are copied into the context's host arrays; the next step of
    the time loop uploads them to the GPU.  A velocity-vorticity context also
    gets W_hat = i K x U_hat, as the reference does.
    """
    from . import config
    d = read_checkpoint(filename)
    key = "%s/3D/%s" % (name, level)
    if key not in d:
        raise KeyError("%s has no dataset %s (has %s)" % (filename, key, sorted(d)))
    U_hat = context.U_hat
    if d[key].shape != U_hat.shape:
        raise ValueError("checkpoint %s has shape %s, the context %s" % (key, d[key].shape, U_hat.shape))
    U_hat[:] = d[key]
    if "VV" in str(config.params.get("solver", "")) and "W_hat" in context:
        context.W_hat = solver.cross2(context.W_hat, context.K, context.U_hat)
    config.params.t = float(d["t"])
    config.params.tstep = int(d["tstep"])
    return context
