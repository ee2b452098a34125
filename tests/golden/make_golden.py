"""Generate golden fixtures from the reference's own slab solver.

Runs ``spectralDNS3D_short.py`` from the spectralDNS source tree, unmodified,
under a single-rank ``mpi4py`` stand-in (the real mpi4py is not installed),
then evaluates the script's own ``ComputeRHS`` on a seeded random solenoidal
field.  Writes ``short64.npz`` next to this file:

* ``tg_k``                    the script's kinetic energy after T=0.1 (10 RK4 steps, N=64)
* ``tg_idx``/``tg_val``       the TG state U_hat after 10 steps, every mode with |U_hat|>1e-12
* ``rhs_seed``                seed of the random input (see ``random_input``)
* ``rhs_idx``/``rhs_val``     ComputeRHS(U_hat=random_input) at 2048 sampled modes

Usage: ``python tests/golden/make_golden.py [path-to-spectralDNS-tree]``.
The reference tree is read only here; the fixture file travels with the tests.
"""
import os
import runpy
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

MPI_STUB = '''
IN_PLACE = object()
DOUBLE = "double"
DOUBLE_COMPLEX = "double_complex"
class _Comm:
    def Get_size(self): return 1
    def Get_rank(self): return 0
    def Alltoall(self, a, b): return None
    def reduce(self, x, op=None, root=0): return x
    def allreduce(self, x, op=None): return x
    def bcast(self, x, root=0): return x
    def barrier(self): return None
COMM_WORLD = _Comm()
'''


def random_input(seed, N=64):
    """Seeded solenoidal field inside the 2/3 set, as used for the RHS fixture."""
    rng = np.random.default_rng(seed)
    shape = (3, N, N, N // 2 + 1)
    uh = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    kx = np.fft.fftfreq(N, 1.0 / N)
    kz = np.arange(N // 2 + 1, dtype=float)
    K = np.array(np.meshgrid(kx, kx, kz, indexing="ij"))
    K2 = np.sum(K * K, 0)
    kmax = 2.0 / 3.0 * (N // 2 + 1)
    mask = (np.abs(K[0]) < kmax) & (np.abs(K[1]) < kmax) & (np.abs(K[2]) < kmax)
    uh *= mask * np.exp(-K2 / 64.0)
    # make it a transform of a real field and solenoidal
    u = np.fft.irfftn(uh, s=(N, N, N), axes=(1, 2, 3))
    uh = np.fft.rfftn(u, axes=(1, 2, 3)) * mask
    K2n = np.where(K2 == 0, 1, K2)
    uh -= np.sum(K * uh, 0) * K / K2n
    return uh


def main(ref_root):
    script = os.path.join(ref_root, "spectralDNS3D_short.py")
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "mpi4py"))
        open(os.path.join(d, "mpi4py", "__init__.py"), "w").close()
        with open(os.path.join(d, "mpi4py", "MPI.py"), "w") as f:
            f.write(MPI_STUB)
        sys.path.insert(0, d)
        try:
            ns = runpy.run_path(script, run_name="__main__")
        finally:
            sys.path.remove(d)
            for m in [m for m in sys.modules if m.startswith("mpi4py")]:
                del sys.modules[m]
    N = ns["N"]
    U_hat = ns["U_hat"]
    U = ns["U"]
    k = 0.5 * np.sum(U * U) / N ** 3
    idx = np.argwhere(np.abs(U_hat) > 1e-12)
    val = U_hat[tuple(idx.T)]
    seed = 20240531
    ns["U_hat"][:] = random_input(seed, N)
    dU = ns["ComputeRHS"](ns["dU"], 1).copy()
    rng = np.random.default_rng(1)
    ridx = np.stack([rng.integers(0, s, 2048) for s in dU.shape], axis=1)
    rval = dU[tuple(ridx.T)]
    out = os.path.join(HERE, "short64.npz")
    np.savez_compressed(out, tg_k=k, tg_idx=idx.astype(np.int16), tg_val=val,
                        rhs_seed=seed, rhs_idx=ridx.astype(np.int16), rhs_val=rval, N=N)
    print("wrote", out, "k=%.12f" % k, "tg modes", len(idx))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
