"""CPU oracle of the learned-closure LES pieces (TEST INFRASTRUCTURE ONLY).

Float64 NumPy restatements the GPU kernels of spectraldns_gb300/csrc/sdns_les.cu
are checked against.  None of this exists in the reference (the closure is
the benchmark's own LES case); parity for these pieces is against these
definitions:

* box filter of ratio r: block averages of u and of u_i u_j; tau_ij =
  bar(u_i u_j) - bar(u_i) bar(u_j), components (xx, yy, zz, xy, xz, yz);
* periodic 3x3x3 convolution, channels last: y[p, o] = b[o] +
  sum_t sum_i W[t, o, i] x[p + d(t), i], d(t) = (t//9 - 1, (t//3)%3 - 1, t%3 - 1),
  with its data and weight gradients;
* spectral gradient i k_j u_hat_i and the projected SGS force
  -P(i k_j tau_hat_ij) on the shenfun-convention spectra of oracle.ns_ref.
"""
import numpy as np

TAU_IDX = ((0, 3, 4), (3, 1, 5), (4, 5, 2))


def offsets():
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def box_filter(u, r):
    """u: (3, N0, N1, N2) -> ubar (3, n0, n1, n2), tau (n0, n1, n2, 6)."""
    u = np.asarray(u, dtype=np.float64)
    _, N0, N1, N2 = u.shape
    n = (N0 // r, N1 // r, N2 // r)

    def avg(f):
        return f.reshape(n[0], r, n[1], r, n[2], r).mean(axis=(1, 3, 5))
    ub = np.stack([avg(u[i]) for i in range(3)])
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    tau = np.stack([avg(u[i] * u[j]) - ub[i] * ub[j] for i, j in pairs], axis=-1)
    return ub, tau


def conv3d(x, W, b=None):
    """x: (n0, n1, n2, Ci), W: (27, Co, Ci) -> (n0, n1, n2, Co)."""
    x = np.asarray(x, dtype=np.float64)
    W = np.asarray(W, dtype=np.float64)
    y = np.zeros(x.shape[:3] + (W.shape[1],))
    for t, d in enumerate(offsets()):
        xs = np.roll(x, shift=(-d[0], -d[1], -d[2]), axis=(0, 1, 2))  # xs[p] = x[p + d]
        y += xs @ W[t].T
    if b is not None:
        y += np.asarray(b, dtype=np.float64)
    return y


def conv3d_bwd_data(g, W):
    """dL/dx for y = conv3d(x, W): g (n0, n1, n2, Co) -> (n0, n1, n2, Ci)."""
    g = np.asarray(g, dtype=np.float64)
    W = np.asarray(W, dtype=np.float64)
    gx = np.zeros(g.shape[:3] + (W.shape[2],))
    for t, d in enumerate(offsets()):
        gs = np.roll(g, shift=(d[0], d[1], d[2]), axis=(0, 1, 2))  # gs[p] = g[p - d]
        gx += gs @ W[t]
    return gx


def conv3d_bwd_weight(x, g):
    """dL/dW (27, Co, Ci) and dL/db (Co,) for y = conv3d(x, W) + b."""
    x = np.asarray(x, dtype=np.float64)
    g = np.asarray(g, dtype=np.float64)
    Ci, Co = x.shape[-1], g.shape[-1]
    dW = np.zeros((27, Co, Ci))
    for t, d in enumerate(offsets()):
        xs = np.roll(x, shift=(-d[0], -d[1], -d[2]), axis=(0, 1, 2))
        dW[t] = g.reshape(-1, Co).T @ xs.reshape(-1, Ci)
    return dW, g.reshape(-1, Co).sum(axis=0)


def grad_hat(grid, uh):
    """ghat[3 i + j] = i K_j u_hat_i (shenfun-ordered spectra of a oracle.ns_ref.Grid)."""
    return np.stack([1j * grid.K[j] * uh[i] for i in range(3) for j in range(3)])


def sgs_force(grid, tau_hat, scale=1.0):
    """S_i = -i K_j tau_hat_ij, projected on K.S = 0 (mean mode zero)."""
    S = np.stack([-1j * sum(grid.K[j] * tau_hat[TAU_IDX[i][j]] for j in range(3)) * scale for i in range(3)])
    K2 = grid.K2
    K2n = np.where(K2 == 0, 1, K2)
    P = sum(grid.K[i] * S[i] for i in range(3)) / K2n
    for i in range(3):
        S[i] = S[i] - P * grid.K[i]
    S[:, K2 == 0] = 0
    return S
