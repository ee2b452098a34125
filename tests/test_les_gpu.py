"""Learned-closure kernels against the CPU oracle (oracle/les_ref.py).

Tolerances: FP32-accumulated convolutions of BF16-exact inputs agree with the
float64 oracle to 2e-5 relative (of the largest output); box filter and
spectral operators to 1e-6 (FP32 data); gradients of the whole network to
1e-4 relative.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import les_ref
from oracle.ns_ref import Grid

pytestmark = pytest.mark.gpu


def _bf16_exact(a):
    """Round float32 values to the nearest bfloat16 (as float32)."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32)


def _t(a, dtype=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.to("cuda:0")


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def _ok(rc):
    from spectraldns_gb300 import _lib
    assert rc == 0, _lib.lib().sdns_last_error()


def test_box_filter(built_lib):
    import torch
    from spectraldns_gb300 import _lib
    from spectraldns_gb300.les import _p, _ivec, _stream
    rng = np.random.default_rng(0)
    u = rng.standard_normal((3, 32, 32, 32)).astype(np.float32)
    ub_ref, tau_ref = les_ref.box_filter(u, 4)
    ub = torch.empty((3, 8, 8, 8), dtype=torch.float32, device="cuda:0")
    tau = torch.empty((8 * 8 * 8, 6), dtype=torch.float32, device="cuda:0")
    _ok(built_lib.sdns_les_box_filter(_p(_t(u)), _lib.SDNS_SINGLE, _ivec((32, 32, 32)), 4, _p(ub), _p(tau), _stream()))
    torch.cuda.synchronize()
    assert _rel(ub.cpu().numpy(), ub_ref) < 1e-6
    assert _rel(tau.cpu().numpy(), tau_ref.reshape(-1, 6)) < 1e-6
    # tau of a box filter is positive semi-definite on the diagonal
    assert tau.cpu().numpy()[:, :3].min() >= -1e-6


def test_grad_and_sgs_force(built_lib):
    import torch
    from spectraldns_gb300 import _lib
    from spectraldns_gb300.les import _p, _ivec, _dvec, _stream
    N, L = (16, 32, 16), (2 * np.pi, 4 * np.pi, 2 * np.pi)
    g = Grid(N, L)
    rng = np.random.default_rng(1)
    uh = g.forward(rng.standard_normal((3,) + N))
    th = g.forward(rng.standard_normal((6,) + N))
    gh = torch.empty((9,) + g.spec_shape, dtype=torch.complex128, device="cuda:0")
    _ok(built_lib.sdns_les_grad_hat(_p(_t(uh)), _p(gh), _lib.SDNS_DOUBLE, _ivec(N), _dvec(L), _stream()))
    F = torch.empty((3,) + g.spec_shape, dtype=torch.complex128, device="cuda:0")
    _ok(built_lib.sdns_les_sgs_force(_p(_t(th)), _p(F), _lib.SDNS_DOUBLE, _ivec(N), _dvec(L), 1.0, _stream()))
    torch.cuda.synchronize()
    assert _rel(gh.cpu().numpy(), les_ref.grad_hat(g, uh)) < 1e-13
    S = les_ref.sgs_force(g, th)
    assert _rel(F.cpu().numpy(), S) < 1e-13
    assert np.max(np.abs(sum(g.K[i] * F.cpu().numpy()[i] for i in range(3)))) < 1e-10  # solenoidal


@pytest.mark.parametrize("ci,co", [(16, 32), (32, 32), (32, 8)])
def test_conv_forward_backward(built_lib, ci, co):
    import torch
    from spectraldns_gb300.les import _p, _ivec, _stream
    n = (16, 8, 24)
    rng = np.random.default_rng(ci + co)
    x = _bf16_exact(rng.standard_normal(n + (ci,)))
    W = _bf16_exact(rng.standard_normal((27, co, ci)) * 0.2)
    b = rng.standard_normal(co).astype(np.float32)
    y_ref = les_ref.conv3d(x, W, b)
    xd, Wd = _t(x, torch.bfloat16), _t(W, torch.bfloat16)
    y = torch.empty(n + (co,), dtype=torch.float32, device="cuda:0")
    ya = torch.empty(n + (co,), dtype=torch.bfloat16, device="cuda:0")
    _ok(built_lib.sdns_conv3d_fwd(_p(xd), _p(Wd), _p(_t(b)), _p(y), _p(ya), _ivec(n), ci, co, 1, _stream()))
    torch.cuda.synchronize()
    assert _rel(y.cpu().numpy(), y_ref) < 2e-5
    assert _rel(ya.float().cpu().numpy(), np.maximum(y_ref, 0)) < 1e-2  # bf16 activation copy
    g = rng.standard_normal(n + (co,)).astype(np.float32)
    gin = torch.empty(n + (ci,), dtype=torch.float32, device="cuda:0")
    _ok(built_lib.sdns_conv3d_bwd_data(_p(_t(g)), _p(Wd), _p(gin), _ivec(n), ci, co, _stream()))
    dW = torch.zeros((27, co, ci), dtype=torch.float32, device="cuda:0")
    db = torch.zeros(co, dtype=torch.float32, device="cuda:0")
    _ok(built_lib.sdns_conv3d_bwd_weight(_p(xd), _p(_t(g)), _p(dW), _p(db), _ivec(n), ci, co, _stream()))
    torch.cuda.synchronize()
    assert _rel(gin.cpu().numpy(), les_ref.conv3d_bwd_data(g, W)) < 2e-5
    dW_ref, db_ref = les_ref.conv3d_bwd_weight(x, g)
    assert _rel(dW.cpu().numpy(), dW_ref) < 2e-5
    assert _rel(db.cpu().numpy(), db_ref) < 2e-5


def test_network_gradient_against_oracle(built_lib):
    """Whole-network parameter gradients of the MSE loss vs float64 backprop on the CPU."""
    import torch
    from spectraldns_gb300.les import ClosureNet, LAYERS, CPAD_OUT, NOUT, _p, _stream
    n = (8, 16, 8)
    P = int(np.prod(n))
    net = ClosureNet(n, seed=3)
    rng = np.random.default_rng(5)
    x = _bf16_exact(rng.standard_normal((P, 16)))
    x[:, 9:] = 0
    tgt = rng.standard_normal((P, NOUT)).astype(np.float32)
    xd = _t(x, torch.bfloat16)
    y = net.forward(xd)
    grad = torch.empty((P, CPAD_OUT), dtype=torch.float32, device="cuda:0")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    _ok(built_lib.sdns_mse_grad(_p(y), CPAD_OUT, NOUT, _p(_t(tgt)), P, _p(grad), _p(loss), _stream()))
    net.backward(xd, grad)
    torch.cuda.synchronize()
    # oracle backpropagation with the same BF16 weights and the same BF16 activations the GPU
    # forward produced (a different FP32 summation order may round an activation to the
    # neighbouring BF16 value; the forward itself is checked in test_conv_forward_backward)
    w = net.wb.float().cpu().numpy()
    Ws, bs = [], []
    for li, (ci, co, _) in enumerate(LAYERS):
        Ws.append(w[net.offs[2 * li]:net.offs[2 * li + 1]].reshape(27, co, ci))
        bs.append(net.w.cpu().numpy()[net.offs[2 * li + 1]:net.offs[2 * li + 2]])
    a0 = x.reshape(n + (16,)).astype(np.float64)
    pre1 = net.pre[0].cpu().numpy().reshape(n + (32,)).astype(np.float64)
    a1 = net.act[0].float().cpu().numpy().reshape(n + (32,)).astype(np.float64)
    pre2 = net.pre[1].cpu().numpy().reshape(n + (32,)).astype(np.float64)
    a2 = net.act[1].float().cpu().numpy().reshape(n + (32,)).astype(np.float64)
    assert np.max(np.abs(pre1 - les_ref.conv3d(a0, Ws[0], bs[0]))) < 2e-5 * np.max(np.abs(pre1))
    assert np.max(np.abs(pre2 - les_ref.conv3d(a1, Ws[1], bs[1]))) < 2e-5 * np.max(np.abs(pre2))
    pre3 = les_ref.conv3d(a2, Ws[2], bs[2])
    d = np.zeros_like(pre3)
    d[..., :NOUT] = pre3[..., :NOUT] - tgt.reshape(n + (NOUT,))
    L_ref = np.mean(d[..., :NOUT] ** 2)
    g3 = 2 * d / (P * NOUT)
    dW3, db3 = les_ref.conv3d_bwd_weight(a2, g3)
    g2 = les_ref.conv3d_bwd_data(g3, Ws[2]) * (pre2 > 0)
    dW2, db2 = les_ref.conv3d_bwd_weight(a1, g2)
    g1 = les_ref.conv3d_bwd_data(g2, Ws[1]) * (pre1 > 0)
    dW1, db1 = les_ref.conv3d_bwd_weight(a0, g1)
    gd = net.g.cpu().numpy()
    ref = [dW1, db1, dW2, db2, dW3, db3]
    assert abs(loss.item() - L_ref) / L_ref < 1e-5
    for k, r in enumerate(ref):
        got = gd[net.offs[k]:net.offs[k + 1]].reshape(r.shape)
        assert _rel(got, r) < 1e-4, k


def test_adam_step(built_lib):
    import torch
    from spectraldns_gb300.les import _p, _stream
    rng = np.random.default_rng(2)
    w = rng.standard_normal(1000).astype(np.float32)
    g = rng.standard_normal(1000).astype(np.float32)
    wd, gd = _t(w), _t(g)
    m = torch.zeros(1000, device="cuda:0")
    v = torch.zeros(1000, device="cuda:0")
    wb = torch.zeros(1000, dtype=torch.bfloat16, device="cuda:0")
    for step in (1, 2):
        _ok(built_lib.sdns_adam_step(_p(wd), _p(gd), _p(m), _p(v), 1000, C.c_float(1e-2), C.c_float(0.9),
                                     C.c_float(0.999), C.c_float(1e-8), step, _p(wb), _stream()))
    torch.cuda.synchronize()
    mr = vr = 0
    wr = w.astype(np.float64)
    for step in (1, 2):
        mr = 0.9 * mr + 0.1 * g
        vr = 0.999 * vr + 0.001 * g * g
        wr = wr - 1e-2 * (mr / (1 - 0.9 ** step)) / (np.sqrt(vr / (1 - 0.999 ** step)) + 1e-8)
    assert np.max(np.abs(wd.cpu().numpy() - wr)) < 1e-5
    assert np.max(np.abs(wb.float().cpu().numpy() - wd.cpu().numpy())) < 1e-2


def test_training_reduces_loss(built_lib):
    """The kernels learn a smooth stencil map of their inputs."""
    import torch
    from spectraldns_gb300.les import ClosureNet, train, CPAD_IN
    n = (16, 16, 16)
    P = 16 ** 3
    rng = np.random.default_rng(0)
    X = np.zeros((4, P, CPAD_IN), dtype=np.float32)
    X[..., :9] = rng.standard_normal((4, P, 9))
    Wt = rng.standard_normal((27, 6, 9)) * 0.1
    T = np.stack([les_ref.conv3d(X[i, :, :9].reshape(n + (9,)), Wt).reshape(P, 6) for i in range(4)])
    Xd = _t(_bf16_exact(X), torch.bfloat16)
    Td = _t(T.astype(np.float32))
    net = ClosureNet(n, seed=1, lr=3e-3)
    hist, _ = train(net, Xd, Td, iters=300, log=None)
    assert hist[-1][1] < 0.2 * hist[0][1], hist[::3]
