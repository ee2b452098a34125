"""Coarse-grid LES with a learned subgrid-stress closure (the benchmark's LES case).

Pipeline, every numerical step in libsdns_gb300.so:

1. ``harvest``: a fine DNS (default 512^3, forced isotropic turbulence) is
   box-filtered (ratio r, default 8) every few steps into the coarse velocity
   ubar and the subgrid stress tau_ij = bar(u_i u_j) - bar(u_i) bar(u_j).
2. Features: the 9 velocity gradients of ubar (spectral, on the coarse grid),
   normalised per channel; targets: tau normalised per component.
3. ``ClosureNet``: three periodic 3x3x3 convolutions 9 -> 32 -> 32 -> 6 with
   ReLU, BF16 activations/weights and FP32 accumulation, trained by its own
   forward/backward kernels and Adam on the GPU.
4. ``LES``: the coarse solver (same viscosity and forcing, CFL time step) adds
   the projected SGS force -P(i k_j tau_hat_ij) of the network's stress as a
   Source held constant over each RK4 step.  Without a network it is the plain
   coarse DNS (the fallback and the ablation).
5. ``evaluate``: energy spectra of the LES and of the filtered DNS at the same
   times for k <= kmax, and the GPU time per unit simulated time of both.

torch is used for device buffers only.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
import sys
import time

import numpy as np

from . import _lib
from ._lib import check
from .gpu import Context
from .init import isotropic_field

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

NU, EPS, KF, CFL = 0.0008, 0.1, 2.0, 0.5
CPAD_IN, NOUT, CPAD_OUT = 16, 6, 8
LAYERS = ((CPAD_IN, 32, True), (32, 32, True), (32, CPAD_OUT, False))


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ivec(v):
    return (C.c_int32 * 3)(*[int(x) for x in v])


def _dvec(v):
    return (C.c_double * 3)(*[float(x) for x in v])


class ClosureNet:
    """9 -> 32 -> 32 -> 6 periodic conv net with its own GPU training kernels."""

    def __init__(self, n, seed=0, device=0, lr=1e-3, nin=9):
        self.n = tuple(int(x) for x in n)
        self.P = int(np.prod(self.n))
        self.dev = torch.device("cuda", device)
        self.lr = lr
        self.L = _lib.lib()
        self.nin = nin
        rng = np.random.default_rng(seed)
        sizes = []
        for ci, co, _ in LAYERS:
            sizes += [27 * co * ci, co]
        self.offs = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
        w = np.zeros(self.offs[-1], dtype=np.float32)
        for li, (ci, co, relu) in enumerate(LAYERS):
            fan_in = 27 * (nin if li == 0 else ci)
            std = math.sqrt(2.0 / fan_in) if relu else 0.1 * math.sqrt(1.0 / fan_in)
            Wl = rng.standard_normal((27, co, ci)).astype(np.float32) * std
            if li == 0:
                Wl[:, :, nin:] = 0  # padded input channels
            w[self.offs[2 * li]:self.offs[2 * li + 1]] = Wl.ravel()
        # 4-byte aligned views: pad each segment start (sizes are multiples of 8 already)
        self.w = torch.from_numpy(w).to(self.dev)
        self.g = torch.zeros_like(self.w)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.wb = torch.zeros(self.w.numel(), dtype=torch.bfloat16, device=self.dev)
        check(self.L.sdns_to_bf16(_p(self.w), _p(self.wb), self.w.numel(), _stream()))
        self.step_no = 0
        P = self.P
        f32 = dict(dtype=torch.float32, device=self.dev)
        bf = dict(dtype=torch.bfloat16, device=self.dev)
        self.pre = [torch.empty(P * co, **f32) for _, co, _ in LAYERS]
        self.act = [torch.empty(P * co, **bf) for _, co, _ in LAYERS[:-1]]
        self.gpost = [torch.empty(P * ci, **f32) for ci, _, _ in LAYERS]
        self.gpre = [torch.empty(P * co, **f32) for _, co, _ in LAYERS]
        self.nv = _ivec(self.n)

    def _W(self, li):
        return C.c_void_p(self.wb.data_ptr() + 2 * int(self.offs[2 * li]))

    def _b(self, li, buf=None):
        t = self.w if buf is None else buf
        return C.c_void_p(t.data_ptr() + 4 * int(self.offs[2 * li + 1]))

    def _gW(self, li):
        return C.c_void_p(self.g.data_ptr() + 4 * int(self.offs[2 * li]))

    def forward(self, x):
        """x: bf16 (P, 16) -> FP32 (P, 8) normalised stresses (first 6 used)."""
        inp = x
        for li, (ci, co, relu) in enumerate(LAYERS):
            act = self.act[li] if li < len(LAYERS) - 1 else None
            check(self.L.sdns_conv3d_fwd(_p(inp), self._W(li), self._b(li), _p(self.pre[li]), _p(act), self.nv, ci,
                                         co, 1 if relu else 0, _stream()))
            inp = act
        return self.pre[-1]

    def backward(self, x, gout):
        """Accumulate parameter gradients for dL/d(output) = gout (FP32 (P, 8))."""
        self.g.zero_()
        g = gout
        for li in range(len(LAYERS) - 1, -1, -1):
            ci, co, relu = LAYERS[li]
            check(self.L.sdns_relu_bwd(_p(g), _p(self.pre[li]), _p(self.gpre[li]), self.P * co, 1 if relu else 0,
                                       _stream()))
            inp = x if li == 0 else self.act[li - 1]
            check(self.L.sdns_conv3d_bwd_weight(_p(inp), _p(self.gpre[li]), self._gW(li), self._b(li, self.g),
                                                self.nv, ci, co, _stream()))
            if li > 0:
                check(self.L.sdns_conv3d_bwd_data(_p(self.gpre[li]), self._W(li), _p(self.gpost[li]), self.nv, ci,
                                                  co, _stream()))
                g = self.gpost[li]

    def adam(self):
        self.step_no += 1
        check(self.L.sdns_adam_step(_p(self.w), _p(self.g), _p(self.m), _p(self.v), self.w.numel(), self.lr, 0.9,
                                    0.999, 1e-8, self.step_no, _p(self.wb), _stream()))

    def state_dict(self):
        return {"w": self.w.detach().cpu().numpy(), "offs": self.offs}

    def load(self, w):
        self.w.copy_(torch.from_numpy(np.asarray(w, dtype=np.float32)).to(self.dev))
        check(self.L.sdns_to_bf16(_p(self.w), _p(self.wb), self.w.numel(), _stream()))


class Features:
    """Velocity-gradient features of a coarse spectral velocity, on the GPU."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.n = ctx.N
        self.P = int(np.prod(ctx.N))
        d = torch.device("cuda", ctx.device)
        cdt = torch.complex64 if ctx.precision == "single" else torch.complex128
        self.gh = torch.empty((9,) + ctx.spec_shape[1:], dtype=cdt, device=d)
        self.gphys = torch.empty((9,) + tuple(ctx.N), dtype=torch.float32, device=d)
        self.x = torch.empty((self.P, CPAD_IN), dtype=torch.bfloat16, device=d)
        self.prec = _lib.SDNS_SINGLE if ctx.precision == "single" else _lib.SDNS_DOUBLE
        self.L = _lib.lib()

    def gradients(self, uhat):
        check(self.L.sdns_les_grad_hat(_p(uhat), _p(self.gh), self.prec, _ivec(self.n), _dvec(self.ctx.L), _stream()))
        for c in range(3):
            self.ctx.backward(self.gh[3 * c:3 * c + 3], out=self.gphys[3 * c:3 * c + 3])
        return self.gphys

    def pack(self, planar, mu, isd):
        check(self.L.sdns_les_pack(_p(planar), planar.shape[0], self.P, CPAD_IN, _p(mu), _p(isd), _p(self.x),
                                   _stream()))
        return self.x


def spectrum_of(ctx: Context, uhat):
    """Shell spectrum (demo/Isotropic.py:88-114 convention) of a spectral velocity, via the GPU."""
    ctx.set_state(uhat)
    return ctx.spectrum()


def harvest(n_dns=512, ratio=8, steps=2000, every=10, seed=0, device=0, log=print):
    """Run the forced DNS and box-filter it every `every` steps (config 2 -> config 3 data)."""
    N = (n_dns,) * 3
    nc = n_dns // ratio
    dev = torch.device("cuda", device)
    ctx = Context(N, nu=NU, precision="single", device=device)
    ctx.set_forcing(EPS, KF)
    ctx.set_cfl(CFL)
    ctx.set_state(isotropic_field(N, k0=4.0, energy=0.5, seed=seed, dtype=np.complex64))
    nsnap = (steps + every - 1) // every
    P = nc ** 3
    ubar = torch.empty((nsnap, 3, nc, nc, nc), dtype=torch.float32, device=dev)
    tau = torch.empty((nsnap, P, 6), dtype=torch.float32, device=dev)
    u = torch.empty((3,) + N, dtype=torch.float32, device=dev)
    times = np.zeros(nsnap)
    L = _lib.lib()
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=dev)
    dns_ms = 0.0
    k = 0
    t0 = time.time()
    for s in range(steps):
        if s % every == 0:
            ctx.velocity(out=u)
            check(L.sdns_les_box_filter(_p(u), _lib.SDNS_SINGLE, _ivec(N), ratio, _p(ubar[k]), _p(tau[k]), _stream()))
            times[k] = ctx.diagnostics()["time"]
            k += 1
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.rk4(0.0, 1)
        e1.record(stream)
        e1.synchronize()
        dns_ms += e0.elapsed_time(e1)
        if log and s % 500 == 0:
            d = ctx.diagnostics()
            log("dns step %d t=%.4f E=%.5f dt=%.2e (%.0f s)" % (s, d["time"], d["energy"], d["last_dt"],
                                                                  time.time() - t0))
    t_end = ctx.diagnostics()["time"]
    ctx.close()
    torch.cuda.synchronize()
    return {"ubar": ubar, "tau": tau, "times": times, "dns_gpu_ms": dns_ms, "dns_time": t_end, "n_dns": n_dns,
            "ratio": ratio, "steps": steps}


class LES:
    """Coarse solver with an optional learned closure."""

    def __init__(self, n, net: ClosureNet | None, norms=None, device=0, scale=1.0):
        self.scale = float(scale)  # amplitude of the subgrid force (calibrated a posteriori)
        self.ctx = Context(n, nu=NU, precision="single", device=device)
        self.ctx.set_forcing(EPS, KF)
        self.ctx.set_cfl(CFL)
        self.net = net
        self.norms = norms
        self.dev = torch.device("cuda", device)
        self.feat = Features(self.ctx)
        self.uhat = torch.empty(self.ctx.spec_shape, dtype=torch.complex64, device=self.dev)
        self.tau = torch.empty((6,) + tuple(n), dtype=torch.float32, device=self.dev)
        self.tauhat = torch.empty((6,) + self.ctx.spec_shape[1:], dtype=torch.complex64, device=self.dev)
        self.force = torch.empty(self.ctx.spec_shape, dtype=torch.complex64, device=self.dev)
        self.L = _lib.lib()
        # the closure's kernels run on the context stream, so one LES step needs no host
        # synchronisation between the network, the transforms and the RK4 step
        self.stream = torch.cuda.ExternalStream(self.ctx.stream_handle(), device=self.dev)

    def set_velocity_phys(self, ubar):
        """Start from a filtered velocity, truncated to the modes the LES keeps (2/3 rule)."""
        self.ctx.set_state(self.ctx.forward(ubar) * dealias_mask(self.ctx))

    def closure_source(self):
        nm = self.norms
        self.stream.wait_stream(torch.cuda.current_stream(self.dev))  # weights and norms come from torch's stream
        self.ctx.ordered = True
        try:
            with torch.cuda.stream(self.stream):
                self.ctx.get_state(out=self.uhat)
                g = self.feat.gradients(self.uhat)
                x = self.feat.pack(g.reshape(9, -1), nm["fmu"], nm["fisd"])
                y = self.net.forward(x)
                check(self.L.sdns_les_unpack(_p(y), CPAD_OUT, NOUT, self.feat.P, _p(nm["tmu"]), _p(nm["tsd"]),
                                             _p(self.tau), _stream()))
                self.ctx.forward(self.tau[0:3], out=self.tauhat[0:3])
                self.ctx.forward(self.tau[3:6], out=self.tauhat[3:6])
                check(self.L.sdns_les_sgs_force(_p(self.tauhat), _p(self.force), _lib.SDNS_SINGLE,
                                                _ivec(self.ctx.N), _dvec(self.ctx.L), self.scale, _stream()))
                self.ctx.set_source(self.force)
        finally:
            self.ctx.ordered = False

    def step(self):
        if self.net is not None:
            self.closure_source()
        self.ctx.rk4(0.0, 1)

    def time(self):
        return self.ctx.diagnostics()["time"]


def normalisers(feat_all, tau_all):
    """Per-channel mean / std of the features (9, .) and targets (., 6)."""
    fmu = feat_all.mean(dim=(0, 2))
    fsd = feat_all.std(dim=(0, 2)) + 1e-12
    tmu = tau_all.mean(dim=(0, 1))
    tsd = tau_all.std(dim=(0, 1)) + 1e-12
    return {"fmu": fmu.float().contiguous(), "fisd": (1.0 / fsd).float().contiguous(), "tmu": tmu.float().contiguous(),
            "tsd": tsd.float().contiguous()}


def dealias_mask(ctx: Context):
    """2/3-rule mask of the full spectral array of a coarse context (the modes the LES keeps)."""
    from .init import dealias_cutoff
    d = torch.device("cuda", ctx.device)
    n0, n1, n2 = ctx.N
    kc = [dealias_cutoff(n) for n in ctx.N]
    k0 = torch.fft.fftfreq(n0, 1.0 / n0).to(d).abs()
    k1 = torch.fft.fftfreq(n1, 1.0 / n1).to(d).abs()
    k2 = torch.arange(n2 // 2 + 1, device=d, dtype=torch.float32)
    return (k0[:, None, None] <= kc[0]) & (k1[None, :, None] <= kc[1]) & (k2[None, None, :] <= kc[2])


def make_training_set(data, ctx64, train_idx):
    """Gradient features (bf16, channels last) and normalised targets of the training snapshots.

    The LES holds only the 2/3-rule modes of the filtered field, so the features are the
    gradients of the truncated filtered velocity T(ubar), and the target stress adds to the
    box-filter stress the stress of the truncated filtered modes themselves:
    tau_ij + ubar_i ubar_j - T(ubar)_i T(ubar)_j."""
    feat = Features(ctx64)
    dev = data["ubar"].device
    nc = ctx64.N
    P = int(np.prod(nc))
    mask = dealias_mask(ctx64)
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    G = torch.empty((len(train_idx), 9, P), dtype=torch.float32, device=dev)
    T = torch.empty((len(train_idx), P, 6), dtype=torch.float32, device=dev)
    for a, i in enumerate(train_idx):
        ub = data["ubar"][i]
        uh = ctx64.forward(ub) * mask
        ut = ctx64.backward(uh)
        G[a] = feat.gradients(uh).reshape(9, P)
        tr = torch.stack([(ub[p] * ub[q] - ut[p] * ut[q]).reshape(P) for p, q in pairs], dim=1)
        T[a] = data["tau"][i] + tr
    nm = normalisers(G, T)
    X = torch.empty((len(train_idx), P, CPAD_IN), dtype=torch.bfloat16, device=dev)
    for a in range(len(train_idx)):
        X[a] = feat.pack(G[a], nm["fmu"], nm["fisd"])
    Tn = ((T - nm["tmu"]) / nm["tsd"]).contiguous()
    return X, Tn, nm


def train(net: ClosureNet, X, Tn, iters=1500, log=print, seed=0, cosine=True):
    """Adam on random training snapshots; the learning rate decays from net.lr to 1% of it
    along a cosine when `cosine` is set."""
    rng = np.random.default_rng(seed)
    lr0 = net.lr
    L = _lib.lib()
    loss = torch.zeros(1, dtype=torch.float64, device=net.dev)
    grad = torch.empty((net.P, CPAD_OUT), dtype=torch.float32, device=net.dev)
    hist = []
    t0 = time.time()
    for it in range(iters):
        if cosine:
            net.lr = lr0 * (0.01 + 0.99 * 0.5 * (1.0 + math.cos(math.pi * it / max(iters - 1, 1))))
        i = int(rng.integers(0, X.shape[0]))
        y = net.forward(X[i])
        loss.zero_()
        check(L.sdns_mse_grad(_p(y), CPAD_OUT, NOUT, _p(Tn[i]), net.P, _p(grad), _p(loss), _stream()))
        net.backward(X[i], grad)
        net.adam()
        if it % 50 == 0 or it == iters - 1:
            hist.append((it, float(loss.item())))
            if log and it % 250 == 0:
                log("train it %d loss %.4f (%.1f s)" % (it, hist[-1][1], time.time() - t0))
    torch.cuda.synchronize()
    net.lr = lr0
    return hist, time.time() - t0


def spectrum_error(E, Eref, kmax=20):
    kmax = min(kmax, len(E) - 1)
    k = np.arange(1, kmax + 1)
    idx = k - 1  # bin i holds i+0.5 < |k| <= i+1.5, i.e. shell k = i+1
    return float(np.max(np.abs(E[idx] - Eref[idx]) / np.maximum(Eref[idx], 1e-300)))


def spectrum_errors_k(E, Eref, kmax=20):
    kmax = min(kmax, len(E) - 1)
    idx = np.arange(kmax)
    return (np.abs(E[idx] - Eref[idx]) / np.maximum(Eref[idx], 1e-300)).tolist()


def run_les(data, net, nm, start, stop, nc, scale=1.0, device=0, scratch=None):
    """LES from filtered-DNS snapshot `start` to snapshot `stop - 1`; the spectrum error against the
    filtered DNS at every snapshot in between."""
    n = (nc,) * 3
    times = data["times"]
    scratch = scratch or Context(n, nu=NU, precision="single", device=device)
    les = LES(n, net, nm, device=device, scale=scale)
    les.set_velocity_phys(data["ubar"][start])
    les.ctx.set_time(times[start])
    errs = []
    gpu_s = 0.0
    nsteps = 0
    ok = True
    E = Eref = None
    Esum = Erefsum = 0.0
    for j in range(start + 1, stop):
        while les.time() < times[j] - 1e-12:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            les.step()
            les.ctx.synchronize()
            gpu_s += time.perf_counter() - t0
            nsteps += 1
        E = les.ctx.spectrum()
        if not np.all(np.isfinite(E)):
            ok = False
            break
        Eref = spectrum_of(scratch, scratch.forward(data["ubar"][j]))
        errs.append(spectrum_error(E, Eref))
        Esum = Esum + E
        Erefsum = Erefsum + Eref
    les_time = les.time() - times[start]
    les.ctx.close()
    avg_ok = ok and len(errs) > 0
    return {"max_err_k<=20_final": errs[-1] if (errs and ok) else float("inf"),
            "max_err_k<=20_mean": float(np.mean(errs)) if (errs and ok) else float("inf"),
            "max_err_k<=20_time_avg_spectrum": spectrum_error(Esum, Erefsum) if avg_ok else float("inf"),
            "err_k_time_avg": spectrum_errors_k(Esum, Erefsum) if avg_ok else None,
            "finite": ok, "steps": nsteps, "sim_time": les_time, "wall_s": gpu_s,
            "s_per_sim_time": gpu_s / max(les_time, 1e-30), "scale": scale,
            "err_k_final": spectrum_errors_k(E, Eref) if (ok and E is not None) else None,
            "spectrum_final": E[:22].tolist() if (ok and E is not None) else None,
            "reference_final": Eref[:22].tolist() if Eref is not None else None}


def calibrate(data, net, nm, start, stop, nc, scales, device=0, log=print):
    """A-posteriori amplitude of the subgrid force: the scale whose LES over training snapshots
    [start, stop) has the lowest error of the time-averaged spectrum (ties: lowest mean error)."""
    scratch = Context((nc,) * 3, nu=NU, precision="single", device=device)
    table = []
    for sc in scales:
        r = run_les(data, net, nm, start, stop, nc, scale=sc, device=device, scratch=scratch)
        table.append((sc, r["max_err_k<=20_time_avg_spectrum"], r["max_err_k<=20_mean"], r["max_err_k<=20_final"]))
        if log:
            log("calibrate scale %.2f: time-avg spectrum err %.3f mean err %.3f final err %.3f" % table[-1])
    best = min(table, key=lambda t: (t[1], t[2]))
    return best[0], table


def evaluate(data, net, nm, start, nc, device=0, log=print, scale=1.0):
    """LES with the calibrated closure, the uncalibrated closure and no closure from filtered-DNS
    snapshot `start` to the last one, compared with the filtered DNS."""
    stop = len(data["times"])
    res = {}
    for name, use, sc in (("closure", True, scale), ("closure_scale1", True, 1.0), ("no_closure", False, 1.0)):
        res[name] = run_les(data, net if use else None, nm, start, stop, nc, scale=sc, device=device)
        if log:
            log("%s (scale %.2f): final err %.3f mean err %.3f time-avg spectrum err %.3f steps %d" % (
                name, sc, res[name]["max_err_k<=20_final"], res[name]["max_err_k<=20_mean"],
                res[name]["max_err_k<=20_time_avg_spectrum"], res[name]["steps"]))
    return res


SCALES = (0.6, 0.8, 0.9, 1.0, 1.1, 1.2, 1.35, 1.5, 2.0, 3.0)


def run_experiment(out_json, n_dns=512, ratio=8, steps=2000, every=10, iters=3000, train_frac=0.75, log=print,
                   scales=SCALES):
    data = harvest(n_dns, ratio, steps, every, log=log)
    nc = n_dns // ratio
    nsnap = data["ubar"].shape[0]
    ntrain = int(nsnap * train_frac)
    ctx64 = Context((nc,) * 3, nu=NU, precision="single")
    X, Tn, nm = make_training_set(data, ctx64, list(range(ntrain)))
    net = ClosureNet((nc,) * 3, seed=0)
    hist, train_s = train(net, X, Tn, iters=iters, log=log)
    # amplitude calibration on the last 50 training snapshots (never on the evaluated ones)
    c0 = max(0, ntrain - 50)
    scale, table = calibrate(data, net, nm, c0, ntrain, nc, scales, log=log)
    ev = evaluate(data, net, nm, ntrain, nc, log=log, scale=scale)
    dns_s_per_time = data["dns_gpu_ms"] / 1e3 / max(data["dns_time"], 1e-30)
    out = {"n_dns": n_dns, "n_les": nc, "ratio": ratio, "dns_steps": steps, "snapshots": nsnap, "train_snapshots": ntrain,
           "train_iters": iters, "train_loss_first": hist[0][1], "train_loss_last": hist[-1][1], "train_s": train_s,
           "calibration": {"snapshots": [c0, ntrain], "scale": scale, "table": table},
           "dns_gpu_s_per_sim_time": dns_s_per_time, "evaluation": ev,
           "speedup_gpu_seconds": dns_s_per_time / ev["closure"]["s_per_sim_time"],
           "speedup_no_closure": dns_s_per_time / ev["no_closure"]["s_per_sim_time"]}
    with open(out_json, "w") as f:
        json.dump(out, f, indent=1)
    save_model(os.path.splitext(out_json)[0] + "_model.npz", net, nm, scale)
    return out


def evaluate_model(out_json, model, n_dns=512, ratio=8, steps=2000, every=10, train_frac=0.75, log=print):
    """The held-out evaluation of run_experiment with saved weights: the DNS trajectory is
    deterministic, so it is regenerated, and the LES with and without the closure is run and
    timed again on the snapshots after the training window."""
    data = harvest(n_dns, ratio, steps, every, log=log)
    nc = n_dns // ratio
    ntrain = int(data["ubar"].shape[0] * train_frac)
    net, nm, scale = load_model(model, (nc,) * 3)
    ev = evaluate(data, net, nm, ntrain, nc, log=log, scale=scale)
    dns_s_per_time = data["dns_gpu_ms"] / 1e3 / max(data["dns_time"], 1e-30)
    out = {"n_dns": n_dns, "n_les": nc, "ratio": ratio, "dns_steps": steps, "snapshots": int(data["ubar"].shape[0]),
           "train_snapshots": ntrain, "model": os.path.basename(model), "scale": scale,
           "dns_gpu_s_per_sim_time": dns_s_per_time, "evaluation": ev,
           "speedup_gpu_seconds": dns_s_per_time / ev["closure"]["s_per_sim_time"],
           "speedup_no_closure": dns_s_per_time / ev["no_closure"]["s_per_sim_time"]}
    with open(out_json, "w") as f:
        json.dump(out, f, indent=1)
    return out


def save_model(path, net, nm, scale=1.0):
    np.savez(path, w=net.state_dict()["w"], scale=np.float64(scale), **{k: v.cpu().numpy() for k, v in nm.items()})


def load_model(path, n, device=0):
    """(net, normalisers, calibrated subgrid-force scale) of a saved closure."""
    d = np.load(path)
    net = ClosureNet(n, device=device)
    net.load(d["w"])
    dev = torch.device("cuda", device)
    nm = {k: torch.from_numpy(d[k]).to(dev) for k in ("fmu", "fisd", "tmu", "tsd")}
    scale = float(d["scale"]) if "scale" in d.files else 1.0
    return net, nm, scale


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="les_results.json")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--ratio", type=int, default=8)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--evaluate", default=None, metavar="MODEL",
                    help="only re-run the held-out evaluation with these saved weights")
    a = ap.parse_args()
    if a.evaluate:
        r = evaluate_model(a.out, a.evaluate, a.n, a.ratio, a.steps, a.every, log=lambda s: print(s, flush=True))
    else:
        r = run_experiment(a.out, a.n, a.ratio, a.steps, a.every, a.iters, log=lambda s: print(s, flush=True))
    print(json.dumps({k: v for k, v in r.items() if k != "evaluation"}))
    print(json.dumps(r["evaluation"]))
