#!/usr/bin/env python
"""Benchmark of the pseudo-spectral Navier-Stokes RK4 step on one GB300.

Workload (the 512^3 case of the headline metric "RK4 steps/s at 512^3 FP32 vs
FP64"): forced isotropic turbulence on a 512^3 grid in [0, 2pi)^3, seeded
solenoidal initial field with E(k) ~ k^4 exp(-2 (k/4)^2) and total energy
0.5, constant-power forcing eps = 0.1 on |k| <= 2, nu = 8e-4, RK4 with CFL
0.5 (dt from the velocity maximum at every step start), 2/3-rule dealiasing.
A "step" is one RK4 step (four right-hand-side evaluations).  All inputs are
synthetic (generated from the seed) and larger than L2 (the state alone is
1.6 GB), so no L2 flush is needed between steps.

Arms:
  python bench.py [--gpus N --steps K --warmup W]          this library
  python bench.py --impl reference [...]                   CPU float32 NumPy/scipy.fft
      restatement of the reference path (the oracle port) on all host cores
Under torchrun each rank runs an independent replica on its own GPU
(replicas only; the whole-job value is the sum of the replicas' steps/s).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK4 steps/s at 512^3 FP32 vs FP64; closure-LES speedup at spectrum err <=5%"
WORKLOAD = ("forced isotropic turbulence 512^3 FP32 (seeded k^4 exp(-2(k/4)^2) field, E=0.5, "
            "eps=0.1 forcing on |k|<=2, nu=8e-4, RK4 CFL 0.5, 2/3 rule)")
NU, EPS, KF, CFL, K0 = 0.0008, 0.1, 2.0, 0.5, 4.0
KERNEL_NAMES = ["x_inv_curl", "y_inv", "z_c2r_cross_r2c", "y_fwd", "x_fwd", "rk_update"]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=("ours", "reference"))
    p.add_argument("--n", type=int, default=512)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-les", action="store_true", help="skip the closure-LES timing")
    p.add_argument("--no-1024", action="store_true", help="skip the 1024^3 decaying-turbulence timing")
    p.add_argument("--no-pad32", action="store_true", help="skip the 3/2-rule timing")
    p.add_argument("--no-cufft", action="store_true", help="skip the same-GPU cuFFT (torch.fft) comparison")
    p.add_argument("--precision", default="single", choices=("single", "double"),
                   help="precision of the main workload (profiling the FP64 kernels); the headline is single")
    p.add_argument("--grid", default=None,
                   help="N0,N1,N2: run the workload on this (small, profiling) grid instead of --n cubed")
    p.add_argument("--decay1024-steps", type=int, default=0, dest="decay1024_steps",
                   help="only run the 1024^3 decaying-turbulence case for this many RK4 steps with FP64 energy and "
                        "dissipation every step, and print its energy budget")
    p.add_argument("--tg256", action="store_true",
                   help="only run the 256^3 Taylor-Green FP32-vs-FP64 comparison (1000 steps) and print it")
    return p.parse_args()


def max_over_ranks(x, ws, device):
    """The largest of the ranks' values (the job's time is its slowest rank's); x itself when ws == 1.
    device: where the reduction tensor lives ("cuda:<i>" for NCCL, "cpu" for gloo)."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if ws > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = os.path.join("/tmp", "sdns_clocks_%d_%d.csv" % (os.getpid(), gpu_index))
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(gpu_index)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic bytes per launch of each kernel class (FP32 state, FP64 RK4 accumulators)
# ---------------------------------------------------------------------------
def kernel_bytes(N, csz=8, acc=16):
    """Algorithmic HBM bytes per launch of each kernel class of one RK4 stage on grid N (an int
    for a cubic grid): every input read once, every output written once."""
    from spectraldns_gb300.init import dealias_cutoff
    n0, n1, n2 = (N, N, N) if isinstance(N, int) else tuple(N)
    K0 = 2 * dealias_cutoff(n0) + 1
    K1 = 2 * dealias_cutoff(n1) + 1
    Kz = dealias_cutoff(n2) + 1
    Kzp = (Kz + 7) // 8 * 8
    comp = K0 * K1 * Kzp        # one compact component
    a1 = n0 * K1 * Kzp          # one field after the first inverse axis
    a2 = n0 * n1 * Kzp          # one field after the second inverse axis
    rk_state = comp * 3 * ((acc + csz + acc) + 2 * (csz + 3 * acc + csz) + (csz + 2 * acc + csz)) / 4.0
    return {
        "x_inv_curl": 3 * comp * csz + 6 * a1 * csz,
        "y_inv": 6 * a1 * csz + 6 * a2 * csz,
        "z_c2r_cross_r2c": 6 * n0 * n1 * Kz * csz + 3 * a2 * csz,
        "y_fwd": 3 * a2 * csz + 3 * a1 * csz,
        "x_fwd": 3 * a1 * csz + 3 * comp * csz,
        "rk_update": 3 * comp * csz + rk_state,
    }


def run_ours(args):
    import torch
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    dev = local
    n = args.n
    N = tuple(int(x) for x in args.grid.split(",")) if args.grid else (n, n, n)
    dbl = args.precision == "double"
    uh0 = isotropic_field(N, k0=K0, energy=0.5, seed=0, dtype=np.complex128 if dbl else np.complex64)
    ctx = Context(N, nu=NU, precision=args.precision, device=dev)
    ctx.set_forcing(EPS, KF)
    ctx.set_cfl(CFL)
    ctx.set_state(uh0)
    for _ in range(args.warmup):
        ctx.rk4(0.0, 1)
    ctx.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", dev))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.set_timing(True)
    t_start = ctx.diagnostics()["time"]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clk = Clocks(dev)
    e0.record(stream)
    ctx.rk4(0.0, args.steps)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    clocks = clk.stop()
    if ws > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1)
    ktimes, klaunch = ctx.get_timing()
    ctx.set_timing(False)
    diag = ctx.diagnostics()
    dns_s_per_sim_time = (ms / 1e3) / max(diag["time"] - t_start, 1e-30)
    ms_max = max_over_ranks(ms, ws, "cuda:%d" % dev)
    value = ws * args.steps / (ms_max / 1e3)

    # per-kernel roofline
    kb = kernel_bytes(N, csz=16 if dbl else 8)
    peak, peak_src = peaks()
    kernels = {}
    for i, name in enumerate(KERNEL_NAMES):
        if klaunch[i] == 0:
            continue
        per = ktimes[i] / klaunch[i]
        kernels[name] = {"ms_per_launch": per, "launches": klaunch[i], "share": ktimes[i] / max(sum(ktimes), 1e-30),
                         "alg_bytes": kb[name], "gbs": kb[name] / (per * 1e-3) / 1e9}
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_launch"] * kernels[k]["launches"])
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            tr = json.load(f)
        if str(n) in tr and dom in tr[str(n)] and not dbl and not args.grid:
            traffic = tr[str(n)][dom]
    except Exception:
        pass
    step_bytes = sum(kernels[k]["alg_bytes"] * kernels[k]["launches"] for k in kernels) / args.steps
    roofline = {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kernels[dom]["gbs"] / peak, "traffic": traffic, "peak_source": peak_src,
                "step_alg_bytes": step_bytes,
                "step_achieved_gbs": step_bytes / (ms / args.steps * 1e-3) / 1e9}
    roofline["step_frac"] = roofline["step_achieved_gbs"] / peak
    # the same step against the full-spectral-array byte model 4 (27 + 9a) F per step,
    # F = 8 N0 N1 (N2/2+1): a = 2 for 16-byte accumulators (the library's compensated FP32 S, A),
    # a = 1 for 8-byte ones; the library stores only the kept modes and moves fewer bytes
    F = 8.0 * N[0] * N[1] * (N[2] // 2 + 1)
    t_step = ms / args.steps * 1e-3
    roofline["full_array_model"] = {
        "bytes_per_step_a2": 4 * (27 + 18) * F, "frac_a2": 4 * (27 + 18) * F / t_step / 1e9 / peak,
        "bytes_per_step_a1": 4 * (27 + 9) * F, "frac_a1": 4 * (27 + 9) * F / t_step / 1e9 / peak}
    launches = sum(klaunch) + args.steps * 3  # + step-begin, CFL dt and step-end kernels

    out = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64" if dbl else "f32",
           "data": "synthetic (seeded spectrum, generated on the host; no dataset)",
           "config": {"workload": WORKLOAD if not dbl else WORKLOAD.replace("FP32", "FP64"), "grid": list(N),
                      "precision": "double (everything FP64)" if dbl else "single (FP32 transforms, compensated "
                      "FP32 RK4 accumulators, FP64 reductions)", "l2": "inputs larger than L2 (1.6 GB state), no flush",
                      "parallelism": "replicas" if ws > 1 else "single GPU",
                      "timing": "CUDA events on the solver stream; per-kernel events in the same region"},
           "roofline": roofline, "kernels": kernels, "gpu_launches": launches, "clocks": clocks,
           "final_energy": diag["energy"], "final_time": diag["time"]}

    # end to end through the public API with pinned host buffers
    if not args.no_e2e:
        ke = max(3, min(args.steps, 10))
        shape = ctx.spec_shape
        cdt = torch.complex128 if dbl else torch.complex64
        hin = torch.empty(shape, dtype=cdt, pin_memory=True)
        hout = torch.empty(shape, dtype=cdt, pin_memory=True)
        hin.numpy()[...] = uh0
        ctx.set_state(hin)
        ctx.rk4(0.0, 1)
        ctx.get_state(hout)
        if ws > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(ke):
            ctx.set_state(hin)       # host -> device: this step's input state
            ctx.rk4(0.0, 1)
            ctx.get_state(hout)      # device -> host: the step's result (synchronous)
        te = time.perf_counter() - t0
        te_max = max_over_ranks(te, ws, "cuda:%d" % dev)
        nbytes = int(np.prod(shape)) * (16 if dbl else 8)
        out["e2e"] = {"value": ws * ke / te_max, "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                      "d2h_bytes_per_step": nbytes, "steps": ke,
                      "path": "Context.set_state(pinned host) + rk4 + get_state(pinned host) per step"}
    ctx.close()
    del ctx

    if not args.no_fp64:
        c64 = Context(N, nu=NU, precision="double", device=dev)
        c64.set_forcing(EPS, KF)
        c64.set_cfl(CFL)
        c64.set_state(uh0.astype(np.complex128))
        c64.rk4(0.0, 2)
        c64.synchronize()
        st = torch.cuda.ExternalStream(c64.stream_handle(), device=torch.device("cuda", dev))
        k64 = max(3, args.steps // 10)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(st)
        c64.rk4(0.0, k64)
        a1.record(st)
        torch.cuda.synchronize(dev)
        m64 = a0.elapsed_time(a1)
        out["fp64"] = {"value": ws * k64 / (m64 / 1e3), "unit": "steps/s", "steps": k64,
                       "ms_per_step": m64 / k64, "dtype": "f64"}
        c64.close()

    if not args.no_les and n >= 64:
        out["les"] = les_measure(dev, n, dns_s_per_sim_time)
    if not args.no_1024 and n == 512:
        out["decaying_1024"] = decay_1024(dev, ws)
    if not args.no_pad32 and n == 512:
        out["dealias_3_2"] = pad32_line(dev, ws)
    if not args.no_cufft:
        out["cufft_comparison"] = cufft_compare(dev, ws, N, out["value"])
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_sample(512 if n >= 512 else n)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def tg256(dev, steps=1000, n=256):
    """Taylor-Green at 256^3, nu = 0.000625, dt = 0.005, 1000 RK4 steps in FP32 and in FP64 on the
    GPU, with energy and dissipation (FP64 reductions) every step; the FP64 run is pinned to the
    float64 oracle by the GPU tests.  Reports the largest relative FP32-FP64 differences and
    both runs' steps/s."""
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import taylor_green
    N = (n,) * 3
    nu, dt = 0.000625, 0.005
    res = {"workload": "Taylor-Green %d^3, nu=0.000625, dt=0.005, %d RK4 steps, FP32 vs FP64" % (n, steps)}
    series = {}
    for prec in ("double", "single"):
        c = Context(N, nu=nu, precision=prec, device=dev)
        u0 = taylor_green(N)
        c.set_state(c.forward(u0.astype(c.real)))
        E, D = [], []
        t0 = time.perf_counter()
        for _ in range(steps):
            d = c.diagnostics()
            E.append(d["energy"])
            D.append(d["dissipation"])
            c.rk4(dt, 1)
        d = c.diagnostics()
        E.append(d["energy"])
        D.append(d["dissipation"])
        wall = time.perf_counter() - t0
        series[prec] = (np.array(E), np.array(D))
        res[prec] = {"steps_per_s_with_diagnostics": steps / wall, "final_energy": E[-1], "final_dissipation": D[-1],
                     "time": d["time"]}
        c.close()
    (E64, D64), (E32, D32) = series["double"], series["single"]
    res["max_rel_diff_energy"] = float(np.max(np.abs(E32 - E64) / E64))
    res["max_rel_diff_dissipation"] = float(np.max(np.abs(D32 - D64) / D64))
    res["rel_diff_energy_step100"] = float(abs(E32[100] - E64[100]) / E64[100])
    res["energy_every_100"] = [float(x) for x in E64[::100]]
    res["dissipation_every_100"] = [float(x) for x in D64[::100]]
    return res


def decay_1024(dev, ws, steps=5):
    """Decaying isotropic turbulence at 1024^3 FP32 (k0 = 6 spectrum, no forcing, nu = 4e-4,
    RK4 at CFL 0.5) with FP64 energy and dissipation reductions: steps/s over `steps` steps."""
    import torch
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field
    N = (1024,) * 3
    uh = isotropic_field(N, k0=6.0, energy=0.5, seed=0, dtype=np.complex64)
    c = Context(N, nu=4e-4, precision="single", device=dev)
    c.set_cfl(CFL)
    c.set_state(uh)
    del uh
    c.rk4(0.0, 2)
    c.synchronize()
    st = torch.cuda.ExternalStream(c.stream_handle(), device=torch.device("cuda", dev))
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record(st)
    c.rk4(0.0, steps)
    a1.record(st)
    torch.cuda.synchronize(dev)
    ms = a0.elapsed_time(a1)
    d = c.diagnostics()
    res = {"value": ws * steps / (ms / 1e3), "unit": "steps/s", "steps": steps, "warmup": 2,
           "ms_per_step": ms / steps, "grid": list(N), "dtype": "f32", "hbm_bytes": c.memory_bytes(),
           "energy": d["energy"], "dissipation": d["dissipation"], "time": d["time"],
           "workload": "decaying isotropic turbulence 1024^3 FP32 (seeded k^4 exp(-2(k/6)^2), E=0.5, "
                       "nu=4e-4, no forcing, RK4 CFL 0.5, FP64 reductions)"}
    c.close()
    return res


def cufft_compare(dev, ws, N, ours_steps_per_s, steps=5, dt=1e-3):
    """The same RK4 step written with cuFFT (torch.fft.rfftn / irfftn) and torch pointwise kernels on
    this GPU: the 2/3-rule Vortex right-hand side of spectralDNS NS.py:219-261 on full spectral arrays,
    FP32, fixed dt, no forcing.  A comparison arm only: it is not part of the library.  Reports its
    steps/s, our steps/s over it, and the relative difference of one right-hand side computed both ways."""
    import torch
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field
    d = torch.device("cuda", dev)
    n0, n1, n2 = N
    kc = [int(math.ceil(2.0 / 3.0 * (n // 2 + 1))) - 1 for n in N]
    for i, n in enumerate(N):  # largest |k| < 2/3 (n/2 + 1)
        while kc[i] >= 2.0 / 3.0 * (n // 2 + 1):
            kc[i] -= 1
    k0 = torch.fft.fftfreq(n0, 1.0 / n0, device=d).float().view(-1, 1, 1)
    k1 = torch.fft.fftfreq(n1, 1.0 / n1, device=d).float().view(1, -1, 1)
    k2 = torch.arange(n2 // 2 + 1, device=d).float().view(1, 1, -1)
    mask = ((k0.abs() <= kc[0]) & (k1.abs() <= kc[1]) & (k2 <= kc[2])).to(torch.complex64)
    K = [k0, k1, k2]
    K2 = k0 * k0 + k1 * k1 + k2 * k2
    iK2 = torch.where(K2 == 0, torch.zeros_like(K2), 1.0 / torch.where(K2 == 0, torch.ones_like(K2), K2))
    scale = float(n0 * n1 * n2)

    def rhs(uh):
        um = uh * mask
        u = torch.fft.irfftn(um, s=N, dim=(1, 2, 3)) * scale
        w = torch.fft.irfftn(torch.stack([1j * (K[1] * um[2] - K[2] * um[1]), 1j * (K[2] * um[0] - K[0] * um[2]),
                                          1j * (K[0] * um[1] - K[1] * um[0])]), s=N, dim=(1, 2, 3)) * scale
        x = torch.stack([u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]])
        nl = torch.fft.rfftn(x, dim=(1, 2, 3)) / scale * mask
        P = (nl[0] * K[0] + nl[1] * K[1] + nl[2] * K[2]) * iK2
        return torch.stack([nl[c] - P * K[c] - NU * K2 * uh[c] for c in range(3)])

    a, b = (1 / 6, 1 / 3, 1 / 3, 1 / 6), (0.5, 0.5, 1.0)

    def step(u0):
        u1 = u0
        u2 = u0.clone()
        for rk in range(4):
            r = rhs(u0)
            if rk < 3:
                u0 = u1 + (b[rk] * dt) * r
            u2 += (a[rk] * dt) * r
        return u2

    uh0 = isotropic_field(N, k0=K0, energy=0.5, seed=0, dtype=np.complex64)
    uh = torch.from_numpy(uh0).to(d)
    ref = rhs(uh)
    c = Context(N, nu=NU, precision="single", device=dev)
    ours = c.compute_rhs(uh.contiguous())
    diff = float((ours - ref).abs().max() / ref.abs().max())
    c.close()
    del ours, ref
    for _ in range(2):
        uh = step(uh)
    torch.cuda.synchronize(d)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        uh = step(uh)
    e1.record()
    torch.cuda.synchronize(d)
    ms = e0.elapsed_time(e1) / steps
    v = ws * 1e3 / ms
    return {"value": v, "unit": "steps/s", "ms_per_step": ms, "steps": steps, "warmup": 2, "dtype": "f32",
            "ours_over_cufft": ours_steps_per_s / v if v > 0 else None, "rhs_max_rel_diff_vs_ours": diff,
            "what": "torch.fft (cuFFT) rfftn/irfftn + torch pointwise kernels, full spectral arrays, 2/3 mask, "
                    "projection, diffusion, classic RK4 in FP32, fixed dt %g" % dt}


def decay_1024_run(dev, steps=500):
    """The 1024^3 decaying-turbulence case run to completion: FP64 kinetic energy E and dissipation
    eps every step.  The dealiased u x w term conserves energy, so E(0) - E(t) must equal the time
    integral of eps (trapezoid rule over the CFL steps); the relative residual of that budget, the
    divergence and the final state are reported."""
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field
    N = (1024,) * 3
    uh = isotropic_field(N, k0=6.0, energy=0.5, seed=0, dtype=np.complex64)
    c = Context(N, nu=4e-4, precision="single", device=dev)
    c.set_cfl(CFL)
    c.set_state(uh)
    del uh
    E, D, T = [], [], []
    d = c.diagnostics()
    E.append(d["energy"]); D.append(d["dissipation"]); T.append(d["time"])
    t0 = time.perf_counter()
    for _ in range(steps):
        c.rk4(0.0, 1)
        d = c.diagnostics()
        E.append(d["energy"]); D.append(d["dissipation"]); T.append(d["time"])
    wall = time.perf_counter() - t0
    E, D, T = np.array(E), np.array(D), np.array(T)
    lost = E[0] - E[-1]
    integral = float(np.sum(0.5 * (D[1:] + D[:-1]) * np.diff(T)))
    res = {"workload": "decaying isotropic turbulence 1024^3 FP32 (seeded k^4 exp(-2(k/6)^2), E=0.5, nu=4e-4, "
                       "no forcing, RK4 CFL 0.5, FP64 energy and dissipation every step)",
           "steps": steps, "wall_s_with_diagnostics": wall, "steps_per_s_with_diagnostics": steps / wall,
           "time": float(T[-1]), "energy_initial": float(E[0]), "energy_final": float(E[-1]),
           "dissipation_initial": float(D[0]), "dissipation_final": float(D[-1]),
           "dissipation_max": float(D.max()), "energy_monotone": bool(np.all(np.diff(E) <= 1e-12 * E[0])),
           "energy_lost": float(lost), "dissipation_integral": integral,
           "budget_rel_residual": float(abs(lost - integral) / max(lost, 1e-300)),
           "divergence_final": d["divergence"], "cfl_rate_final": d["cfl_rate"],
           "energy_every_50": E[::50].tolist(), "dissipation_every_50": D[::50].tolist(), "time_every_50": T[::50].tolist(),
           "hbm_bytes": c.memory_bytes()}
    c.close()
    return res


def pad32_line(dev, ws, n=256, steps=10):
    """RK4 steps/s of the same seeded isotropic field at n^3 FP32 (fixed dt) with the 3/2 rule (padded
    3n/2 transforms, generic mixed-radix kernels) and with the 2/3 rule (fused sweeps), for the cost of
    the reference's second dealiasing mode."""
    import torch
    from spectraldns_gb300.gpu import Context
    from spectraldns_gb300.init import isotropic_field
    N = (n,) * 3
    uh = isotropic_field(N, k0=K0, energy=0.5, seed=0, dtype=np.complex64)
    res = {"grid": list(N), "dtype": "f32", "steps": steps, "warmup": 3, "dt": 1e-3, "unit": "steps/s"}
    for rule, key in (("3/2-rule", "three_halves"), ("2/3-rule", "two_thirds")):
        c = Context(N, nu=NU, precision="single", dealias=rule, device=dev)
        c.set_state(uh)
        c.rk4(1e-3, 3)
        c.synchronize()
        st = torch.cuda.ExternalStream(c.stream_handle(), device=torch.device("cuda", dev))
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(st)
        c.rk4(1e-3, steps)
        a1.record(st)
        torch.cuda.synchronize(dev)
        ms = a0.elapsed_time(a1)
        res[key] = ws * steps / (ms / 1e3)
        res[key + "_hbm_bytes"] = c.memory_bytes()
        c.close()
    return res


def les_measure(dev, n_dns, dns_s_per_sim_time, ratio=8, steps=30):
    """GPU time per unit simulated time of the 64^3 closure LES (network inference + RK4 step),
    timed on this GPU, against the DNS measured above; spectrum errors from the committed
    closure experiment (profiles/les_closure_512to64.json)."""
    import torch
    from spectraldns_gb300 import les as L
    from spectraldns_gb300.init import isotropic_field
    nc = n_dns // ratio
    n = (nc,) * 3
    model = os.path.join(ROOT, "spectraldns_gb300", "data", "closure_%d.npz" % nc)
    if os.path.exists(model):
        net, nm, scale = L.load_model(model, n, device=dev)
        trained = True
    else:
        net = L.ClosureNet(n, device=dev)
        d = torch.device("cuda", dev)
        nm = {"fmu": torch.zeros(9, device=d), "fisd": torch.ones(9, device=d), "tmu": torch.zeros(6, device=d),
              "tsd": torch.full((6,), 1e-3, device=d)}
        trained = False
        scale = 1.0
    les = L.LES(n, net, nm, device=dev, scale=scale)
    les.ctx.set_state(isotropic_field(n, k0=4.0, energy=0.5, seed=0, dtype=np.complex64))
    for _ in range(3):
        les.step()
    les.ctx.synchronize()
    t0 = les.time()
    w0 = time.perf_counter()
    for _ in range(steps):
        les.step()
    les.ctx.synchronize()
    wall = time.perf_counter() - w0
    sim = les.time() - t0
    les_s = wall / max(sim, 1e-30)
    out = {"value": dns_s_per_sim_time / les_s, "unit": "x fewer GPU-seconds per simulated time than the %d^3 DNS"
           % n_dns, "les_grid": list(n), "les_ms_per_step": 1e3 * wall / steps, "les_s_per_sim_time": les_s,
           "dns_s_per_sim_time": dns_s_per_sim_time, "trained_weights": trained,
           "timing": "wall clock around steps x (closure inference + RK4 step), synchronised"}
    try:
        with open(os.path.join(ROOT, "profiles", "les_closure_512to64.json")) as f:
            ex = json.load(f)
        ev = ex["evaluation"]
        out["spectrum_err_k<=20"] = {"closure_scale": ev["closure"].get("scale", 1.0),
                                     "closure_time_avg_spectrum": ev["closure"].get("max_err_k<=20_time_avg_spectrum"),
                                     "no_closure_time_avg_spectrum": ev["no_closure"].get(
                                         "max_err_k<=20_time_avg_spectrum"),
                                     "closure_final": ev["closure"]["max_err_k<=20_final"],
                                     "closure_mean": ev["closure"]["max_err_k<=20_mean"],
                                     "no_closure_final": ev["no_closure"]["max_err_k<=20_final"],
                                     "no_closure_mean": ev["no_closure"]["max_err_k<=20_mean"],
                                     "source": "profiles/les_closure_512to64.json"}
    except Exception:
        pass
    les.ctx.close()
    return out


def cpu_stage(n, workers):
    """One RK4 stage (ComputeRHS + stage update) of the float32 oracle port at n^3."""
    from oracle.ns_ref import Grid
    from spectraldns_gb300.init import isotropic_field
    g = Grid((n, n, n), nu=NU, dtype=np.float32, workers=workers)
    uh = isotropic_field((n, n, n), k0=K0, seed=0, dtype=np.complex64)
    u1 = uh.copy()

    def stage():
        rhs = g.compute_rhs(uh)
        u0 = u1 + np.float32(0.5 * 1e-3) * rhs
        u1[...] += np.float32(1e-3 / 6) * rhs
        return u0
    return stage


def cpu_sample(n):
    workers = os.cpu_count() or 1
    stage = cpu_stage(n, workers)
    t0 = time.perf_counter()
    stage()
    t = time.perf_counter() - t0
    return {"value": 1.0 / (4 * t), "unit": "steps/s", "cores": workers, "kind": "port",
            "sample": "one RK4 stage (ComputeRHS + stage update) of the float32 NumPy/scipy.fft oracle at %d^3 on "
                      "%d threads, %.1f s; steps/s = 1/(4 x stage time)" % (n, workers, t)}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    n = args.n
    nsteps = args.steps + args.warmup
    # a bounded per-step sample: one RK4 stage, on a grid small enough for the whole run to fit in a few minutes
    ns = n
    for cand in (n, n // 2, n // 4, n // 8):
        ns = cand
        est = 12.0 * (cand / 512.0) ** 3 * (math.log2(cand ** 3) / 27.0) if cand > 0 else 0
        if est * nsteps <= 200.0:
            break
    stage = cpu_stage(ns, workers)
    for _ in range(args.warmup):
        stage()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        stage()
    t = (time.perf_counter() - t0) / args.steps
    scale = (n / ns) ** 3 * (math.log2(n ** 3) / math.log2(ns ** 3))
    value = 1.0 / (4 * t * scale)
    sample = ("each step: one RK4 stage (ComputeRHS + stage update) of the float32 NumPy/scipy.fft restatement of "
              "spectralDNS NS.py at %d^3 on %d threads (%.3f s)" % (ns, workers, t))
    if ns != n:
        sample += "; scaled to %d^3 by the N^3 log N work ratio %.2f" % (n, scale)
    out = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 4 * t * scale * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded spectrum)", "impl": "reference",
           "config": {"workload": WORKLOAD, "grid": [n, n, n], "parallelism": "host threads"},
           "cpu_baseline": {"value": value, "unit": "steps/s", "cores": workers, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.tg256:
        print(json.dumps(tg256(int(os.environ.get("LOCAL_RANK", "0")))), flush=True)
    elif args.decay1024_steps > 0:
        print(json.dumps(decay_1024_run(int(os.environ.get("LOCAL_RANK", "0")), args.decay1024_steps)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
