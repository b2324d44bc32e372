"""Benchmark of the GB300 Euler step (Gcell-updates/s), one JSON line.

Workload (the reference's per-operator benchmark configuration, scaled to one
fused step): a 512^3-interior grid (514^3 with ghosts, following
benchmarks/benchmark_godunov.cpp:18) holding a seeded random state -- rho and
p log-uniform on [0.1, 10], each velocity component N(0, 1), gamma = 1.4,
dx = 1/512, CFL 0.4 -- advanced by the fused step (time_step -> godunov ->
cons_to_prim of simulations/euler_simulation.cpp:57-67 in one pass).  A step
updates 512^3 interior cells.  Inputs are 5.4 GB per bundle, far larger than
L2, so no flush is needed between steps.

Reported:
  value      device-resident throughput (state already in HBM)
  e2e        the same step through the C ABI from host buffers: host->device
             prim, step, device->host prim, every step
  roofline   the fused kernel against the FP64 pipe: algorithmic FLOPs per
             interior cell x cells / CUDA-event kernel time, over the FP64 FMA
             rate measured on this GPU in the same run
  operators  each reference operator alone at 514^3 (prim_to_cons,
             cons_to_prim, time_step, godunov), CUDA-event timed
  cpu_baseline  the CPU oracle (C restatement of the reference operators,
             OpenMP on all host cores) on a bounded slab of the same workload
  adjoint    the differentiation workload (128^3 implosion with density
             noise, 400 fixed-dt steps, checkpoints every 20): reverse-step
             and recompute cost per step against a plain forward step, and
             central differences of the FP64 solver against the gradient

`--impl reference` times the reference's CPU implementation instead (the
oracle port; the reference's own sources are not present where this runs).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "benchmark-euler-kernels_gb300")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gcell-updates/s per step, plain FP64 vs FP32-compensated at stated L1 error"
UNIT = "Gcell-updates/s"
GAMMA = 1.4
CFL = 0.4

# Algorithmic FP64 flops per interior cell of one fused step: each face solved
# once (3 faces per cell), the conservative update, cons_to_prim of the new
# state and the next step's wavespeed.  +,-,*,/,sqrt count 1, min/max/abs/
# select 0.  Counted by instantiating the reference's own hllc/godunov/
# cons_to_prim/time_step arithmetic with a counting scalar (oracle/count_flops.cpp).
FLOPS_PER_CELL_DEFAULT = None

# DRAM bytes (read + write) per interior cell of the fused FP64 kernel, from
# one ncu capture at 192^3 (736 MB read + 640 MB written over 7.08 M interior
# cells); the kernel streams each plane once, so traffic scales with cells.
FLUX_F64_DRAM_BYTES_PER_CELL = 194.4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=512, help="interior cells per axis")
    # the first step's host->device copy and the last step's device->host
    # copy do not overlap compute; 48 steps amortise them as a stream of
    # problems does
    ap.add_argument("--e2e-steps", type=int, default=48)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ops", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-fp32c", action="store_true")
    ap.add_argument("--fp32c-implosion-n", type=int, default=256,
                    help="interior cells per axis of the FP32c error run (implosion); 0 skips it")
    ap.add_argument("--fp32c-implosion-steps", type=int, default=1000)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-grids", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--precision-study", action="store_true",
                    help="implosion, FP32 states vs the plain FP64 run (L1/Linf of rho, p, |u|); prints its own JSON")
    ap.add_argument("--study-n", type=int, nargs="+", default=[512, 768])
    ap.add_argument("--study-steps", type=int, default=1000)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-study", action="store_true",
                    help="only the differentiation workload, with --adj-dirs central-difference directions")
    ap.add_argument("--adj-n", type=int, default=128)
    ap.add_argument("--adj-steps", type=int, default=400)
    ap.add_argument("--adj-every", type=int, default=20)
    ap.add_argument("--adj-dirs", type=int, default=16)
    ap.add_argument("--adj-smooth-dirs", type=int, default=8,
                    help="central-difference directions of the smooth-state check (64^3, 50 steps); 0 skips it")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, device="cpu") -> float:
    """The largest of every rank's value (the slowest rank's time); the
    value itself with one process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells_per_rank: int, steps: int, world: int, ms_max: float) -> float:
    """Whole-job Gcell-updates/s of `world` replicas that each update
    `cells_per_rank` cells per step, timed by the slowest rank."""
    return world * cells_per_rank * steps / (ms_max * 1e-3) / 1e9


def flops_per_cell():
    path = os.path.join(ROOT, "oracle", "flops_per_cell.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------- CPU
CPU_SLAB_PLANES = 32


def cpu_loop_sample(n: int, seconds: float, warmup: int, steps: int | None = None):
    """Times the reference loop (time_step, godunov, cons_to_prim) of the
    oracle -- the C restatement of the reference operators, OpenMP on every
    host core -- on an n x n x kz-interior slab of the workload's random state.

    Both CPU legs (the cpu_baseline leg and the reference arm) call this one
    sampler on the same slab: kz = max(CPU_SLAB_PLANES, 2 x threads) planes
    (at most n), so that every thread has rows to work on (godunov shares the
    (k, j) rows among the threads).  With steps=None the number of timed steps
    is chosen so that warmup + steps steps take about `seconds`.  Returns
    (Gcell-updates/s, record)."""
    import numpy as np

    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    import oracle as O

    O.build(ref=False)
    lib, _ = O._lib("port")
    threads = int(lib.oracle_omp_threads())
    dx = (1.0 / n,) * 3
    kz = min(n, max(CPU_SLAB_PLANES, 2 * threads))
    prim = O.random_prim(n + 2, n + 2, kz + 2, seed=0)
    cons = O.prim_to_cons(prim, GAMMA)
    if steps is None:
        t0 = time.perf_counter()
        O.simulate(prim, cons, GAMMA, dx, CFL, 1)
        per_step = max(time.perf_counter() - t0, 1e-6)
        warmup = max(warmup - 1, 0)
        steps = max(3, int(seconds / per_step) - warmup - 1)
    O.simulate(prim, cons, GAMMA, dx, CFL, warmup)
    t0 = time.perf_counter()
    O.simulate(prim, cons, GAMMA, dx, CFL, steps)
    el = time.perf_counter() - t0
    value = n * n * kz * steps / el / 1e9
    rec = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
           "omp_threads": threads, "host_cpus": cores, "timed_s": el, "steps": steps, "slab_planes": kz,
           "sample": f"{steps} timed steps of the reference loop (time_step, godunov, cons_to_prim) after "
                     f"warm-up, on a {n}x{n}x{kz}-interior slab of the {n}^3 workload's random state, "
                     f"{el:.1f} s, {threads} OpenMP threads",
           "numpy": np.__version__}
    return value, rec


def cpu_baseline(n: int, seconds: float):
    """The cpu_baseline leg of the GPU arm: the shared CPU sampler with one
    warm-up step and as many timed steps as fill `seconds`."""
    _, rec = cpu_loop_sample(n, seconds, 1)
    return rec


def run_reference(args):
    """The reference arm: the reference's CPU implementation of the path (the
    oracle port: the reference's own sources are not present where this runs)
    on all host cores.  A step is one step of the reference loop (time_step,
    godunov, cons_to_prim) on a slab of the same random state, through the
    shared CPU sampler, sized so that --warmup + --steps steps take about
    --cpu-seconds.  Under torchrun only rank 0 works and prints; the other
    ranks exit 0."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    n = args.n
    value, rec = cpu_loop_sample(n, args.cpu_seconds, args.warmup, args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": rec["timed_s"] * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"fused Euler step, {n}^3 interior, seeded random state (rho, p log-uniform "
                               "[0.1,10], u ~ N(0,1)), gamma 1.4, CFL 0.4", "n": n,
                   "l2": "CPU run (no GPU caches involved)"},
        "cpu_baseline": rec,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference arm: the reference's CPU implementation of the path, as the oracle port (the "
                "reference sources are not present where this runs); OpenMP over all host cores, the same "
                "sampler as the GPU arm's cpu_baseline leg",
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------- GPU
def random_prim_device(torch, n0, n1, n2, seed=0):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    prim = torch.empty((5, n2, n1, n0), dtype=torch.float64, device="cuda")
    lo, hi = torch.log(torch.tensor(0.1)).item(), torch.log(torch.tensor(10.0)).item()
    for f in (0, 1):
        prim[f].uniform_(lo, hi, generator=g)
        prim[f].exp_()
    for f in (2, 3, 4):
        prim[f].normal_(0.0, 1.0, generator=g)
    return prim


def rel_errors(torch, a, b):
    """Relative L1 (sum|a-b|/sum|b|) and Linf (max|a-b|/max|b|) over interior cells."""
    a = a[1:-1, 1:-1, 1:-1]
    b = b[1:-1, 1:-1, 1:-1]
    d = (a - b).abs()
    return (d.sum() / b.abs().sum()).item(), (d.max() / b.abs().max()).item()


def state_errors(torch, prim, prim_ref):
    """L1/Linf of rho, p and |u| of prim against prim_ref (device tensors)."""
    out = {}
    for name, f in (("rho", 0), ("p", 1)):
        l1, li = rel_errors(torch, prim[f], prim_ref[f])
        out[name] = {"l1": l1, "linf": li}
    speed = prim[2:5].square().sum(0).sqrt()
    speed_ref = prim_ref[2:5].square().sum(0).sqrt()
    l1, li = rel_errors(torch, speed, speed_ref)
    out["|u|"] = {"l1": l1, "linf": li}
    return out


def run_fp32c_leg(torch, E, args, stream, n0, dx, interior, steps_total, prim_ref, hbm_peak):
    """The FP32-compensated state on the same workload: throughput, HBM
    roofline and the error against the FP64 state after the same steps."""
    prim = random_prim_device(torch, n0, n0, n0, seed=0)
    out = {}
    with E.Simulation(n0, n0, n0, GAMMA, dx, CFL, precision="f32c", stream=stream) as sim:
        sim.set_prim(prim)
        del prim
        for _ in range(args.warmup):
            sim.advance(1)
        prof = [sim.profile_step() for _ in range(3)]
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        sim.advance(args.steps)
        e.record(stream)
        e.synchronize()
        ms = s.elapsed_time(e)
        assert args.warmup + 3 + args.steps == steps_total
        got = torch.empty((5, n0, n0, n0), dtype=torch.float64, device="cuda")
        sim.get_state(prim=got)
        status = sim.status()
        bytes_step = sim.state_bytes()
    flux_ms = min(p[1] for p in prof)
    err = state_errors(torch, got, prim_ref)
    del got
    torch.cuda.empty_cache()
    out = {"value": interior * args.steps / (ms * 1e-3) / 1e9, "unit": UNIT, "ms_per_step": ms / args.steps,
           "precision": "f32c: FP32 state, FP32 HLLC, compensated update (axis flux differences, TwoProduct "
                        "and TwoSum into the cell with their errors folded back: one rounding at the state's "
                        "scale), FP64 internal energy for low-pressure cells",
           "errors_vs_f64": err, "errors_after_steps": steps_total, "status": status,
           "roofline": {"bound": "hbm", "unit": "GB/s", "algorithmic_bytes_per_cell": bytes_step / interior,
                        "achieved": bytes_step / (flux_ms * 1e-3) / 1e9, "peak": hbm_peak,
                        "peak_source": "MEASURED_PEAKS.json (measured)" if hbm_peak else None,
                        "kernel_ms": flux_ms,
                        "limiter": "instruction issue, not HBM: ncu shows the SM issuing on 67% of cycles at "
                                   "409 thread-instructions per cell, DRAM at the algorithmic 40 B/cell "
                                   "(ncu at 256^3)"}}
    if hbm_peak:
        out["roofline"]["frac"] = out["roofline"]["achieved"] / hbm_peak
    return out


def implosion_precision(torch, E, stream, n, steps, precisions):
    """The implosion (init_implode, n^3 interior, CFL 0.4) advanced `steps`
    steps in FP64 and in each FP32 state of `precisions`: the FP32 states'
    L1/Linf errors of rho, p and |u| against the FP64 run, their run times
    and final times."""
    n0 = n + 2
    dx = (1.0 / n,) * 3
    rec = {"n": n, "steps": steps}
    with E.Simulation(n0, n0, n0, GAMMA, dx, CFL, precision="f64", stream=stream) as sim:
        sim.init_implode()
        t0 = time.perf_counter()
        sim.advance(steps)
        torch.cuda.synchronize()
        rec["f64_seconds"] = time.perf_counter() - t0
        ref = torch.empty((5, n0, n0, n0), dtype=torch.float64, device="cuda")
        sim.get_state(prim=ref)
        rec["t_final"] = sim.time()[0]
        rec["f64_totals"] = sim.totals()
    torch.cuda.empty_cache()
    for precision in precisions:
        with E.Simulation(n0, n0, n0, GAMMA, dx, CFL, precision=precision, stream=stream) as sim:
            sim.init_implode()
            t0 = time.perf_counter()
            sim.advance(steps)
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            got = torch.empty((5, n0, n0, n0), dtype=torch.float64, device="cuda")
            sim.get_state(prim=got)
            rec[precision] = {"seconds": el, "t_final": sim.time()[0], "status": sim.status(),
                              "totals": sim.totals(), "errors": state_errors(torch, got, ref)}
            del got
        torch.cuda.empty_cache()
    del ref
    torch.cuda.empty_cache()
    return rec


def run_precision_study(args):
    """Implosion (init_implode) at each N for study-steps steps: FP32 states
    against the plain FP64 run, L1/Linf of rho, p, |u|."""
    import torch

    import euler_gb300 as E

    E.build()
    E.load()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    for n in args.study_n:
        rec = implosion_precision(torch, E, stream, n, args.study_steps, ("f32c", "f32c_hilo", "f32"))
        print(json.dumps({"precision_study": rec}), flush=True)
    return 0


def implode_noise_device(torch, E, nx, sigma=1e-3, seed=0):
    """The differentiation workload's initial state: init_implode on an nx^3
    interior (ghosts included), rho += N(0, sigma^2) in every cell (numpy
    PCG64, seeded)."""
    import numpy as np

    n = nx + 2
    prim = E.init_implode(n, n, n, (1.0 / nx,) * 3)
    rng = np.random.Generator(np.random.PCG64(seed))
    prim[0] += torch.from_numpy(rng.normal(0.0, sigma, size=(n, n, n))).to(prim.device)
    return prim


def box_weight_device(torch, nx):
    """J's weight: dv on cells whose centres ((i-1)+1/2)/nx lie in [0.4, 0.6]^3."""
    n = nx + 2
    x = (torch.arange(n, dtype=torch.float64) - 1 + 0.5) / nx
    inside = ((x >= 0.4) & (x <= 0.6)).to(torch.float64)
    w = inside[:, None, None] * inside[None, :, None] * inside[None, None, :] / nx ** 3
    return w.cuda()


def smooth_prim_device(torch, nx):
    """A smooth, subsonic, everywhere-moving state on an nx^3 interior (ghosts
    included), away from every kink of the HLLC flux: each normal velocity
    rises strictly along its own axis, the sound speed rises strictly along
    every axis, every velocity is positive and well below the sound speed."""
    n = nx + 2
    x = (torch.arange(n, dtype=torch.float64) - 1 + 0.5) / nx
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    s = (X + Y + Z) / 3
    prim = torch.empty((5, n, n, n), dtype=torch.float64)
    prim[0] = 1.0 - 0.1 * s
    prim[1] = 1.0 + 0.3 * s
    prim[2] = (0.3 + 0.2 * X).expand(n, n, n)
    prim[3] = (0.2 + 0.15 * Y).expand(n, n, n)
    prim[4] = (0.25 + 0.1 * Z).expand(n, n, n)
    return prim.cuda()


def central_differences(torch, E, stream, prim0, w, dts, g0, ndirs, seed, eps=1e-6):
    """Central differences of J = sum(rho(T) w) of the FP64 solver on the
    fixed dt sequence, at eps and 2 eps, along seeded random (rho, p)
    directions, beside the adjoint's <g0, v>."""
    import numpy as np

    n = prim0.shape[-1]
    nx = n - 2
    rng = np.random.default_rng(seed)
    rows = []
    with E.Simulation(n, n, n, GAMMA, (1.0 / nx,) * 3, CFL, stream=stream) as sim:
        sim.set_dt_sequence(dts)
        p = torch.empty_like(prim0)

        def J_at(x):
            sim.set_prim(x.contiguous())
            sim.advance(len(dts))
            sim.get_state(prim=p)
            return float((p[0] * w).sum())

        for _ in range(ndirs):
            v = torch.zeros_like(prim0)
            v[0] = torch.from_numpy(rng.normal(size=(n, n, n))).cuda()
            v[1] = torch.from_numpy(rng.normal(size=(n, n, n))).cuda()
            fd = {}
            for h in (eps, 2 * eps):
                fd[h] = (J_at(prim0 + h * v) - J_at(prim0 - h * v)) / (2 * h)
            rows.append({"adjoint": float((g0 * v).sum()), "fd": fd[eps], "fd_2eps": fd[2 * eps],
                         "richardson": 2 * fd[eps] - fd[2 * eps]})
    scale = float(np.sqrt(np.mean([r["adjoint"] ** 2 for r in rows])))
    rel = [abs(r["fd"] - r["adjoint"]) / abs(r["adjoint"]) for r in rows]
    rel_r = [abs(r["richardson"] - r["adjoint"]) / abs(r["adjoint"]) for r in rows]
    return {"eps": eps, "directions": ndirs,
            "max_rel_err": max(rel), "median_rel_err": float(np.median(rel)),
            "max_err_over_rms": max(abs(r["fd"] - r["adjoint"]) for r in rows) / scale,
            "richardson_max_rel_err": max(rel_r), "richardson_median_rel_err": float(np.median(rel_r)),
            "richardson_max_err_over_rms": max(abs(r["richardson"] - r["adjoint"]) for r in rows) / scale,
            "rows": rows}


def run_smooth_fd(torch, E, stream, ndirs, nx=64, nsteps=50):
    """The adjoint against central differences on a kink-free state (64^3,
    50 CFL steps held fixed, J over [0.4, 0.6]^3): the adjoint's own error,
    apart from the HLLC kinks of the differentiation workload."""
    n = nx + 2
    prim0 = smooth_prim_device(torch, nx)
    w = box_weight_device(torch, nx)
    adj = E.Adjoint(n, n, n, nsteps, gamma=GAMMA, dx=(1.0 / nx,) * 3, cfl=CFL, checkpoint_every=10, stream=stream)
    out = torch.empty_like(prim0)
    adj.forward(prim0, out=out)
    dts = adj.dts()
    gT = torch.zeros_like(prim0)
    gT[0] = w
    g0 = torch.empty_like(prim0)
    adj.backward(gT, g0)
    adj.close()
    rec = central_differences(torch, E, stream, prim0, w, dts, g0, ndirs, seed=77)
    rec["workload"] = (f"smooth subsonic state {nx}^3 (velocities and sound speed strictly monotone along each "
                       f"axis: no HLLC kink), {nsteps} CFL steps held fixed; J = sum over [0.4,0.6]^3 of rho(T) dv")
    rec["target"] = {"max_rel_err": 1e-6, "met": bool(rec["max_rel_err"] <= 1e-6)}
    return rec


def run_adjoint_leg(torch, E, stream, args, ndirs):
    """Differentiation workload: gradient of J = sum_box rho(T) dv with respect
    to the initial rho and p (128^3 implosion with density noise, 400 steps at
    the forward pass's CFL dt sequence held fixed, checkpoints every 20 steps),
    its cost against a plain forward step, and central differences
    (eps = 1e-6) of the FP64 solver along seeded random (rho, p) directions."""
    nx, nsteps, every = args.adj_n, args.adj_steps, args.adj_every
    n = nx + 2
    dx = (1.0 / nx,) * 3
    prim0 = implode_noise_device(torch, E, nx, seed=0)
    w = box_weight_device(torch, nx)
    # plain fused forward step at this size, device-resident
    with E.Simulation(n, n, n, GAMMA, dx, CFL, stream=stream) as sim:
        sim.set_prim(prim0)
        sim.advance(3)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        sim.advance(100)
        e.record(stream)
        e.synchronize()
        fwd_step_ms = s.elapsed_time(e) / 100
    adj = E.Adjoint(n, n, n, nsteps, gamma=GAMMA, dx=dx, cfl=CFL, checkpoint_every=every, stream=stream)
    out = torch.empty_like(prim0)
    adj.forward(prim0, out=out)  # CFL steps, recorded
    dts = adj.dts()
    adj.forward(prim0, dts=dts, out=out)  # the same steps at the fixed sequence (no per-step dt reads)
    gT = torch.zeros_like(prim0)
    gT[0] = w
    g0 = torch.empty_like(prim0)
    adj.backward(gT, g0)  # warm-up
    t0 = time.perf_counter()
    adj.backward(gT, g0)
    wall = time.perf_counter() - t0
    tm = adj.timing()
    J = float((out[0] * w).sum())
    rec = {"workload": f"init_implode {nx}^3 + rho noise N(0, (1e-3)^2), {nsteps} steps at fixed CFL dts, "
                       f"checkpoints every {every}; J = sum over [0.4,0.6]^3 of rho(T) dv",
           "J": J, "t_final": float(sum(dts)),
           "forward_step_ms": fwd_step_ms,
           "forward_pass_ms": tm["forward_ms"],
           "reverse_step_ms": tm["reverse_ms"] / nsteps,
           "recompute_step_ms": tm["recompute_ms"] / nsteps,
           "backward_wall_s": wall}
    rec["reverse_over_forward"] = rec["reverse_step_ms"] / fwd_step_ms
    rec["gradient_step_over_forward"] = (rec["reverse_step_ms"] + rec["recompute_step_ms"]) / fwd_step_ms
    # central differences on the fixed dt sequence, at eps and 2 eps: the flux
    # has kinks exactly at the initial state (a gas at rest with uniform
    # pressure sits at ustar == 0 on every face), where a central difference
    # carries an O(eps) term; 2 FD(eps) - FD(2 eps) cancels it
    if ndirs > 0:
        rec["central_differences"] = central_differences(torch, E, stream, prim0, w, dts, g0, ndirs, seed=2024)
    if args.adj_smooth_dirs > 0:
        rec["smooth_state_central_differences"] = run_smooth_fd(torch, E, stream, args.adj_smooth_dirs)
    adj.close()
    return rec


def run_adjoint_study(args):
    import torch

    import euler_gb300 as E

    E.build()
    E.load()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    rec = run_adjoint_leg(torch, E, stream, args, args.adj_dirs)
    print(json.dumps({"adjoint_study": rec}), flush=True)
    return 0


def draw_batch(ngrids, seed=0):
    """The batched workload: each axis length drawn from {24,32,48,64,96,128}
    (interior cells; dx = 1/n per axis), gamma U[1.1, 1.67], inner/outer
    pressure ratio log-U[0.01, 1], density ratio log-U[0.05, 1], step on
    x + y + z < c with c U[0.1, 0.5] (numpy PCG64)."""
    import numpy as np

    rng = np.random.Generator(np.random.PCG64(seed))
    grids, ics = [], []
    for _ in range(ngrids):
        n = [int(rng.choice((24, 32, 48, 64, 96, 128))) for _ in range(3)]
        gamma = float(rng.uniform(1.1, 1.67))
        pr = float(np.exp(rng.uniform(np.log(0.01), 0.0)))
        rr = float(np.exp(rng.uniform(np.log(0.05), 0.0)))
        c = float(rng.uniform(0.1, 0.5))
        grids.append((n[0] + 2, n[1] + 2, n[2] + 2, gamma, 1.0 / n[0], 1.0 / n[1], 1.0 / n[2]))
        ics.append((c, rr, pr))
    return grids, ics


def run_batch_leg(torch, E, stream, args, precision):
    """All grids of the batched workload advanced together (one persistent
    launch per step), autotuned tile shape and chunk length."""
    grids, ics = draw_batch(args.batch_grids, seed=0)
    with E.Batch(grids, cfl=CFL, precision=precision, stream=stream) as bt:
        for g, (c, rr, pr) in enumerate(ics):
            bt.init_step(g, c, rr, pr)
        tune = bt.autotune(trial_steps=2)
        info = bt.info()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        bt.advance(args.batch_steps)
        e.record(stream)
        e.synchronize()
        ms = s.elapsed_time(e)
        status = bt.status()
        t0 = bt.time(0)
    return {"value": info["interior_cells"] * args.batch_steps / (ms * 1e-3) / 1e9, "unit": UNIT,
            "grids": len(grids), "steps": args.batch_steps, "interior_cells": info["interior_cells"],
            "ms_per_step": ms / args.batch_steps, "work_items": info["items"], "autotune": tune, "status": status,
            "grid0_t": t0[0]}


def time_ops(torch, E, prim, n_int, fpc=None, fp64_peak=None, hbm_peak=None):
    """Each reference operator alone, one call after warm-up (CUDA events),
    with its HBM and FP64 rooflines: the reference's byte counters and the
    algorithmic FLOPs per cell of oracle/flops_per_cell.json (godunov: 3 faces
    per interior cell, each face solved once)."""
    n0 = n_int + 2
    dx = (1.0 / n_int,) * 3
    cons = E.prim_to_cons(prim, GAMMA)
    prim2 = torch.empty_like(prim)
    dt = E.time_step(prim, GAMMA, dx)
    cells = n0 ** 3
    interior = n_int ** 3
    out = {}

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = None
        for _ in range(reps):
            s.record()
            fn()
            e.record()
            e.synchronize()
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
        return best

    # bytes: the reference's own counters (benchmarks/benchmark_*.cpp:37-52)
    ms = timed(lambda: E.prim_to_cons(prim, GAMMA, out=cons))
    out["prim_to_cons"] = {"ms": ms, "gcells_s": cells / ms / 1e6, "gb_s": 80 * cells / ms / 1e6}
    ms = timed(lambda: E.cons_to_prim(cons, GAMMA, out=prim2))
    out["cons_to_prim"] = {"ms": ms, "gcells_s": cells / ms / 1e6, "gb_s": 80 * cells / ms / 1e6}
    ms = timed(lambda: E.time_step(prim, GAMMA, dx, out=dt))
    out["time_step"] = {"ms": ms, "gcells_s": cells / ms / 1e6, "gb_s": 40 * cells / ms / 1e6}
    ms = timed(lambda: E.godunov(prim, cons, GAMMA, dx, 1e-9))
    out["godunov"] = {"ms": ms, "gcells_s": cells / ms / 1e6, "gb_s": 120 * cells / ms / 1e6,
                      "interior_gcells_s": interior / ms / 1e6}
    ms = timed(lambda: E.godunov(prim, cons, GAMMA, dx, 1e-9, exact=True), reps=1)
    out["godunov_exact"] = {"ms": ms, "gcells_s": cells / ms / 1e6, "gb_s": 120 * cells / ms / 1e6,
                            "interior_gcells_s": interior / ms / 1e6,
                            "note": "eulr_godunov_exact_f64: bit-identical to the reference (its operation order, "
                                    "every operation rounded separately). Each face is solved once and each cell's "
                                    "sound speed and total energy computed once, as the default godunov does, so "
                                    "the algorithmic FLOPs are the same; its 3 correctly rounded divides per face "
                                    "and divide + sqrt per cell take several FP64 instructions each"}
    del cons, prim2
    if fpc:
        flops = {"prim_to_cons": (fpc["prim_to_cons_per_cell"]["total"], cells),
                 "cons_to_prim": (fpc["cons_to_prim_per_cell"]["total"], cells),
                 "time_step": (fpc["time_step_per_cell"]["total"], cells),
                 "godunov": (3 * fpc["hllc_face"]["total"] + fpc["godunov_update_per_cell"]["total"], interior),
                 "godunov_exact": (3 * fpc["hllc_face"]["total"] + fpc["godunov_update_per_cell"]["total"],
                                   interior)}
        for name, (per_cell, units) in flops.items():
            rec = out[name]
            rec["flops_per_cell"] = per_cell
            rec["fp64_tflops"] = per_cell * units / (rec["ms"] * 1e-3) / 1e12
            if fp64_peak and name != "time_step":
                rec["fp64_frac"] = rec["fp64_tflops"] * 1e12 / fp64_peak
            if hbm_peak:
                rec["hbm_frac"] = rec["gb_s"] / hbm_peak
    # the roofline that bounds each operator on GB300 (ncu of each operator at 256^3)
    for name in ("prim_to_cons", "cons_to_prim", "godunov", "godunov_exact"):
        out[name]["bound"] = "fp64"
    out["time_step"]["bound"] = "hbm"
    out["time_step"]["note"] = ("the max wavespeed is screened by an FP32 estimate built on the integer and FP32 "
                                "pipes; the exact FP64 wavespeed (correctly rounded divide and sqrt) is evaluated "
                                "only for the cells that can hold the max, so the dt is the reference's bit for bit "
                                "and the kernel streams its 40 B per cell: no FP64 fraction applies")
    return out


def run_ours(args):
    import torch

    import euler_gb300 as E

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    E.build()
    E.load()
    n = args.n
    n0 = n + 2
    dx = (1.0 / n,) * 3
    interior = n ** 3
    # a dedicated stream: the simulation captures its step loop into a CUDA
    # graph (not possible on the legacy default stream) and the timing events
    # are recorded on the same stream
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    # replicas: every rank advances its own grid, no data-path collective
    prim = random_prim_device(torch, n0, n0, n0, seed=rank)
    sim = E.Simulation(n0, n0, n0, GAMMA, dx, CFL, stream=stream)
    sim.set_prim(prim)
    del prim
    torch.cuda.synchronize()

    for _ in range(args.warmup):
        sim.advance(1)
    torch.cuda.synchronize()
    # per-launch device times of one step (the fused kernel dominates)
    prof = [sim.profile_step() for _ in range(3)]
    flux_ms = min(p[1] for p in prof)
    step_ms_launches = min(sum(p) for p in prof)

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    sim.advance(args.steps)
    e.record(stream)
    e.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(s.elapsed_time(e), device="cuda")
    ms_per_step = ms / args.steps
    value = replica_throughput(interior, args.steps, world, ms)
    status = sim.status()
    t_sim, next_dt, nsteps = sim.time()
    launches = args.steps * sim.launches_per_step()

    # roofline of the fused kernel on the FP64 pipe
    fpc = flops_per_cell()
    peak = E.fma_rate("f64")
    props = torch.cuda.get_device_properties(local)
    nominal = 2 * 2 * props.multi_processor_count * 2.07e9  # 2 DFMA/clk/SM at the 2070 MHz max clock
    roof = {"bound": "fp64", "unit": "TFLOP/s", "peak": nominal / 1e12,
            "peak_source": "nominal FP64 rate: 2 DFMA/clk/SM (ncu's figure for this GPU), FMA = 2 FLOP, "
                           f"{props.multi_processor_count} SMs at the 2070 MHz maximum clock (the clocks record "
                           "shows the clock held during the timed region); MEASURED_PEAKS.json has no FP64 figure",
            "peak_probe": peak / 1e12,
            "peak_probe_source": "measured in this run: FP64 FMA probe (eulr_probe_fma_rate), a chain of "
                                 "independent DFMAs; it reaches ~84% of the nominal rate",
            "kernel": "flux_tile_kernel<double, step>", "kernel_ms": flux_ms,
            "step_ms_sum_of_launches": step_ms_launches,
            "traffic": FLUX_F64_DRAM_BYTES_PER_CELL * interior,
            "traffic_note": "dram bytes read+write per launch: 194.4 B per interior cell from an ncu capture at "
                            "192^3, scaled by cells"}
    if fpc:
        fl = fpc["fused_step_fp64"] * interior
        roof["achieved"] = fl / (flux_ms * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / roof["peak"]
        roof["frac_of_probe"] = roof["achieved"] / roof["peak_probe"]
        roof["flops_per_cell"] = fpc["fused_step_fp64"]
    else:
        roof["achieved"] = None
        roof["frac"] = None
    # the same kernel against HBM (algorithmic 80 B per interior cell:
    # cons read + cons written)
    hbm_peak = None
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        with open(mp) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    hbm = {"algorithmic_bytes_per_cell": 80, "achieved_gbs": 80 * interior / (flux_ms * 1e-3) / 1e9,
           "peak_gbs": hbm_peak, "peak_source": "MEASURED_PEAKS.json (measured)" if hbm_peak else None}
    if hbm_peak:
        hbm["frac"] = hbm["achieved_gbs"] / hbm_peak
    roof["hbm"] = hbm

    fp32c = None
    if not args.no_fp32c:
        ref = torch.empty((5, n0, n0, n0), dtype=torch.float64, device="cuda")
        sim.get_state(prim=ref)
        fp32c = run_fp32c_leg(torch, E, args, stream, n0, dx, interior, args.warmup + 3 + args.steps, ref, hbm_peak)
        fp32c["speedup_vs_f64"] = fp32c["value"] / value
        del ref
        torch.cuda.empty_cache()
        if args.fp32c_implosion_n > 0 and rank == 0:
            # the stated error: the implosion after 1000 steps, FP32c against
            # the plain FP64 run on the same grid
            imp = implosion_precision(torch, E, stream, args.fp32c_implosion_n, args.fp32c_implosion_steps,
                                      ("f32c",))
            err = imp["f32c"]["errors"]
            fp32c["errors_vs_f64_random_state"] = fp32c.pop("errors_vs_f64")
            fp32c["errors_vs_f64_random_state_after_steps"] = fp32c.pop("errors_after_steps")
            fp32c["errors_vs_f64"] = err
            fp32c["errors_after_steps"] = imp["steps"]
            fp32c["errors_workload"] = (f"init_implode {imp['n']}^3 interior, CFL 0.4, {imp['steps']} steps, "
                                        "FP32c state against the plain FP64 run on the same grid")
            fp32c["target"] = {"rho_l1_max": 1e-6, "speedup_min": 1.7,
                               "met": bool(err["rho"]["l1"] <= 1e-6 and fp32c["speedup_vs_f64"] >= 1.7)}
            fp32c["implosion"] = imp

    batch = None
    if not args.no_batch:
        batch = {p: run_batch_leg(torch, E, stream, args, p) for p in ("f64", "f32c")}
        torch.cuda.empty_cache()

    ops = None
    if not args.no_ops and rank == 0:
        prim = random_prim_device(torch, n0, n0, n0, seed=1)
        ops = time_ops(torch, E, prim, n, fpc, nominal, hbm_peak)
        del prim
        torch.cuda.empty_cache()

    e2e = None
    if not args.no_e2e:
        # Each step starts from the host and ends on the host: prim copied in
        # from pinned memory (with prim_to_cons, the sound speed and the first
        # dt on the device), one step, prim copied back to pinned memory.
        # Three simulations on three streams take the steps in turn (a stream
        # of independent problems), so each one's copies overlap the others'
        # compute; a simulation is reused once its previous result is in host
        # memory.
        nsim = 3
        host = torch.empty((5, n0, n0, n0), dtype=torch.float64, pin_memory=True)
        outs = [torch.empty((5, n0, n0, n0), dtype=torch.float64, pin_memory=True) for _ in range(nsim)]
        src = random_prim_device(torch, n0, n0, n0, seed=2)
        host.copy_(src)
        torch.cuda.synchronize()
        # the host link this run sees: it differs between machines, with the
        # host's other traffic, and it bounds the copies of every step
        link = {}
        for name, fn in (("h2d", lambda: src.copy_(host, non_blocking=True)),
                         ("d2h", lambda: host.copy_(src, non_blocking=True))):
            fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            link[name] = 2 * host.numel() * 8 / (time.perf_counter() - t0) / 1e9
        del src
        torch.cuda.synchronize()
        streams = [torch.cuda.Stream() for _ in range(nsim)]
        sims = [E.Simulation(n0, n0, n0, GAMMA, dx, CFL, stream=st) for st in streams]
        for q, sm in enumerate(sims):  # warm-up: graph, staging paths
            sm.set_prim(host)
            sm.advance(1)
            sm.get_state(prim=outs[q])
        torch.cuda.synchronize()
        runs = []
        e2e_clocks = ClockSampler(local)
        e2e_clocks.start()
        for _ in range(3):  # host-link bandwidth varies with the machine's other tenants: median of 3
            t0 = time.perf_counter()
            for step in range(args.e2e_steps):
                q = step % nsim
                sm = sims[q]
                if step >= nsim:
                    sm.synchronize()  # its previous result is in host memory
                sm.set_prim(host)
                sm.advance(1)
                sm.get_state(prim=outs[q], wait=False)
            for sm in sims:
                sm.synchronize()
            runs.append(world * interior * args.e2e_steps / (time.perf_counter() - t0) / 1e9)
        e2e_clk = e2e_clocks.stop()
        for sm in sims:
            sm.close()
        nbytes = 5 * n0 ** 3 * 8
        e2e = {"value": sorted(runs)[1], "unit": UNIT, "runs": runs,
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": args.e2e_steps,
               "link_gbs": link, "clocks": e2e_clk,
               "how": "per step: eulr_sim_set_prim_f64 from pinned host prim (H2D, then prim_to_cons, sound speed "
                      "and first dt in one kernel), eulr_sim_advance(1), eulr_sim_get_state_async_f64 of prim to "
                      "pinned host (D2H); three simulations on three streams take the steps in turn so copies "
                      "overlap compute; wall clock from the first copy to the last result in host memory; "
                      "median of 3 runs"}
        del host, outs
        torch.cuda.empty_cache()

    adjoint = None
    if not args.no_adjoint and rank == 0:
        adjoint = run_adjoint_leg(torch, E, stream, args, args.adj_dirs)
        torch.cuda.empty_cache()

    cpu = None
    if not args.no_cpu and rank == 0:
        cpu = cpu_baseline(n, args.cpu_seconds)
        cpu.pop("_np", None)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"fused Euler step, {n}^3 interior ({n0}^3 with ghosts), seeded random state "
                                   "(rho, p log-uniform [0.1,10], u ~ N(0,1)), gamma 1.4, CFL 0.4",
                       "n": n, "precision": "f64", "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (5.4 GB per bundle); no flush"},
            "gpu_launches": launches,
            "roofline": roof,
            "clocks": clk,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "fp32c": fp32c,
            "batch": batch,
            "operators": ops,
            "adjoint": adjoint,
            "status": status,
            "sim": {"t": t_sim, "steps_taken": nsteps},
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.precision_study:
        return run_precision_study(args)
    if args.adjoint_study:
        return run_adjoint_study(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
