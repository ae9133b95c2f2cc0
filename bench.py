#!/usr/bin/env python
"""Bratu3D 255^3 time to ||F||/||F0|| <= 1e-10 on one GB300 (the path's headline metric).

One step = one full Newton-Krylov solve of -Lap_h u - lambda e^u = 0 on the 255^3 interior grid
(16,581,375 unknowns), lambda = 6, u0 = 0, GMRES(30) right-preconditioned by the geometric
multigrid V(2,2) on 8 levels, Eisenstat-Walker forcing, rtol 1e-10 — through the library's C ABI
with every vector resident in HBM.  Inputs are synthetic and deterministic (u0 = 0).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--path fp64|mixed]

Printed JSON line: value = seconds per solve of the headline path (the mixed path by default:
FP32 V-cycle and FP32 Jacobian products inside FGMRES, FP64 residual and outer iteration; --path
fp64 makes the plain FP64 drop-in the headline), e2e = the same through
numa_gpu_solve_bratu3d_host with pinned host buffers (host to device copy of u0 and device to
host copy of the solution inside the timed region), mixed_vs_plain = the other path timed in the
same run with the error between the two solutions, roofline = the V-cycle's dominant kernel (the
finest colour pass), cpu_baseline = the oracle port (the reference's algorithm restated in C++
with the reference's OpenMP layout) on the host cores.

--impl reference times the reference's CPU implementation of the same solve (the oracle port:
the reference's own build cannot travel to the GPU host) on all host cores; each step is a
127^3 solve whose time is scaled by N(255)/N(127) (the work of every primitive is linear in N
and the counts are mesh-independent: 5 Newton steps, 12 JVPs, 17 V-cycles at 31^3 ... 255^3).

Multi-GPU: the path does not shard across GPUs (replicas only): with N ranks each GPU solves its
own instance; value is the max over ranks of the time per step.
"""
from __future__ import annotations

import argparse
import contextlib
import gc
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "chebyshev-nonlinear-lab_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Bratu3D 255^3 s-to-1e-10 residual: learned/mixed vs plain FP64, one GB300"
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=255)
    ap.add_argument("--lam", type=float, default=6.0)
    ap.add_argument("--method", choices=["nk", "cheb", "rec", "tf2018"], default="nk")
    ap.add_argument("--path", choices=["fp64", "mixed"], default="mixed",
                    help="headline path (the plain FP64 drop-in is timed beside it)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-solves leg")
    ap.add_argument("--no-brusselator", action="store_true", help="skip the 2D Brusselator leg")
    ap.add_argument("--cpu-sample-n", type=int, default=127)
    ap.add_argument("--cpu-reps", type=int, default=2)
    ap.add_argument("--kernel-case", choices=["none", "vcycle", "solve", "conv", "bruss", "stencils"], default="none",
                    help="profiling driver: run only this small case (for ncu)")
    return ap.parse_args(argv)


# ------------------------------------------------------------------ distributed plumbing
class Dist:
    """torch.distributed when launched by torchrun (one rank per GPU), else a single rank."""

    def __init__(self, backend: str = "nccl"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            if backend == "nccl":
                import torch
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            if self.pg.get_backend() == "nccl":
                import torch
                self.pg.barrier(device_ids=[self.local])
                torch.cuda.synchronize()
            else:
                self.pg.barrier()

    def max(self, v: float) -> float:
        return self._reduce(v, "max")

    def sum(self, v: float) -> float:
        return self._reduce(v, "sum")

    def _reduce(self, v: float, op: str) -> float:
        if not self.pg:
            return v
        import torch
        dev = f"cuda:{self.local}" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


@contextlib.contextmanager
def quiet_gc():
    """No cyclic garbage collection inside a timed region: a collection there could run the finaliser
    of an earlier leg's device object (a device free synchronises) in the middle of the timing."""
    gc.collect()
    gc.disable()
    try:
        yield
    finally:
        gc.enable()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples every 50 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi's start-up (driver and NVML initialisation) happens before the timed region:
            # wait for its first sample (at most 5 s)
            t0 = time.time()
            while not self.lines and self.proc.poll() is None and time.time() - t0 < 5.0:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU side (oracle port)
def cpu_solve_time(n: int, lam: float, method: str, reps: int) -> tuple[float, int, dict]:
    """Median seconds of `reps` oracle-port solves at n^3 on all host threads."""
    from oracle.oracle_lib import Oracle, default_params
    o = Oracle()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    p = default_params(rtol_nl=1e-10, gmres_restart=30)
    times, res = [], {}
    for _ in range(reps):
        t0 = time.perf_counter()
        _, res = o.solve(n, lam, method, "mg", p)
        times.append(time.perf_counter() - t0)
    return float(np.median(times)), cores, res


def run_reference(args) -> int:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0  # replicas of the CPU reference are not run: rank 0 alone reports
    n_s = args.cpu_sample_n
    scale = (args.n ** 3) / (n_s ** 3)
    from oracle.oracle_lib import Oracle, default_params
    o = Oracle()
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    p = default_params(rtol_nl=1e-10, gmres_restart=30)
    for _ in range(args.warmup):
        o.solve(n_s, args.lam, args.method, "mg", p)
    times = []
    res = {}
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, res = o.solve(n_s, args.lam, args.method, "mg", p)
        times.append(time.perf_counter() - t0)
    per = float(np.mean(times)) * scale
    sample = (f"{args.method} solve at {n_s}^3 (lambda={args.lam}, rtol 1e-10, GMRES(30), MG V(2,2)) per step, "
              f"mean of {args.steps}, scaled by N({args.n})/N({n_s}) = {scale:.4f}; counts "
              f"{res.get('iters')}/{res.get('n_JVP')}/{res.get('n_prec')} (iters/JVP/prec)")
    line = {
        "impl": "reference", "metric": METRIC, "value": per, "unit": "s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (u0 = 0)",
        "config": workload_config(args, "fp64"),
        "cpu_baseline": {"value": per, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": per, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, path: str) -> dict:
    return {
        "workload": f"Bratu3D {args.n}^3 lambda={args.lam} u0=0, {args.method.upper()} + GMRES(30) right-preconditioned "
                    f"by GMG V(2,2) (8 levels), Eisenstat-Walker forcing, stop at ||F||/||F0|| <= 1e-10",
        "n": args.n, "unknowns": args.n ** 3, "lambda": args.lam, "method": args.method, "path": path,
        "precond": "PoissonMG V(2,2) red-black Gauss-Seidel", "gmres_restart": 30, "rtol_nl": 1e-10,
        "jvp": "analytic (Bratu3D::jvp)",
        "l2": "inputs larger than L2: one vector is 133 MB and the solve's working set ~6 GB vs 129 MB L2",
    }


# ------------------------------------------------------------------ our arm
def params_for(G, path: str):
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30)
    if path == "mixed":
        p.flexible = 1
        p.jvp_precision = G.FP32
        p.orth = G.CGS1
    return p


def timed_solves(G, ctx, op, pc, x, u0, method, params, steps, warmup, dist: Dist, stream):
    import torch
    for _ in range(warmup):
        x.copy_from(u0)
        G.solve(op, x, method, params, pc)
    ctx.sync()
    dist.barrier()
    ctx.reset_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.sync()
    res = None
    with quiet_gc():
        ev0.record(stream)
        for _ in range(steps):
            x.copy_from(u0)
            res = G.solve(op, x, method, params, pc)
        ev1.record(stream)
        ev1.synchronize()
    ctx.sync()
    dist.barrier()
    sec = ev0.elapsed_time(ev1) * 1e-3 / steps
    return dist.max(sec), res, ctx.kernel_launches()


def run_ours(args) -> int:
    import torch
    dist = Dist("nccl")
    dev = dist.local
    torch.cuda.set_device(dev)
    import numa_gpu as G
    ctx = G.Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=f"cuda:{dev}")
    n, N = args.n, args.n ** 3

    if args.kernel_case != "none":
        return run_kernel_case(G, ctx, args)

    op = G.Bratu3D(ctx, n, args.lam)
    pc64 = G.Provider.poisson_mg(ctx, n, precision=G.FP64)
    pc32 = G.Provider.poisson_mg(ctx, n, precision=G.FP32)
    u0 = ctx.vec(N).fill(0.0)
    x = ctx.vec(N)

    heads = {"fp64": (pc64, params_for(G, "fp64")), "mixed": (pc32, params_for(G, "mixed"))}
    pc, prm = heads[args.path]
    with ClockSampler(dev) as clk:
        sec, res, launches = timed_solves(G, ctx, op, pc, x, u0, args.method, prm, args.steps, args.warmup, dist,
                                          stream)
    x_head = x.numpy() if dist.rank == 0 else None

    # the other path, for the learned/mixed-vs-plain comparison
    other = "mixed" if args.path == "fp64" else "fp64"
    pco, prmo = heads[other]
    sec_o, res_o, _ = timed_solves(G, ctx, op, pco, x, u0, args.method, prmo, max(1, args.steps // 2), 1, dist,
                                   stream)
    x_other = x.numpy() if dist.rank == 0 else None

    # the inexact Chebyshev method (chebyshev_inexact, two linear solves and F'' per step) on both paths
    sec_c64, res_c64, _ = timed_solves(G, ctx, op, pc64, x, u0, "cheb", params_for(G, "fp64"), 2, 1, dist, stream)
    x_c64 = x.numpy() if dist.rank == 0 else None
    sec_c32, res_c32, _ = timed_solves(G, ctx, op, pc32, x, u0, "cheb", params_for(G, "mixed"), 2, 1, dist, stream)
    x_c32 = x.numpy() if dist.rank == 0 else None
    ckeys = ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_prec", "converged")
    cheb = {"plain_fp64_s": sec_c64, "mixed_s": sec_c32, "ratio": sec_c64 / sec_c32,
            "counts_fp64": {k: res_c64[k] for k in ckeys}, "counts_mixed": {k: res_c32[k] for k in ckeys},
            "rel_err_between_paths": (float(np.linalg.norm(x_c32 - x_c64) / np.linalg.norm(x_c64))
                                      if dist.rank == 0 else None),
            "note": "chebyshev_inexact (J z = F, J w = F''[z, z], trial x - z - w/2, analytic F''), same "
                    "configuration and preconditioners as the headline; mixed = FGMRES with the FP32 V-cycle and "
                    "FP32 J v for both linear solves"}

    # the learned preconditioner beside the V-cycle inside FGMRES (trained here, on this GPU, from
    # GMG-preconditioned solves of this grid at seeded lambda; lambda of the bench is held out)
    learned = None
    if not args.no_learned:
        try:
            net = G.LearnedNet(ctx, 31, seed=3)
            trep = net.train(n, instances=4, states=3, rhs_per_state=2, krylov_per_state=8, epochs=8, batch=4,
                             lr=2e-3, seed=11)
            pcl = G.Provider.learned(ctx, n, net, stall=0.9)
            sec_l, res_l, _ = timed_solves(G, ctx, op, pcl, x, u0, args.method, params_for(G, "mixed"),
                                           max(1, args.steps // 2), 1, dist, stream)
            x_l = x.numpy() if dist.rank == 0 else None
            applies, fallbacks = pcl.learned_stats()
            learned = {"s": sec_l, "res": res_l, "x": x_l, "training": trep, "applies": applies,
                       "fallbacks": fallbacks}
        except G.NumaGPUError as exc:
            learned = {"skipped": str(exc)}

    # batched solves: 128 instances, n from {31, 63, 127}, lambda ~ U[1, 6.5] (seeded), mixed path
    batched = None
    if not args.no_batch and dist.rank == 0:
        rng = np.random.default_rng(42)
        inst = [(int(nn), float(lm)) for nn, lm in zip(rng.choice([31, 63, 127], 128), rng.uniform(1.0, 6.5, 128))]
        pb = params_for(G, "mixed")
        ex = G.BatchExecutor(workers=32, device=dev)
        # the schedule (concurrent workers, each with its own stream) is autotuned on this batch
        chosen, tune = ex.autotune(inst, (4, 8, 16, 24, 32), "nk", G.FP32, pb)
        rb, wall = ex.solve(inst, "nk", G.FP32, pb)
        ex.set_workers(1)
        _, wall1 = ex.solve(inst, "nk", G.FP32, pb)
        ex.close()
        batched = {
            "instances": len(inst), "sizes": {str(k): sum(1 for nn, _ in inst if nn == k) for k in (31, 63, 127)},
            "solves_per_s": len(inst) / wall, "wall_s": wall, "workers": chosen,
            "autotune_s": tune,
            "one_worker_solves_per_s": len(inst) / wall1,
            "all_converged": all(r["converged"] == 1 for r in rb),
            "iters_range": [min(r["iters"] for r in rb), max(r["iters"] for r in rb)],
            "lin_iters_total": sum(r["n_lin_iters"] for r in rb),
            "note": "mixed NK (FGMRES(30), FP32 V-cycle and J v), u0 = 0, rtol 1e-10; host workers with one "
                    "stream each, operators, hierarchies and workspaces kept between batches; the worker count is "
                    "autotuned on this batch (each candidate: one untimed, one timed batch), then one more batch "
                    "is timed",
        }

    # 2D Brusselator: 2048^2 periodic, 2 species, 20 implicit-Euler steps, NK + FGMRES(40) with the
    # FP32 coupled-block multigrid (FP64 outer), beside the all-FP64 form
    bruss = None
    if not args.no_brusselator and dist.rank == 0:
        bruss = brusselator_leg(G, ctx, stream, torch)

    # end to end through the host-buffer entry point, pinned buffers
    h_in = torch.zeros(N, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    mgp = G.FP64 if args.path == "fp64" else G.FP32
    for _ in range(2):  # warm: allocations, the host entry's operator, hierarchy and captured graphs
        G.solve_bratu3d_host(ctx, n, args.lam, h_in, h_out, args.method, "mg", mgp, prm)
    e2e_steps = max(1, args.steps)
    dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with quiet_gc():
        ev0.record(stream)
        for _ in range(e2e_steps):
            G.solve_bratu3d_host(ctx, n, args.lam, h_in, h_out, args.method, "mg", mgp, prm)
        ev1.record(stream)
        ev1.synchronize()
    e2e_sec = dist.max(ev0.elapsed_time(ev1) * 1e-3 / e2e_steps)

    # per-primitive breakdown of one solve of each path (CUDA-event timers inside the library)
    breakdown = {}
    for name, (pcb, prmb) in heads.items():
        ctx.set_timing(True)
        x.copy_from(u0)
        rb = G.solve(op, x, args.method, prmb, pcb)
        ctx.set_timing(False)
        breakdown[name] = {k: rb[k] for k in ("t_F", "t_JVP", "t_prec", "t_setup_dynamic", "t_total")}

    # roofline of the dominant kernel: the finest-level red-black colour pass
    mg_head = G.PoissonMG(ctx, n, precision=mgp)
    ms_pass = mg_head.time_smoother(20)
    fp64_peak = ctx.fp64_peak_tflops()
    ctx.sync()

    if dist.rank == 0:
        peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
        hbm_peak = float(peaks.get("hbm_gbs", FALLBACK_HBM_GBS))
        eb = 8 if mgp == G.FP64 else 4
        # algorithmic bytes of the dominant kernel, one red-black colour pass: the own-colour
        # right-hand side (N/2) and the other-colour neighbours (N/2) read once, the own-colour
        # values (N/2) written once
        pass_bytes = 3 * (N / 2) * eb
        achieved = pass_bytes / (ms_pass * 1e-3) / 1e9
        # FP64 instructions of one pass: per updated point 6 adds + 3 for the division by 6
        # (one multiply, two FMAs); the FP64 pipe issues one such instruction per lane-cycle,
        # so its instruction peak is the measured FMA peak (2 flops each) / 2
        pass_instr = 9 * (N / 2)
        traffic = load_profile_traffic(mgp)
        roofline = {
            "kernel": (f"k_rbgs<double> colour pass, {n}^3" if mgp == G.FP64 else
                       f"k_pass_split colour pass (FP32, colour-split layout), {n}^3"),
            "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": traffic, "ms_per_launch": ms_pass,
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
        }
        if mgp == G.FP64:
            rate = pass_instr / (ms_pass * 1e-3) / 1e12
            roofline["fp64_pipe"] = {
                "achieved_tinstr_per_s": rate, "peak_tinstr_per_s": fp64_peak / 2,
                "peak_fma_tflops_measured": fp64_peak, "frac": rate / (fp64_peak / 2),
                "note": "FP64 arithmetic, not HBM, bounds the FP64 kernels on this GPU: DP instructions "
                        "per second vs the FMA-chain peak measured live",
            }
        cpu = None
        if not args.no_cpu_baseline:
            t_cpu, cores, rcpu = cpu_solve_time(args.cpu_sample_n, args.lam, args.method, args.cpu_reps)
            scale = N / args.cpu_sample_n ** 3
            cpu = {"value": t_cpu * scale, "unit": "s", "cores": cores, "kind": "port",
                   "sample": f"{args.method} solve at {args.cpu_sample_n}^3 (same lambda/rtol/GMRES/MG), median of "
                             f"{args.cpu_reps}, scaled by N({n})/N({args.cpu_sample_n}) = {scale:.4f}; counts "
                             f"{rcpu.get('iters')}/{rcpu.get('n_JVP')}/{rcpu.get('n_prec')}"}
        err = float(np.linalg.norm(x_other - x_head) / np.linalg.norm(x_head))
        fp64_sec = sec if args.path == "fp64" else sec_o
        mixed_sec = sec_o if args.path == "fp64" else sec
        line = {
            "metric": METRIC, "value": sec, "unit": "s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.path == "fp64" else "f64+f32",
            "data": "synthetic (u0 = 0, deterministic)", "config": workload_config(args, args.path),
            "counts": {k: res[k] for k in ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_prec", "converged")},
            "res_rel": res["res"] / res["res0"],
            "mixed_vs_plain": {"plain_fp64_s": fp64_sec, "mixed_s": mixed_sec, "ratio": fp64_sec / mixed_sec,
                               "rel_err_between_paths": err,
                               "other_counts": {k: res_o[k] for k in ("iters", "n_JVP", "n_prec", "converged")},
                               "note": "mixed = FP32 V-cycle + FP32 Jacobian products inside FGMRES(30) with one-pass "
                                       "classical Gram-Schmidt, FP64 residual / updates / Arnoldi; no learned "
                                       "preconditioner"},
            "chebyshev": cheb,
            "learned_mixed": learned_summary(learned, fp64_sec, x_head if args.path == "fp64" else x_other),
            "batched": batched,
            "brusselator2d": bruss,
            "clocks": clk.summary(),
            "e2e": {"value": e2e_sec, "unit": "s", "h2d_bytes_per_step": N * 8, "d2h_bytes_per_step": N * 8,
                    "api": "numa_gpu_solve_bratu3d_host, pinned host buffers"},
            "gpu_launches": launches,
            "breakdown_s": breakdown,
            "roofline": roofline,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def brusselator_leg(G, ctx, stream, torch, n: int = 2048, steps: int = 20) -> dict:
    """Twenty implicit-Euler steps of the periodic 2-species Brusselator at 2048^2 (A = 1, B = 3.4,
    D = 0.002, dt = 0.01, seeded initial state): device-resident (CUDA events) and end to end
    through numa_gpu_brusselator2d_advance_host with pinned buffers; the CPU restatement times one
    step at 512^2 on the host cores, scaled by the unknowns and the step count."""
    prm = G.brusselator_params()
    N = 2 * n * n
    x0 = G.brusselator2d_initial(n)
    op = G.Brusselator2D(ctx, n, prm)
    # rtol 1e-6 per step: once the initial noise has decayed (step ~14) a step starts from
    # ||F|| ~ 1, while ||F|| cannot fall below ~sqrt(N) 4 D h^-2 ulp(u) / 2 ~ 1e-8 at 2048^2 (an
    # FP64 state rounded to the ulp moves F by that much), so 1e-8 is out of reach there
    kp = dict(rtol_nl=1e-6, gmres_restart=40, gmres_max_iters=400)
    legs = {"mixed": (G.Provider.brusselator_mg(op, G.FP32),
                      G.default_params(flexible=1, jvp_precision=G.FP32, orth=G.CGS1, **kp)),
            "fp64": (G.Provider.brusselator_mg(op, G.FP64), G.default_params(**kp))}
    x0d = ctx.from_numpy(x0)
    x = ctx.vec(N)
    out = {}
    for name, (pc, p) in legs.items():
        x.copy_from(x0d)
        op.advance(x, 1, "nk", p, pc)  # warm: workspaces, multigrid graph
        x.copy_from(x0d)
        ctx.sync()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with quiet_gc():
            ev0.record(stream)
            res = op.advance(x, steps, "nk", p, pc)
            ev1.record(stream)
            ev1.synchronize()
        out[name] = {"s": ev0.elapsed_time(ev1) * 1e-3, "x": x.numpy(), "res": res}
    mixed, fp64 = out["mixed"], out["fp64"]
    h_in = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = x0
    # warm: the host entry's operator, multigrid hierarchy and captured graph
    G.brusselator2d_advance_host(ctx, n, h_in, 1, prm, "nk", "mg", G.FP32, legs["mixed"][1], h_out)
    h_in[:] = x0
    with quiet_gc():
        t0 = time.perf_counter()
        _, res_h = G.brusselator2d_advance_host(ctx, n, h_in, steps, prm, "nk", "mg", G.FP32, legs["mixed"][1],
                                                h_out)
        e2e = time.perf_counter() - t0
    # roofline of the dominant multigrid kernel: one FP32 colour pass on the 2048^2 level; algorithmic
    # bytes per grid point: the other colour's pairs (4), the own colour's right-hand side (4) and
    # blocks (8) read, its pairs written (4)
    mg = G.BrussMG2D(ctx, n, prm, G.FP32)
    mg.set_state(x0d)
    ms_pass = mg.time_pass(40)
    pass_bytes = 20.0 * n * n
    peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", FALLBACK_HBM_GBS))
    prof = ROOT / "profiles" / "k_bmg_pass_fp32_2048.json"
    traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch") if prof.exists() else None
    achieved = pass_bytes / (ms_pass * 1e-3) / 1e9
    roofline = {"kernel": f"k_bmg_pass<float> colour pass, {n}^2", "bound": "hbm", "achieved": achieved,
                "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                "ms_per_launch": ms_pass, "algorithmic_bytes": pass_bytes,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback"}
    mg.close()
    # one step at 512^2 on the host cores (the CPU restatement, FP64 multigrid, same parameters)
    from oracle.oracle_lib import Oracle, default_params as oparams
    o = Oracle()
    cores = o.max_threads()
    o.set_threads(cores)
    ns = 512
    xs = G.brusselator2d_initial(ns)
    t0 = time.perf_counter()
    _, rcpu = o.solve_bruss2d(ns, dict(A=prm.A, B=prm.B, Du=prm.Du, Dv=prm.Dv, dt=prm.dt), xs, "nk", "mg",
                              oparams(**kp))
    t_cpu = time.perf_counter() - t0
    scale = (n * n) / (ns * ns) * steps
    agg = lambda rs, k: sum(r[k] for r in rs)  # noqa: E731
    return {
        "workload": f"Brusselator2D {n}^2 periodic, 2 species, A=1 B=3.4 D_u=D_v=0.002, implicit Euler dt=0.01 x "
                    f"{steps} steps, NK + FGMRES(40) + coupled-block multigrid V(2,2) (FP32, with FP32 Jacobian "
                    "products and one-pass classical Gram-Schmidt; FP64 residual, updates and Arnoldi "
                    "coefficients), rtol 1e-6 per step; initial "
                    "u = 1 + 0.01 N(0,1), v = 3.4 + 0.01 N(0,1) (numpy PCG64, seed 20261203)",
        "unknowns": N, "steps": steps,
        "mixed_s": mixed["s"], "fp64_s": fp64["s"], "ratio": fp64["s"] / mixed["s"],
        "ms_per_step_mixed": mixed["s"] / steps * 1e3,
        "rel_err_mixed_vs_fp64": float(np.linalg.norm(mixed["x"] - fp64["x"]) / np.linalg.norm(fp64["x"])),
        "all_converged": all(r["converged"] == 1 for r in mixed["res"] + fp64["res"] + res_h),
        "not_converged": [[leg, k, r["iters"], r["res"] / r["res0"] if r["res0"] else 0.0]
                          for leg, rs in (("mixed", mixed["res"]), ("fp64", fp64["res"]), ("host", res_h))
                          for k, r in enumerate(rs) if r["converged"] != 1],
        "counts_mixed": {k: agg(mixed["res"], k) for k in ("iters", "n_JVP", "n_lin_iters", "n_prec")},
        "counts_fp64": {k: agg(fp64["res"], k) for k in ("iters", "n_JVP", "n_lin_iters", "n_prec")},
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes": N * 8, "d2h_bytes": N * 8,
                "api": "numa_gpu_brusselator2d_advance_host, pinned host buffers"},
        "cpu_baseline": {"value": t_cpu * scale, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"one NK step at {ns}^2 (FP64 multigrid), {t_cpu:.3f} s, scaled by "
                                   f"{n}^2/{ns}^2 x {steps} steps = {scale:.0f}; counts "
                                   f"{rcpu['iters']}/{rcpu['n_JVP']}/{rcpu['n_prec']}"},
        "roofline": roofline,
        "note": "no reference implementation of this configuration exists (the reference's Brusselator is 1D): "
                "the oracle is this project's CPU restatement",
    }


def learned_summary(learned, fp64_sec, x_fp64):
    """The learned-preconditioner leg of the JSON line."""
    if learned is None:
        return None
    if "skipped" in learned:
        return learned
    r = learned["res"]
    return {
        "s": learned["s"], "ratio_vs_plain": fp64_sec / learned["s"],
        "counts": {k: r[k] for k in ("iters", "n_JVP", "n_lin_iters", "n_prec", "converged")},
        "rel_err_vs_fp64": float(np.linalg.norm(learned["x"] - x_fp64) / np.linalg.norm(x_fp64)),
        "net_applies": learned["applies"], "fallbacks_to_vcycle": learned["fallbacks"],
        "training": {k: learned["training"][k] for k in ("samples", "gen_seconds", "train_seconds", "loss_first",
                                                          "loss_last", "target_ms")},
        "note": "FGMRES(30) preconditioned by the FP32 V-cycle plus a 4-level 3D conv net (BF16, tcgen05) on the "
                "31^3 level, fed the residual the V-cycle leaves and lambda e^u; trained on this GPU before the "
                "timed solves (training time not in s); falls back to the V-cycle when an iteration stalls",
    }


def load_profile_traffic(mgp) -> float | None:
    """DRAM bytes per launch of the colour pass from the committed ncu summary, if present."""
    f = ROOT / "profiles" / ("k_rbgs_fp64_255.json" if mgp == 0 else "k_pass_split_fp32_255.json")
    if f.exists():
        try:
            return float(json.loads(f.read_text())["dram_bytes_per_launch"])
        except (KeyError, ValueError):
            return None
    return None


def run_kernel_case(G, ctx, args) -> int:
    """Small fixed cases for ncu captures: a few V-cycles, or one solve."""
    n, N = args.n, args.n ** 3
    if args.kernel_case == "conv":
        # the learned preconditioner's tensor-core convolution at its largest supported shape
        rng = np.random.default_rng(0)
        nc = 63
        xin = rng.standard_normal((nc ** 3, 32)).astype(np.float32)
        w = (rng.standard_normal((27, 32, 32)) * 0.1).astype(np.float32)
        for _ in range(max(1, args.steps)):
            G.diag_conv3d(ctx, nc, xin, w)
        print(json.dumps({"kernel_case": "conv", "n": nc, "launches": ctx.kernel_launches()}))
        return 0
    if args.kernel_case == "stencils":
        # the finite-difference and second-difference products of Bratu3D at n^3, and the 5-point
        # Burgers2D stencils with one HelmholtzMG2D V-cycle at 511^2
        op = G.Bratu3D(ctx, n, args.lam)
        xv = ctx.from_numpy(0.3 * np.sin(0.37 * np.arange(N) + 0.5))
        vv = ctx.from_numpy(np.sin(0.37 * np.arange(N) + 0.5))
        out = ctx.vec(N)
        op.jvp(xv, vv, out, G.FD)
        op.d2(xv, vv, out, G.ANALYTIC)
        op.d2(xv, vv, out, G.FD)
        nb = 511
        bop = G.Burgers2D(ctx, nb, 0.05, 0.1, 1.0)
        w = ctx.from_numpy(0.5 * np.sin(0.37 * np.arange(2 * nb * nb) + 0.5))
        d = ctx.from_numpy(0.7 * np.sin(0.37 * np.arange(2 * nb * nb) + 1.1))
        bo = ctx.vec(2 * nb * nb)
        bop.eval(w, bo)
        bop.jvp(w, d, bo)
        hmg = G.HelmholtzMG2D(ctx, nb, 10.0, 0.05)
        r = ctx.from_numpy(np.sin(0.37 * np.arange(nb * nb) + 0.5))
        z = ctx.vec(nb * nb)
        hmg(r, z)
        ctx.sync()
        print(json.dumps({"kernel_case": "stencils", "n": n, "launches": ctx.kernel_launches()}))
        return 0
    if args.kernel_case == "bruss":
        # implicit-Euler steps of the 2D Brusselator at n^2 (FP32 coupled multigrid inside FGMRES(40))
        op = G.Brusselator2D(ctx, n, G.brusselator_params())
        pc = G.Provider.brusselator_mg(op, G.FP32)
        x = ctx.from_numpy(G.brusselator2d_initial(n))
        op.advance(x, max(1, args.steps), "nk", G.default_params(rtol_nl=1e-6, gmres_restart=40, gmres_max_iters=400,
                                                                  flexible=1, jvp_precision=G.FP32, orth=G.CGS1), pc)
        ctx.sync()
        print(json.dumps({"kernel_case": "bruss", "n": n, "launches": ctx.kernel_launches()}))
        return 0
    if args.kernel_case == "vcycle":
        for prec in (G.FP64, G.FP32):
            mg = G.PoissonMG(ctx, n, precision=prec)
            r = ctx.from_numpy(np.sin(0.37 * np.arange(N) + 0.5))
            z = ctx.vec(N)
            for _ in range(max(1, args.steps)):
                mg(r, z)
            ctx.sync()
    else:
        op = G.Bratu3D(ctx, n, args.lam)
        pc = G.Provider.poisson_mg(ctx, n, precision=G.FP64 if args.path == "fp64" else G.FP32)
        x = ctx.vec(N)
        for _ in range(max(1, args.steps)):
            x.fill(0.0)
            G.solve(op, x, args.method, params_for(G, args.path), pc)
    print(json.dumps({"kernel_case": args.kernel_case, "n": n, "launches": ctx.kernel_launches()}))
    return 0


def main(argv=None) -> int:
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
