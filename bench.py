#!/usr/bin/env python
"""Bratu3D 255^3 time to ||F||/||F0|| <= 1e-10 on one GB300 (the path's headline metric).

One step = one full Newton-Krylov solve of -Lap_h u - lambda e^u = 0 on the 255^3 interior grid
(16,581,375 unknowns), lambda = 6, u0 = 0, Eisenstat-Walker forcing, rtol 1e-10, multigrid
V(2,2) on the full 8-level hierarchy, through the library's C ABI with every vector resident in
HBM.  Inputs are synthetic and deterministic (u0 = 0).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--path fp64|mixed]

Paths.  mixed (the headline, default): flexible GMRES(30) whose cycles run to 30 steps, classical
Gram-Schmidt (one pass by default, --orth cgs2 for two) on lazily normalised basis vectors (an
FP32 basis in double-FP32 arithmetic while the forcing term is >= 1e-6), FP32 V-cycle, FP32
Jacobian products while the forcing term is >= 1e-5 and products of FP64 accuracy below; FP64
residual, Newton update, Arnoldi coefficients and Hessenberg least squares.  fp64 (the drop-in): the reference's right-preconditioned GMRES(30) with modified
Gram-Schmidt, FP64 V-cycle and FP64 Jacobian products.

Printed JSON line: value = seconds per solve of the headline path (CUDA events, vectors resident),
e2e = the same through numa_gpu_solve_bratu3d_host with pinned host buffers (host to device copy
of u0 and device to host copy of the solution inside the timed region), e2e_fp64 = the plain FP64
drop-in through the same call, mixed_vs_plain = the other path timed in the same run with the
error between the two solutions, roofline = the dominant kernel (the residual evaluation, with its
HBM and FP64-pipe fractions) beside the V-cycle's colour pass, cpu_baseline = the reference's
algorithm on the host cores at 255^3 itself (all cores and one thread).

--impl reference times the reference's CPU implementation of the same 255^3 solve on all host
cores: the reference's own build where it was compiled (oracle/_ref), else the oracle port (the
reference's algorithm restated in C++ with the reference's OpenMP layout), W warm-up and K timed
solves (fewer if they would not end within --ref-budget seconds; the line then says so), plus one
single-thread solve.

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
    ap.add_argument("--orth", choices=["cgs1", "cgs2"], default="cgs1",
                    help="Gram-Schmidt form of the mixed path's FGMRES")
    ap.add_argument("--cpu-reps", type=int, default=2, help="all-core CPU solves of the cpu_baseline leg")
    ap.add_argument("--ref-budget", type=float, default=270.0,
                    help="seconds the reference arm may spend on its warm-up and timed solves")
    ap.add_argument("--kernel-case", choices=["none", "vcycle", "solve", "conv", "bruss", "stencils", "eval", "batch",
                                              "learned-config"],
                    default="none",
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


# ------------------------------------------------------------------ CPU side (the reference's algorithm)
def cpu_solver():
    """(solve function, kind, Oracle for thread control): the reference's own build where it was
    compiled here (oracle/_ref), else the oracle port."""
    from oracle.oracle_lib import Oracle
    port = Oracle()
    ref = None
    try:
        ref = Oracle.reference()
    except OSError:
        ref = None
    if ref is not None:
        return ref.solve, "reference", port
    return port.solve, "port", port


def cpu_params():
    from oracle.oracle_lib import default_params
    return default_params(rtol_nl=1e-10, gmres_restart=30)


def cpu_solve_times(n: int, lam: float, method: str, reps: int) -> dict:
    """Median seconds of `reps` solves at n^3 on all host cores and of one single-thread solve."""
    solve, kind, ctl = cpu_solver()
    cores = os.cpu_count() or 1
    p = cpu_params()
    out = {"kind": kind, "cores": cores}
    for threads, r in ((cores, reps), (1, 1)):
        ctl.set_threads(threads)
        times, res = [], {}
        for _ in range(r):
            t0 = time.perf_counter()
            _, res = solve(n, lam, method, "mg", p)
            times.append(time.perf_counter() - t0)
        out[threads] = (float(np.median(times)), len(times), res)
    ctl.set_threads(cores)
    return out


def host_cpu_model() -> str:
    try:
        for line in subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.TimeoutExpired):
        pass
    return "unknown"


def run_reference(args) -> int:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0  # replicas of the CPU reference are not run: rank 0 alone reports
    solve, kind, ctl = cpu_solver()
    cores = os.cpu_count() or 1
    ctl.set_threads(cores)
    p = cpu_params()
    n = args.n
    t_start = time.perf_counter()
    times, res = [], {}
    warm_done = 0
    for _ in range(args.warmup):
        t0 = time.perf_counter()
        solve(n, args.lam, args.method, "mg", p)
        times.append(time.perf_counter() - t0)  # the first solve sizes the budget
        warm_done += 1
        if (time.perf_counter() - t_start) + times[0] * (args.steps + 1) > args.ref_budget:
            break
    times = []
    for _ in range(args.steps):
        if times and (time.perf_counter() - t_start) + float(np.mean(times)) > args.ref_budget:
            break
        t0 = time.perf_counter()
        _, res = solve(n, args.lam, args.method, "mg", p)
        times.append(time.perf_counter() - t0)
    per = float(np.mean(times))
    ctl.set_threads(1)
    t0 = time.perf_counter()
    _, res1 = solve(n, args.lam, args.method, "mg", p)
    one = time.perf_counter() - t0
    ctl.set_threads(cores)
    sample = (f"{args.method} solve at {n}^3 itself (lambda={args.lam}, u0 = 0, rtol 1e-10, GMRES(30), MG V(2,2)), "
              f"{warm_done} warm-up and {len(times)} timed solves on {cores} threads ({host_cpu_model()}), mean; "
              f"counts {res.get('iters')}/{res.get('n_JVP')}/{res.get('n_prec')} (iters/JVP/prec); "
              f"{'the reference built from its own headers' if kind == 'reference' else 'the oracle port (the reference build cannot travel to this host)'}")
    line = {
        "impl": "reference", "metric": METRIC, "value": per, "unit": "s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": warm_done, "ms_per_step": per * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (u0 = 0)",
        "config": workload_config(args, "fp64", None),
        "cpu_baseline": {"value": per, "unit": "s", "cores": cores, "kind": kind, "sample": sample,
                         "single_thread": {"value": one, "unit": "s", "cores": 1,
                                           "counts": [res1.get("iters"), res1.get("n_JVP"), res1.get("n_prec")]}},
        "e2e": {"value": per, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if len(times) < args.steps or warm_done < args.warmup:
        line["steps_requested"] = args.steps
        line["warmup_requested"] = args.warmup
        line["note"] = f"solves capped by --ref-budget {args.ref_budget:.0f} s"
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, path: str, levels: int | None) -> dict:
    lv = f"{levels} levels" if levels else "the full hierarchy"
    if path == "mixed":
        orth = "two-pass (CGS2)" if args.orth == "cgs2" else "one-pass (CGS1)"
        solver = (f"FGMRES(30) (cycles up to 30 steps; {orth} classical Gram-Schmidt on lazily normalised basis "
                  f"vectors, the basis FP32 in double-FP32 arithmetic while the forcing term is >= 1e-6 and FP64 "
                  f"below) right-preconditioned by the FP32 GMG V(2,2) ({lv}; the levels n <= 15 with the "
                  f"Jacobian -Lap_h - lambda e^u of the iterate), Jacobian products of the FP32 preconditioned "
                  f"vectors in FP32 arithmetic while the forcing term is >= 1e-5 and to FP64 accuracy below "
                  f"(double-FP32 stencil; rounded once to FP32 with RN32(lambda e^u) for the FP32 basis, with the "
                  f"FP64 coefficient for the FP64 basis); FP64 residual, Newton update, Arnoldi coefficients and "
                  f"least squares")
    else:
        solver = (f"GMRES(30) with modified Gram-Schmidt (the reference's) right-preconditioned by the FP64 GMG "
                  f"V(2,2) ({lv}), FP64 Jacobian products")
    return {
        "workload": f"Bratu3D {args.n}^3 lambda={args.lam} u0=0, {args.method.upper()} (Eisenstat-Walker forcing) + "
                    f"{solver}, stop at ||F||/||F0|| <= 1e-10",
        "n": args.n, "unknowns": args.n ** 3, "lambda": args.lam, "method": args.method, "path": path,
        "precond": (f"PoissonMG V(2,2) red-black Gauss-Seidel, {lv}" if path != "mixed" else
                    f"PoissonMG V(2,2) red-black Gauss-Seidel in FP32, {lv}, Jacobian-aware levels n <= 15"),
        "gmres_restart": 30, "rtol_nl": 1e-10,
        "orth": args.orth if path == "mixed" else "mgs",
        "jvp": "analytic (Bratu3D::jvp)",
        "l2": "inputs larger than L2: one vector is 133 MB and the solve's working set ~6 GB vs 129 MB L2",
    }


# ------------------------------------------------------------------ our arm
def params_for(G, path: str, orth: str = "cgs1"):
    """fp64: the reference's GMRES(30) with MGS.  mixed_fp32: FGMRES(30), CGS, FP32 Jacobian products.
    mixed: the same with products of FP64 accuracy in the linear solves whose tolerance is below 1e-5."""
    p = G.default_params(rtol_nl=1e-10, gmres_restart=30)
    if path in ("mixed", "mixed_fp32"):
        p.flexible = 1
        p.jvp_precision = G.FP32
        p.orth = G.CGS2 if orth == "cgs2" else G.CGS1
        p.jvp_tight = 1 if path == "mixed" else 0
    return p


def batch_params(G):
    """The batched leg's settings: the headline's mixed path (accurate products below forcing 1e-5) with the
    batched solver's multigrid tail solving with the Jacobian, as the headline's provider does."""
    p = params_for(G, "mixed", "cgs1")
    p.coarse_jacobian = 1
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
    pcj = G.Provider.jacobian_mg(ctx, n)
    u0 = ctx.vec(N).fill(0.0)
    x = ctx.vec(N)

    heads = {"fp64": (pc64, params_for(G, "fp64")), "mixed": (pcj, params_for(G, "mixed", args.orth))}
    mg_probe = G.PoissonMG(ctx, n)
    levels = mg_probe.levels()
    mg_probe.close()
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
    sec_c32, res_c32, _ = timed_solves(G, ctx, op, pcj, x, u0, "cheb", params_for(G, "mixed", args.orth), 2, 1, dist,
                                       stream)
    x_c32 = x.numpy() if dist.rank == 0 else None
    ckeys = ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_prec", "converged")
    cheb = {"plain_fp64_s": sec_c64, "mixed_s": sec_c32, "ratio": sec_c64 / sec_c32,
            "counts_fp64": {k: res_c64[k] for k in ckeys}, "counts_mixed": {k: res_c32[k] for k in ckeys},
            "rel_err_between_paths": (float(np.linalg.norm(x_c32 - x_c64) / np.linalg.norm(x_c64))
                                      if dist.rank == 0 else None),
            "note": "chebyshev_inexact (J z = F, J w = F''[z, z], trial x - z - w/2, analytic F''), same "
                    "configuration and preconditioners as the headline; mixed = FGMRES with the FP32 V-cycle "
                    "(Jacobian-aware coarse levels) and FP32 J v, of FP64 accuracy below forcing 1e-5, for both "
                    "linear solves"}

    # the learned preconditioner beside the V-cycle inside FGMRES (trained here, on this GPU, from
    # GMG-preconditioned solves of this grid at seeded lambda; lambda of the bench is held out)
    learned = None
    if not args.no_learned:
        try:
            net = G.LearnedNet(ctx, 31, seed=3)
            trep = net.train(n, instances=4, states=3, rhs_per_state=2, krylov_per_state=8, epochs=8, batch=4,
                             lr=2e-3, seed=11)
            pcl = G.Provider.learned(ctx, n, net, stall=0.9)
            sec_l, res_l, _ = timed_solves(G, ctx, op, pcl, x, u0, args.method,
                                           params_for(G, "mixed_fp32", args.orth), max(1, args.steps // 2), 1, dist,
                                           stream)
            x_l = x.numpy() if dist.rank == 0 else None
            applies, fallbacks = pcl.learned_stats()
            # held-out lambda at 127^3: a network trained the same way on that grid's hierarchy
            held = []
            if dist.rank == 0:
                n2 = 127
                net2 = G.LearnedNet(ctx, 31, seed=3)
                net2.train(n2, instances=4, states=3, rhs_per_state=2, krylov_per_state=8, epochs=8, batch=4,
                           lr=2e-3, seed=11)
                pm2 = G.Provider.poisson_mg(ctx, n2, precision=G.FP32)
                pl2 = G.Provider.learned(ctx, n2, net2, stall=0.9)
                x2 = ctx.vec(n2 ** 3)
                for lam2 in (2.7, 5.3):
                    op2 = G.Bratu3D(ctx, n2, lam2)
                    row = {"n": n2, "lambda": lam2}
                    for tag, pcx in (("mixed", pm2), ("learned", pl2)):
                        x2.fill(0.0)
                        rr = G.solve(op2, x2, "nk", params_for(G, "mixed_fp32", args.orth), pcx)
                        row[tag] = [rr["iters"], rr["n_lin_iters"], rr["converged"]]
                    held.append(row)
            learned = {"s": sec_l, "res": res_l, "x": x_l, "training": trep, "applies": applies,
                       "fallbacks": fallbacks, "held_out": held}
        except G.NumaGPUError as exc:
            learned = {"skipped": str(exc)}

    # the mixed path's two steps, one at a time: the plain FP32 Poisson V-cycle with FP32 products
    # throughout, then the Jacobian-aware coarse levels alone (levels n <= 15 with -Lap_h - lambda e^u)
    steps_mixed = {}
    if dist.rank == 0:
        for tag, pcs, prms, note in (
                ("poisson_vcycle_fp32_products", pc32, params_for(G, "mixed_fp32", args.orth),
                 "FP32 Poisson V-cycle (coarse levels -Lap_h), FP32 Jacobian products in every linear solve"),
                ("jacobian_coarse_fp32_products", pcj, params_for(G, "mixed_fp32", args.orth),
                 "Jacobian-aware coarse levels, FP32 Jacobian products in every linear solve")):
            sec_s, res_s, _ = timed_solves(G, ctx, op, pcs, x, u0, args.method, prms, max(1, args.steps // 2), 1,
                                           dist, stream)
            steps_mixed[tag] = {"s": sec_s, "x": x.numpy(), "res_rel": res_s["res"] / res_s["res0"], "note": note,
                                "counts": {k: res_s[k] for k in ("iters", "n_F", "n_JVP", "n_lin_iters", "n_prec",
                                                                 "converged")}}

    # batched solves: 128 instances, n from {31, 63, 127}, lambda ~ U[1, 6.5] (seeded), mixed path
    batched = None
    if not args.no_batch and dist.rank == 0:
        batched = batched_leg(G, ctx, stream, torch, dev, batch_params(G))

    # 2D Brusselator: 2048^2 periodic, 2 species, 20 implicit-Euler steps, NK + FGMRES(40) with the
    # FP32 coupled-block multigrid (FP64 outer), beside the all-FP64 form
    bruss = None
    if not args.no_brusselator and dist.rank == 0:
        bruss = brusselator_leg(G, ctx, stream, torch)

    # end to end through the host-buffer entry point, pinned buffers: the headline path, then the
    # plain FP64 drop-in through the same call
    h_in = torch.zeros(N, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    mgp = G.FP64 if args.path == "fp64" else G.FP32

    def e2e_leg(path, prm_e, steps):
        kind, mg_prec = ("mg", G.FP64) if path == "fp64" else ("jacobian_mg", G.FP32)
        for _ in range(2):  # warm: allocations, the host entry's operator, hierarchy and captured graphs
            G.solve_bratu3d_host(ctx, n, args.lam, h_in, h_out, args.method, kind, mg_prec, prm_e)
        dist.barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with quiet_gc():
            ev0.record(stream)
            for _ in range(steps):
                G.solve_bratu3d_host(ctx, n, args.lam, h_in, h_out, args.method, kind, mg_prec, prm_e)
            ev1.record(stream)
            ev1.synchronize()
        return dist.max(ev0.elapsed_time(ev1) * 1e-3 / steps), h_out.copy()

    e2e_sec, x_e2e = e2e_leg(args.path, prm, max(1, args.steps))
    e2e_other, _ = e2e_leg(other, prmo, max(1, args.steps // 2))

    # per-primitive breakdown of one solve of each path (CUDA-event timers inside the library)
    breakdown = {}
    for name, (pcb, prmb) in heads.items():
        ctx.set_timing(True)
        x.copy_from(u0)
        rb = G.solve(op, x, args.method, prmb, pcb)
        ctx.set_timing(False)
        breakdown[name] = {k: rb[k] for k in ("t_F", "t_JVP", "t_prec", "t_setup_dynamic", "t_total")}

    # roofline: the dominant kernel of the headline solve (the residual evaluation, FP64-pipe bound)
    # and the V-cycle's dominant kernel (the finest-level red-black colour pass)
    x.copy_from(u0)
    G.solve(op, x, args.method, prm, pc)
    ms_eval = op.time_eval(x, G.FP32 if mgp == G.FP32 else G.FP64, 20)
    mg_head = G.PoissonMG(ctx, n, precision=mgp)
    ms_pass = mg_head.time_smoother(20)
    fp64_peak = ctx.fp64_peak_tflops()
    ctx.sync()

    if dist.rank == 0:
        peaks = json.loads(PEAKS_FILE.read_text()) if PEAKS_FILE.exists() else {}
        hbm_peak = float(peaks.get("hbm_gbs", FALLBACK_HBM_GBS))
        peak_source = "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback"
        eb = 8 if mgp == G.FP64 else 4
        # the residual evaluation: algorithmic 16 B a point (u read, F written once); the drivers'
        # cache adds c = lambda e^u (8 B) and, on the mixed path, RN32(c) and RN32(F) (4 + 4 B).
        # Instructions a point: ncu's counts from the committed capture of the mixed path's evaluation
        # (FP64: e^u 4 with lambda in the table, F 1, the norm 1 and the block reduction; ALU: the 7-point
        # sum in 64-bit fixed point, the FP32 conversions, addressing); the plain FP64 evaluation sums
        # in the reference's FP64 chain instead: 13.4 FP64 instructions a point by an earlier capture
        eval_bytes = 16.0 * N
        eval_moved = (32.0 if mgp == G.FP32 else 24.0) * N
        prof = load_profile(ROOT / "profiles" / "k_eval_fp32cache_255.json")
        dp_mixed = prof["fp64_thread_instructions"] / prof["points"] if prof.get("points") else 6.4
        alu_mixed = 32.0 * prof["alu_warp_instructions"] / prof["points"] if prof.get("alu_warp_instructions") else None
        eval_dp_per_pt = dp_mixed if mgp == G.FP32 else 13.4
        if mgp != G.FP32:
            prof, alu_mixed = {}, None
        ach_eval = eval_bytes / (ms_eval * 1e-3) / 1e9
        dp_rate = eval_dp_per_pt * N / (ms_eval * 1e-3) / 1e12
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        sm_mhz = (clk.summary().get("sm_mhz") or 2070.0)
        alu_peak = 64.0 * sm_count * sm_mhz * 1e6 / 1e12  # 64 ALU operations a clock an SM
        alu_rate = alu_mixed * N / (ms_eval * 1e-3) / 1e12 if alu_mixed else None
        # one red-black colour pass: the own-colour right-hand side (N/2) and the other-colour
        # neighbours (N/2) read once, the own-colour values (N/2) written once
        pass_bytes = 3 * (N / 2) * eb
        achieved = pass_bytes / (ms_pass * 1e-3) / 1e9
        roofline = {
            "kernel": f"k_eval (FP64 residual F, its norm and the drivers' cache), {n}^3",
            "bound": "hbm", "achieved": ach_eval, "peak": hbm_peak, "unit": "GB/s", "frac": ach_eval / hbm_peak,
            "traffic": prof.get("dram_bytes_per_launch"), "ms_per_launch": ms_eval,
            "algorithmic_bytes": eval_bytes, "bytes_written_and_read": eval_moved,
            "peak_source": peak_source,
            "fp64_pipe": {
                "achieved_tinstr_per_s": dp_rate, "peak_tinstr_per_s": fp64_peak / 2,
                "peak_fma_tflops_measured": fp64_peak, "frac": dp_rate / (fp64_peak / 2),
                "dp_instr_per_point": eval_dp_per_pt,
                "note": f"FP64 arithmetic ({eval_dp_per_pt:.1f} FP64 instructions a point by ncu) against the FMA-chain "
                        "peak measured live",
            },
            "alu_pipe": (None if alu_rate is None else {
                "achieved_tops": alu_rate, "peak_tops": alu_peak, "frac": alu_rate / alu_peak,
                "alu_ops_per_point": alu_mixed,
                "note": "the bound that holds on the mixed path: the integer work of the fixed-point 7-point sum "
                        "(ALU operations a point by ncu) against 64 ALU operations a clock an SM at the sampled SM "
                        "clock; ncu reads the ALU pipe 77 % and the FP64 pipe 72 % busy, HBM 16 %",
            }),
            "vcycle_colour_pass": {
                "kernel": (f"k_rbgs<double> colour pass, {n}^3" if mgp == G.FP64 else
                           f"k_pass_split colour pass (FP32, colour-split layout), {n}^3"),
                "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": load_profile_traffic(mgp), "ms_per_launch": ms_pass, "algorithmic_bytes": pass_bytes,
            },
        }
        cpu = None
        if not args.no_cpu_baseline:
            ct = cpu_solve_times(n, args.lam, args.method, args.cpu_reps)
            cores = ct["cores"]
            t_all, reps_all, rcpu = ct[cores]
            t_one, _, _ = ct[1]
            cpu = {"value": t_all, "unit": "s", "cores": cores, "kind": ct["kind"],
                   "sample": f"{args.method} solve at {n}^3 itself (same lambda / rtol / GMRES(30) / MG V(2,2), "
                             f"plain FP64), median of {reps_all} on {cores} threads ({host_cpu_model()}); counts "
                             f"{rcpu.get('iters')}/{rcpu.get('n_JVP')}/{rcpu.get('n_prec')}",
                   "single_thread": {"value": t_one, "unit": "s", "cores": 1}}
        err = float(np.linalg.norm(x_other - x_head) / np.linalg.norm(x_head))
        x_fp64 = x_head if args.path == "fp64" else x_other
        fp64_sec = sec if args.path == "fp64" else sec_o
        mixed_sec = sec_o if args.path == "fp64" else sec
        line = {
            "metric": METRIC, "value": sec, "unit": "s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.path == "fp64" else "f64+f32",
            "data": "synthetic (u0 = 0, deterministic)", "config": workload_config(args, args.path, levels),
            "counts": {k: res[k] for k in ("iters", "n_F", "n_JVP", "n_D2", "n_lin_iters", "n_prec", "converged")},
            "res_rel": res["res"] / res["res0"],
            "mixed_vs_plain": {"plain_fp64_s": fp64_sec, "mixed_s": mixed_sec, "ratio": fp64_sec / mixed_sec,
                               "rel_err_between_paths": err,
                               "other_counts": {k: res_o[k] for k in ("iters", "n_JVP", "n_prec", "converged")},
                               "note": "mixed = FP32 V-cycle with Jacobian-aware coarse levels inside FGMRES(30) "
                                       "with one-pass classical Gram-Schmidt, FP32 Jacobian products while the "
                                       "forcing term is >= 1e-5 and products of FP64 accuracy below, FP64 residual / "
                                       "updates / Arnoldi; no learned preconditioner"},
            "chebyshev": cheb,
            "learned_mixed": learned_summary(learned, fp64_sec, x_head if args.path == "fp64" else x_other),
            "mixed_steps": {tag: dict({k: v for k, v in st.items() if k != "x"},
                                      rel_err_vs_fp64=float(np.linalg.norm(st["x"] - x_fp64) / np.linalg.norm(x_fp64)))
                            for tag, st in steps_mixed.items()},
            "batched": batched,
            "brusselator2d": bruss,
            "clocks": clk.summary(),
            "e2e": {"value": e2e_sec, "unit": "s", "h2d_bytes_per_step": N * 8, "d2h_bytes_per_step": N * 8,
                    "api": "numa_gpu_solve_bratu3d_host, pinned host buffers",
                    "rel_err_vs_device_path": float(np.linalg.norm(x_e2e - x_head) / np.linalg.norm(x_head))},
            ("e2e_mixed" if args.path == "fp64" else "e2e_fp64"): {
                "value": e2e_other, "unit": "s", "h2d_bytes_per_step": N * 8, "d2h_bytes_per_step": N * 8,
                "api": "numa_gpu_solve_bratu3d_host, pinned host buffers",
                "path": "mixed" if args.path == "fp64" else "plain FP64 drop-in (GMRES(30) MGS, FP64 V-cycle)"},
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


def batched_leg(G, ctx, stream, torch, dev, pb) -> dict:
    """The batched configuration: 128 Bratu3D instances (n from {31, 63, 127}, lambda ~ U[1, 6.5], numpy
    PCG64 seed 42), mixed Newton-Krylov, u0 = 0, rtol 1e-10.  The batched solver (one launch per
    operation over the packed instance table, device-side decisions, captured step graphs), its tile
    shapes autotuned on this batch, the median of 5 batches timed with CUDA events after one warm batch; beside
    it the stream-parallel executor (host workers, one stream each) for comparison."""
    inst = G.batch_config_instances(128, seed=42)
    bs = G.BatchSolver(ctx, inst, pb)
    tune = bs.autotune((2, 4, 8), (8192, 16384, 32768))
    rb, _, _ = bs.solve()
    reps = 5
    per_batch = []
    with quiet_gc():
        for _ in range(reps):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            rb, _, _ = bs.solve()  # returns once the batch has finished (it reads the status word)
            ev1.record(stream)
            ev1.synchronize()
            per_batch.append(ev0.elapsed_time(ev1) * 1e-3)
    wall = float(np.median(per_batch))  # the median batch: one slow batch does not move it
    bs.close()
    ex = G.BatchExecutor(workers=16, device=dev)
    chosen, _ = ex.autotune(inst, (8, 16), "nk", G.FP32, pb)
    re, wall_ex = ex.solve(inst, "nk", G.FP32, pb)
    ex.close()
    return {
        "instances": len(inst), "sizes": {str(k): sum(1 for nn, _ in inst if nn == k) for k in (31, 63, 127)},
        "unknowns_total": sum(nn ** 3 for nn, _ in inst),
        "solves_per_s": len(inst) / wall, "wall_s": wall, "batch_s": per_batch, "tuning": {k: tune[k] for k in ("planes", "elems_per_block")},
        "autotune_s": tune.get("seconds"),
        "all_converged": all(r["converged"] == 1 for r in rb),
        "per_instance": {"n": [nn for nn, _ in inst], "lambda": [round(lm, 6) for _, lm in inst],
                         "iters": [r["iters"] for r in rb], "n_F": [r["n_F"] for r in rb],
                         "n_JVP": [r["n_JVP"] for r in rb], "n_lin_iters": [r["n_lin_iters"] for r in rb],
                         "converged": [r["converged"] for r in rb]},
        "stream_executor": {"solves_per_s": len(inst) / wall_ex, "workers": chosen,
                            "iters": [r["iters"] for r in re]},
        "note": "batched solver: every instance in lockstep, one kernel launch per operation over the packed "
                "instance table (the multigrid levels of one size from all instances in one launch, the levels "
                "<= 15 one CTA per instance), forcing / Givens / least squares / restarts / Armijo on the device, "
                "each Arnoldi step and line-search trial a replayed CUDA graph; mixed NK (FGMRES(30), FP32 basis "
                "with one-pass CGS, FP32 V(2,2) whose levels <= 15 solve with the Jacobian of each iterate, FP32 "
                "J v with the stencil in double-FP32 below forcing 1e-5, FP64 residual and updates); the solutions "
                "stay on the device (not copied out inside the timed batches); the stream executor runs each "
                "instance alone (Poisson V-cycle) on worker streams",
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
        "held_out_127": learned.get("held_out"),
        "training": {k: learned["training"][k] for k in ("samples", "gen_seconds", "train_seconds", "loss_first",
                                                          "loss_last", "target_ms")},
        "note": "FGMRES(30) preconditioned by the FP32 V-cycle plus a 4-level 3D conv net (BF16, tcgen05) on the "
                "31^3 level, fed the residual the V-cycle leaves and lambda e^u; trained on this GPU before the "
                "timed solves (training time not in s); falls back to the V-cycle when an iteration stalls",
    }


def learned_config_case(G, ctx, args) -> int:
    """The learned preconditioner at the scale of the learned-preconditioner configuration: trained on
    ~20k residual-error pairs from GMG-preconditioned solves of Bratu3D 127^3 at seeded lambda ~ U[1, 6.5]
    (200 instances x 3 states x (F(u), 29 Arnoldi vectors of its solve, 4 sums of 8 seeded Gaussian
    bumps)), then evaluated inside FGMRES(30) against the mixed path without it and the plain FP64 path
    at lambda values the training did not draw, at 127^3 and 255^3 (u0 = 0, rtol 1e-10).  Opt-in: it
    takes a few minutes and is not part of the default run."""
    import time
    net = G.LearnedNet(ctx, 31, seed=3)
    t0 = time.perf_counter()
    rep = net.train(127, instances=200, states=3, rhs_per_state=4, krylov_per_state=29, epochs=2, batch=8,
                    lr=1e-3, lambda_min=1.0, lambda_max=6.5, seed=2024, solve_rtol=1e-6)
    t_train = time.perf_counter() - t0
    rows = []
    for n, lams in ((127, (2.0, 4.0, 6.0)), (255, (3.0, 6.0))):
        N = n ** 3
        x = ctx.vec(N)
        pcs = {"fp64": G.Provider.poisson_mg(ctx, n, precision=G.FP64),
               "mixed": G.Provider.poisson_mg(ctx, n, precision=G.FP32),
               "learned": G.Provider.learned(ctx, n, net, stall=0.9)}
        prm = {"fp64": params_for(G, "fp64"), "mixed": params_for(G, "mixed_fp32"),
               "learned": params_for(G, "mixed_fp32")}
        for lam in lams:
            op = G.Bratu3D(ctx, n, lam)
            row = {"n": n, "lambda": lam}
            xref = None
            for tag in ("fp64", "mixed", "learned"):
                x.fill(0.0)
                G.solve(op, x, "nk", prm[tag], pcs[tag])  # warm
                ctx.sync()
                x.fill(0.0)
                t1 = time.perf_counter()
                r = G.solve(op, x, "nk", prm[tag], pcs[tag])
                ctx.sync()
                dt = time.perf_counter() - t1
                xv = x.numpy()
                if tag == "fp64":
                    xref = xv
                row[tag] = {"s": dt, "iters": r["iters"], "lin_iters": r["n_lin_iters"], "converged": r["converged"],
                            "rel_err_vs_fp64": float(np.linalg.norm(xv - xref) / np.linalg.norm(xref))}
            applies, fallbacks = pcs["learned"].learned_stats()
            row["learned"]["net_applies"], row["learned"]["fallbacks"] = applies, fallbacks
            rows.append(row)
            op.close()
        for pc in pcs.values():
            pc.close()
    print(json.dumps({"kernel_case": "learned-config", "params": net.num_params(),
                      "training": {k: rep[k] for k in ("samples", "gen_seconds", "train_seconds", "loss_first",
                                                        "loss_last", "target_ms")},
                      "training_wall_s": t_train, "held_out": rows}), flush=True)
    return 0


def load_profile(f: Path) -> dict:
    """A committed ncu summary (JSON beside its .md), or {} when absent."""
    try:
        return json.loads(f.read_text()) if f.exists() else {}
    except ValueError:
        return {}


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
    if args.kernel_case == "batch":
        # the batched configuration through the batched solver: one warm batch, then args.steps batches
        inst = G.batch_config_instances(128, seed=42)
        bs = G.BatchSolver(ctx, inst, batch_params(G))
        bs.solve()
        t = 0.0
        for _ in range(max(1, args.steps)):
            _, secs, _ = bs.solve()
            t += secs
        bs.close()
        print(json.dumps({"kernel_case": "batch", "instances": len(inst), "s_per_batch": t / max(1, args.steps),
                          "launches": ctx.kernel_launches()}))
        return 0
    if args.kernel_case == "learned-config":
        return learned_config_case(G, ctx, args)
    if args.kernel_case == "eval":
        # the residual evaluation with the mixed path's cache, on a smooth iterate of the solve's size
        op = G.Bratu3D(ctx, n, args.lam)
        i = np.arange(N, dtype=np.float64)
        xv = ctx.from_numpy(0.4 * np.sin(np.pi * (i % n + 1) / (n + 1)))
        ms = op.time_eval(xv, G.FP32 if args.path == "mixed" else G.FP64, max(1, args.steps))
        print(json.dumps({"kernel_case": "eval", "n": n, "ms_per_eval": ms, "launches": ctx.kernel_launches()}))
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
        pc = (G.Provider.poisson_mg(ctx, n, precision=G.FP64) if args.path == "fp64" else
              G.Provider.jacobian_mg(ctx, n))
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
