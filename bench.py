"""Benchmark of the accelerated PT diffusion solver (T_eff, the reference's metric).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload 2d_nonlin_4096]
                    [--precision fp64|dfh|df64|fp32_dc|fp32_rb] [--impl ours|reference]

Workload (default): 2D nonlinear diffusion D = H^3 on 4096^2 cells, 10x10
domain, H0 = 1 + exp(-r^2), H = 1 on the boundary, dt = 0.2, tol = 1e-8,
residual check every nchk = 100 iterations, FP64.  One bench *step* is one
implicit physical time step: the PT iteration driven to err <= tol.

Metric: T_eff = A_eff * iterations / time, with A_eff = (2*3+2)*nx*ny*8 bytes
per PT iteration in 2D and (2*4+2)*nx*ny*nz*8 in 3D -- the reference's own
effective-throughput definition (scripts/diff_2D_nonlin_perf.jl:107,
scripts/diff_3D/diff_3D_nonlin_perf.jl:114), in GB/s (1e9 bytes).

* ``value``: device-resident state, timed with CUDA events on the library's
  stream around K physical steps (after W untimed ones), every check and the
  stopping decision included.  The working set (7 arrays of 134 MB) is larger
  than L2, so no flush is needed.
* ``e2e``: the same metric through the C ABI call a driver makes,
  ``ptd_solve`` on pinned host buffers (H0 uploaded, one physical step solved,
  H downloaded) per step, wall clock.
* ``roofline``: the fused PT kernel alone (fixed iterations, the reference's
  perf protocol, scripts/diff_3D/diff_3D_nonlin_perf.jl:97-105), A_eff per
  launch over the mean launch time, against the measured HBM copy bandwidth.
* ``dfh`` / ``df64``: the same K steps with double-float arithmetic on the
  FP32 pipe (DFH: H kept in FP64; DF64: every value a double-float, 3D only),
  with their iteration counts and distance to the FP64 solution.
* ``cpu_baseline`` / ``--impl reference``: the CPU restatement of the
  reference (oracle/, OpenMP on all host cores; the reference's own Julia
  Threads backend cannot run here: no Julia) on a bounded sample of the same
  workload: a fixed number of PT iterations, timed, as T_eff.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pseudotransientdiffusion.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

# Published T_eff of the reference for the same metric and size (A100 SXM4,
# output/out_diff_2D_nonlin_perf_ampere.txt:40; 3D: out_diff_3D_nonlin_perf_ampere.txt:24).
PUBLISHED = {"2d_nonlin_4096": 805.77, "3d_nonlin_512": 927.66}


def a_eff_bytes(shape) -> float:
    n = 1
    for v in shape:
        n *= v
    arrays = {1: 2 * 2 + 2, 2: 2 * 3 + 2, 3: 2 * 4 + 2}[len(shape)]
    return float(arrays * n * 8)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(workload: str, summary: str = None):
    """dram bytes per launch of the dominant kernel, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", summary or f"pt_kernel_{workload}.md")
    try:
        with open(path) as fh:
            for ln in fh:
                if ln.startswith("traffic_bytes_per_launch:"):
                    return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(gpu_index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def reduce_max(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(pg, v: float) -> float:
    if pg is None:
        return v
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def cpu_baseline(script, shape, budget_s=15.0):
    """Time the oracle's fixed-iteration loop on all host cores (bounded sample)."""
    from oracle import oracle as O

    nth = os.cpu_count() or 1
    H0 = __import__("ptdiff").initial_condition(script, *shape)
    H = np.array(H0, order="F")
    q = [np.zeros_like(H) for _ in range(3)]
    t0 = time.perf_counter()
    O.iterate(script, H, H0, q, 2, nthreads=nth)
    t_probe = (time.perf_counter() - t0) / 2
    n = int(max(2, min(2000, budget_s / max(t_probe, 1e-9))))
    t0 = time.perf_counter()
    O.iterate(script, H, H0, q, n, nthreads=nth)
    dt = time.perf_counter() - t0
    teff = a_eff_bytes(shape) * n / dt / 1e9
    return {"value": round(teff, 3), "unit": "GB/s", "cores": nth, "kind": "port",
            "sample": f"{n} fixed PT iterations (no checks) of the {len(shape)}D workload "
                      f"{'x'.join(map(str, shape))}, {dt:.1f} s, CPU restatement of the reference "
                      f"(OpenMP, {nth} threads); the reference's Julia Threads backend cannot run (no Julia)"}


def run_reference(args, world, rank, pg):
    import ptdiff

    if rank != 0:
        return 0
    if args.workload not in ptdiff.scripts.CONFIGS:
        print(json.dumps({"impl": "reference", "unavailable": f"the reference has no {args.workload} "
                          "workload (batched and adjoint solvers are new here)"}), flush=True)
        return 0
    s = ptdiff.scripts.CONFIGS[args.workload]
    shape = (args.n or s.default_n,) * s.ndim
    cb = None
    vals = []
    budget = max(4.0, 60.0 / max(args.steps, 1))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cb = cpu_baseline(s, shape, budget_s=budget)
        times.append(time.perf_counter() - t0)
        vals.append(cb["value"])
    value = statistics.median(vals) if vals else 0.0
    cb["value"] = value
    line = {
        "impl": "reference", "metric": "T_eff", "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(statistics.median(times) * 1e3, 3) if times else None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "shape": list(shape), "protocol": "fixed PT iterations"},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args, world, rank, local, pg):
    """The batched 2D step-diffusion workload: 256 instances, sides log-uniform
    in [128, 1024] (seeded), FP32 + FP64 defect correction, tol 1e-8; the
    instances are sharded over the ranks by cell count (no collective on the
    data path).  Metric: instances solved per second (one physical step)."""
    import torch

    import ptdiff
    from ptdiff import dist as PD

    torch.cuda.set_device(local)
    n = 256
    sizes, Hs, Ds = ptdiff.batch_instances(n, seed=0)
    mine = PD.shard_by_cells([int(s) ** 2 for s in sizes], world)[rank]
    sz = [int(sizes[i]) for i in mine]
    p = ptdiff.batch_params(len(mine), model=1, precision=args.precision if args.precision != "fp64" else "fp32_dc",
                            nt=1)
    b = ptdiff.BatchSolver(p, sz, sz)
    w, c, us = b.tune()
    depth = b.config()[2]
    for _ in range(args.warmup):
        b.solve([Hs[i].copy(order="F") for i in mine], [Ds[i] for i in mine])
    barrier(pg)
    l0, i0 = b.counters()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        iters, err = b.solve([Hs[i].copy(order="F") for i in mine], [Ds[i] for i in mine])
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    l1, i1 = b.counters()
    b.close()
    t_max = reduce_max(pg, dt)
    total = reduce_sum(pg, len(mine) * args.steps)
    if rank == 0:
        print(json.dumps({"metric": "batch instances per second (one implicit step to tol)",
                          "value": round(total / t_max, 3), "unit": "instances/s", "n_gpus": world,
                          "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": round(t_max / args.steps * 1e3, 3), "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner + f64 outer",
                          "data": "synthetic", "config": {"workload": "batch_linstep_256", "instances": n,
                                                          "sides": "log-uniform 128..1024, seed 0",
                                                          "tuned": {"warps": w, "chunk": c, "inner_iterations_per_launch": depth,
                                                                    "us_per_iter": us}},
                          "gpu_launches": int(l1 - l0), "inner_iterations": int(i1 - i0),
                          "max_err_last": float(max(err))}), flush=True)
    return 0


def run_adjoint(args, world, rank, local, pg):
    """The adjoint workload: 3D D = exp(m) H^3 on 256^3, m a smooth Gaussian
    random field (correlation length 1, std 0.3, seeded), 10 implicit steps of
    dt = 0.1, L2 misfit of H^10 against a target from a perturbed m; one bench
    step = one gradient evaluation (forward with one checkpoint per physical
    step + adjoint), dL/dm and dL/dH0.  The gradient is checked against
    central finite differences (Richardson-combined) in random directions.
    Replicas only for N > 1."""
    import torch

    import ptdiff
    from ptdiff import scripts as S

    torch.cuda.set_device(local)
    n = args.n or 256
    shape = (n,) * 3
    # itmax bounds every solve (the forward at tol 1e-10 needs ~450 PT
    # iterations per step at 256^3, an adjoint solve ~450 or stops at its
    # arithmetic floor, see ptd_adj_residuals)
    s = S.SCRIPTS["diff_3D_nonlin_multixpu"].with_(
        name="adjoint_3d_256", model=S.NONLIN_EXPM, shift=1.0, dirichlet=1.0, ttot=1.0, dt=0.1,
        tol=args.adj_tol, itmax=20000, ic="linrange")
    log = lambda *a: print(*a, file=sys.stderr, flush=True)
    H0 = S.initial_condition(s, *shape)
    m = S.log_coefficient_field(shape, seed=0)
    mt = m + S.log_coefficient_field(shape, seed=1)   # the perturbed coefficient of the target
    dev = lambda a: torch.from_numpy(np.ravel(a, order="F").copy()).cuda()
    out = {}
    Ht = None
    head = "fp32_rb"   # the headline form: FP32 iterations on the change since an FP64 base
    for prec in (head, "df64", "fp64"):
        A = ptdiff.AdjointSolver(ptdiff.make_params(s, shape, precision=prec, nchk=10))
        if Ht is None:
            _, Ht = A.forward(H0, mt, H0, want_HN=True)
        H0d, md, Htd = dev(H0), dev(m), dev(Ht)
        gmd, ghd = torch.empty_like(H0d), torch.empty_like(H0d)
        for _ in range(args.warmup if prec == head else 1):
            A.forward(H0d, md, Htd)
            A.gradient(out_m=gmd, out_H0=ghd)
        torch.cuda.synchronize()
        barrier(pg)
        l0, i0 = A.counters()
        t_fwd = t_adj = 0.0
        nsteps = args.steps if prec == head else 1
        fwd_iters = adj_iters = 0
        for _ in range(nsteps):
            t0 = time.perf_counter()
            loss = A.forward(H0d, md, Htd)
            t1 = time.perf_counter()
            A.gradient(out_m=gmd, out_H0=ghd)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            t_fwd += t1 - t0
            t_adj += t2 - t1
            fwd_iters += int(A.forward_iters.sum())
            adj_iters += int(A.adjoint_iters.sum())
        l1, i1 = A.counters()
        res_err, res_target = A.residuals()
        log(f"adjoint {prec}: forward {t_fwd / nsteps:.2f} s, adjoint {t_adj / nsteps:.2f} s per gradient, "
            f"forward iterations {list(A.forward_iters)}, adjoint {list(A.adjoint_iters)}")
        t_tot = reduce_max(pg, t_fwd + t_adj)
        rec = {"grads_per_s": round(world * nsteps / t_tot, 4), "ms_per_gradient": round(t_tot / nsteps * 1e3, 2),
               "forward_ms": round(t_fwd / nsteps * 1e3, 2), "adjoint_ms": round(t_adj / nsteps * 1e3, 2),
               "adjoint_over_forward": round(t_adj / t_fwd, 3),
               "forward_pt_iterations": fwd_iters // nsteps, "adjoint_pt_iterations": adj_iters // nsteps,
               "gpu_launches": int(l1 - l0), "loss": loss,
               "adjoint_final_rel_residual": [float(e / t * 1e-10) if t > 0 else 0.0
                                              for e, t in zip(res_err, res_target)]}
        if prec == head:
            # e2e: host arrays in and out, the library copies them
            gm_h, gh_h = None, None
            t0 = time.perf_counter()
            for _ in range(nsteps):
                A.forward(H0, m, Ht)
                gm_h, gh_h = A.gradient()
            rec["e2e_grads_per_s"] = round(world * nsteps / reduce_max(pg, time.perf_counter() - t0), 4)
            # central differences (eps, eps/2, Richardson) in random joint directions (m, H0)
            rng = np.random.default_rng(7)
            worst = 0.0
            rels = []
            for _ in range(args.fd_directions if rank == 0 else 0):
                vm = rng.standard_normal(shape)
                vh = rng.standard_normal(shape)
                gv = float(np.sum(gm_h * vm) + np.sum(gh_h * vh))
                f = lambda e: A.forward(H0 + e * vh, m + e * vm, Ht)
                eps = args.fd_eps
                d1 = (f(eps) - f(-eps)) / (2 * eps)
                d2 = (f(eps / 2) - f(-eps / 2)) / eps
                fd = (4 * d2 - d1) / 3
                rel = abs(fd - gv) / max(abs(gv), 1e-300)
                rels.append(rel)
                log(f"fd direction {len(rels)}: adjoint {gv:.9e} fd {fd:.9e} rel {rel:.2e}")
                worst = max(worst, rel)
            rec["fd_check"] = {"directions": len(rels), "eps": args.fd_eps, "max_rel_err": worst,
                               "median_rel_err": float(np.median(rels)) if rels else None}
        out[prec] = rec
        A.close()
    if rank != 0:
        return 0
    d = out[head]
    print(json.dumps({
        "metric": "adjoint gradient evaluations per second", "value": d["grads_per_s"], "unit": "gradients/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": d["ms_per_gradient"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 changes on an f64 base (rebased)", "data": "synthetic",
        "config": {"workload": "adjoint_3d_256", "shape": list(shape), "nt": 10, "dt": 0.1, "tol": s.tol,
                   "model": "D = exp(m) H^3", "m": "Gaussian random field, corr 1, std 0.3, seed 0",
                   "target": "H^10 of m + a second such field (seed 1)", "checkpoints": "one per step",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": d["e2e_grads_per_s"], "unit": "gradients/s",
                "h2d_bytes_per_step": int(3 * H0.size * 8), "d2h_bytes_per_step": int(2 * H0.size * 8)},
        "gpu_launches": d["gpu_launches"],
        "adjoint_over_forward": d["adjoint_over_forward"],
        "fd_check": d["fd_check"],
        "fp32_rb": d, "df64": out["df64"], "fp64": out["fp64"]}), flush=True)
    return 0


def run_ours(args, world, rank, local, pg):
    import torch

    import ptdiff

    s = ptdiff.scripts.CONFIGS[args.workload]
    n = args.n or s.default_n
    shape = (n,) * s.ndim
    A = a_eff_bytes(shape)
    torch.cuda.set_device(local)
    H0 = ptdiff.initial_condition(s, *shape)
    params = ptdiff.make_params(s, shape, nt=1, precision=args.precision)
    sol = ptdiff.Solver(params)
    ext = torch.cuda.ExternalStream(sol.stream)

    def timed_steps(sol_, nsteps):
        """Set H0, run W untimed physical steps, set H0 again, time nsteps steps."""
        sol_.set_state(H0)
        for _ in range(args.warmup):
            sol_.step(1)
        sol_.set_state(H0)
        sol_.sync()
        l0_, i0_ = sol_.counters()
        st = torch.cuda.ExternalStream(sol_.stream)
        barrier(pg)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(st)
        its_ = []
        for _ in range(nsteps):
            its, _ = sol_.step(1)
            its_.append(int(its[0]))
        a1.record(st)
        a1.synchronize()
        torch.cuda.synchronize()
        barrier(pg)
        l1_, i1_ = sol_.counters()
        return a0.elapsed_time(a1) / 1e3, its_, l1_ - l0_, i1_ - i0_

    # ---- device-resident value: FP64 PT, K physical steps from H0
    clocks = ClockSampler(local) if rank == 0 else None
    t_dev, step_iters, launches, iters_timed = timed_steps(sol, args.steps)
    clk = clocks.stop() if clocks else None
    H_fp64 = sol.get_state()
    t_max = reduce_max(pg, t_dev)
    total_bytes = reduce_sum(pg, A * iters_timed)
    value = total_bytes / t_max / 1e9

    # ---- roofline: the fused kernel alone, fixed iterations (perf protocol)
    nfix = args.fixed_iters
    sol.iterate(8)
    sol.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    sol.iterate(nfix)
    e1.record(ext)
    e1.synchronize()
    t_launch = e0.elapsed_time(e1) / 1e3 / nfix
    achieved = A / t_launch / 1e9
    peak, peak_kind = read_peaks()
    traffic = profile_traffic(args.workload)
    kernel_name, kernel_bytes, launch_t = f"pt{s.ndim}d_kernel (fused PT iteration)", A, t_launch
    if args.precision == "fp32_rb":
        # the rebased FP32 kernel: 40 B per cell in 2D (52 in 3D) per launch,
        # two iterations per launch in 2D when the check cadence is even
        ipl = 2 if (s.ndim == 2 and params.nchk % 2 == 0) else 1
        kernel_bytes = (2 + 3 * s.ndim + 2) * 4 * float(np.prod(shape))
        launch_t = t_launch * ipl
        achieved = kernel_bytes / launch_t / 1e9
        kernel_name = f"rb{s.ndim}d{'_tb2' if ipl == 2 else ''}_kernel ({ipl} FP32 iterations per launch)"
        traffic = profile_traffic(args.workload, "rb2d_fp32rb_nonlin_4096.md") if (
            args.workload == "2d_nonlin_4096" and ipl == 2) else None
    sol.close()
    # the native-FP64 kernel's own roofline: FP64 instructions per cell x
    # cells / launch time against this GPU's FP64 FMA rate, measured now
    rate = ctypes.c_double(0.0)
    ptdiff._abi.check(ptdiff._abi.lib().ptd_measure_fp64_rate(ctypes.byref(rate)), "ptd_measure_fp64_rate")
    # FP64 instructions per cell of the nonlinear kernel: per face s, s^3 (2),
    # g, the flux FMA and the damping FMA (6 each), H - Hold, the flux
    # differences and their sum (square cells: no sigma multiply), the
    # residual FMA and the update FMA
    fp64_per_cell = {2: 18, 3: 26}.get(s.ndim) if s.model == ptdiff.scripts.NONLIN else None
    fp64_pipe = None
    if fp64_per_cell and args.precision == "fp64":
        ach = fp64_per_cell * float(np.prod(shape)) / t_launch / 1e9
        fp64_pipe = {"bound": "fp64 pipe", "achieved": round(ach, 1), "peak": round(rate.value / 1e9, 1),
                     "unit": "G FP64 instr/s", "frac": round(ach / (rate.value / 1e9), 4),
                     "instr_per_cell": fp64_per_cell, "peak_kind": "measured live (DFMA chains)"}

    # ---- the same FP64-accuracy iteration with double-float arithmetic on the
    # FP32 pipe: DFH (FP64 H, double-float fluxes) everywhere; DF64 (every value
    # a double-float) in 3D only -- its 48-bit H cannot reach tol on the fine 2D
    # grid and would run to itmax
    def alt_precision(prec):
        pa = ptdiff.make_params(s, shape, nt=1, precision=prec)
        sa = ptdiff.Solver(pa)
        t_a, a_iters, _, _ = timed_steps(sa, args.steps)
        H_a = sa.get_state()
        ext_a = torch.cuda.ExternalStream(sa.stream)
        sa.iterate(8)
        sa.sync()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(ext_a)
        sa.iterate(nfix)
        f1.record(ext_a)
        f1.synchronize()
        t_launch_a = f0.elapsed_time(f1) / 1e3 / nfix
        sa.close()
        t_a = reduce_max(pg, t_a)
        return {"value": round(reduce_sum(pg, A * sum(a_iters)) / t_a / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(t_a / args.steps * 1e3, 3), "pt_iterations_per_step": a_iters,
                "same_iterations_as_fp64": a_iters == step_iters,
                "rel_l2_vs_fp64": float(np.linalg.norm(H_a - H_fp64) / np.linalg.norm(H_fp64)),
                "kernel_achieved": round(A / t_launch_a / 1e9, 1),
                "kernel_frac": round(A / t_launch_a / 1e9 / peak, 4),
                "launch_us": round(t_launch_a * 1e6, 2)}

    alts = {}
    if args.precision == "fp64" and not args.no_df64:
        alts["dfh"] = alt_precision("dfh")
        if s.ndim == 3:
            alts["df64"] = alt_precision("df64")

    # ---- time to tol of the two FP32 + FP64 forms, same K steps from H0:
    # FP32_RB (FP32 PT iterations on the change since an FP64 base, rebased in
    # FP64) and FP32_DC (FP32 inner solves in an FP64 inexact-Newton loop)
    ttt = None
    if args.precision == "fp64" and not args.no_dc:
        ttt = {"fp64_ms_per_step": round(t_max / args.steps * 1e3, 3)}
        for form in ("fp32_rb", "fp32_dc"):
            pf = ptdiff.make_params(s, shape, nt=1, precision=form)
            sf = ptdiff.Solver(pf)
            t_f, f_iters, _, _ = timed_steps(sf, args.steps)
            H_f = sf.get_state()
            kern_us = None
            if form == "fp32_rb":   # the FP32 kernel alone, fixed iterations
                ext_f = torch.cuda.ExternalStream(sf.stream)
                sf.iterate(8)
                sf.sync()
                g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                g0.record(ext_f)
                sf.iterate(nfix)
                g1.record(ext_f)
                g1.synchronize()
                kern_us = round(g0.elapsed_time(g1) * 1e3 / nfix, 2)
            sf.close()
            t_f = reduce_max(pg, t_f)
            rel = float(np.linalg.norm(H_f - H_fp64) / np.linalg.norm(H_fp64))
            ttt[form] = {"ms_per_step": round(t_f / args.steps * 1e3, 3), "speedup": round(t_max / t_f, 3),
                         "rel_l2_vs_fp64": rel,
                         ("pt_iterations_per_step" if form == "fp32_rb" else "fp32_inner_iterations_per_step"):
                             f_iters}
            if kern_us is not None:
                # bytes of one launch: delta, omega_d, t_b_d, R_b, H read, delta and omega_d written;
                # in 2D a launch runs two FP32 iterations (temporal blocking, even check cadence)
                ipl = 2 if (s.ndim == 2 and pf.nchk % 2 == 0) else 1
                fb = (2 + 3 * s.ndim + 2) * 4 * float(np.prod(shape))
                launch_us = kern_us * ipl
                ttt[form].update({"kernel_us_per_iteration": kern_us, "iterations_per_launch": ipl,
                                  "kernel_us_per_launch": round(launch_us, 2),
                                  "kernel_gbs": round(fb / launch_us / 1e3, 1),
                                  "kernel_frac": round(fb / launch_us / 1e3 / peak, 4),
                                  "kernel_bytes_per_cell_per_launch": (2 + 3 * s.ndim + 2) * 4})
        ttt["speedup"] = ttt["fp32_rb"]["speedup"]

    # ---- e2e: ptd_solve on pinned host buffers, one physical step per call
    pin = torch.empty(H0.size, dtype=torch.float64, pin_memory=True)
    Hh = pin.numpy()

    def e2e_run(precision):
        sol2 = ptdiff.Solver(ptdiff.make_params(s, shape, nt=1, precision=precision))
        for _ in range(args.warmup):
            Hh[:] = np.ravel(H0, order="F")
            sol2.solve(Hh)
        barrier(pg)
        e2e_time, e2e_iters = 0.0, 0
        for _ in range(args.steps):
            Hh[:] = np.ravel(H0, order="F")
            t0 = time.perf_counter()
            its, _, _ = sol2.solve(Hh)
            e2e_time += time.perf_counter() - t0
            e2e_iters += int(its.sum())
        sol2.close()
        return reduce_max(pg, e2e_time), e2e_iters

    e2e_t, e2e_iters = e2e_run(args.precision)
    e2e_val = reduce_sum(pg, A * e2e_iters) / e2e_t / 1e9
    if ttt is not None:
        # time to tol end to end: H0 uploaded from and H downloaded to pinned
        # host memory inside every timed ptd_solve call
        t_rb, _ = e2e_run("fp32_rb")
        ttt["fp32_rb"]["e2e_ms_per_step"] = round(t_rb / args.steps * 1e3, 3)
        ttt["fp64_e2e_ms_per_step"] = round(e2e_t / args.steps * 1e3, 3)
        ttt["e2e_speedup"] = round(e2e_t / t_rb, 3)

    if rank != 0:
        return 0
    cb = cpu_baseline(s, shape, budget_s=args.cpu_budget) if world == 1 and not args.no_cpu else None
    ws_gb = (7 if s.ndim == 2 else 9) * np.prod(shape) * 8 / 1e9
    pub = PUBLISHED.get(args.workload) if args.precision == "fp64" else None
    line = {
        "metric": "T_eff", "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_max / max(args.steps, 1) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": round(value / pub, 3) if pub else None,
        "dtype": {"fp64": "f64", "df64": "df64 (f32x2)", "dfh": "f64 state, df64 (f32x2) arithmetic",
                  "fp32_dc": "f32 inner + f64 outer", "fp32_rb": "f32 changes on an f64 base"}[args.precision],
        "data": "synthetic",
        "config": {"workload": args.workload, "shape": list(shape), "precision": args.precision,
                   "nchk": s.nout, "tol": s.tol, "dt": s.dt, "step": "one physical time step to tol",
                   "l2": f"inputs larger than L2 (working set {ws_gb:.2f} GB), no flush",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_kind": peak_kind, "kernel": kernel_name,
                     "launch_us": round(launch_t * 1e6, 2), "algorithmic_bytes_per_launch": kernel_bytes},
        "fp64_pipe": fp64_pipe,
        "cpu_baseline": cb,
        "e2e": {"value": round(e2e_val, 2), "unit": "GB/s", "h2d_bytes_per_step": int(H0.size * 8),
                "d2h_bytes_per_step": int(H0.size * 8)},
        "gpu_launches": int(launches),
        "clocks": clk,
        "pt_iterations_per_step": step_iters,
        "time_to_tol": ttt,
        "dfh": alts.get("dfh"),
        "df64": alts.get("df64"),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="2d_nonlin_4096")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "df64", "dfh", "fp32_dc", "fp32_rb"])
    ap.add_argument("--n", type=int, default=0, help="override the grid size (testing)")
    ap.add_argument("--fixed-iters", type=int, default=200)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-dc", action="store_true", help="skip the FP32+DC time-to-tol comparison")
    ap.add_argument("--no-df64", action="store_true", help="skip the double-float (DFH, DF64) runs")
    ap.add_argument("--adj-tol", type=float, default=1e-10, help="adjoint workload: PT tolerance of the solves")
    ap.add_argument("--fd-directions", type=int, default=20, help="adjoint workload: finite-difference checks")
    ap.add_argument("--fd-eps", type=float, default=1e-3, help="adjoint workload: finite-difference step")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world, rank, local, pg = dist_setup(args.gpus)
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank, pg)
        if args.workload == "batch_linstep_256":
            return run_batch(args, world, rank, local, pg)
        if args.workload == "adjoint_3d_256":
            return run_adjoint(args, world, rank, local, pg)
        return run_ours(args, world, rank, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
