"""Benchmark of the accelerated PT diffusion solver (T_eff, the reference's metric).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload suite|3d_nonlin_512|2d_nonlin_4096|
                    1d_lin_512|batch_linstep_256|adjoint_3d_256] [--precision fp64|dfh|df64|fp32_dc|fp32_rb]
                    [--impl ours|reference]

Default (``--workload suite``): the headline is the 3D nonlinear benchmark
problem, D = H^3 on 512^3 cells of a 10^3 domain, H0 = 1 + exp(-r^2), H = 1 on
the boundary, dt = 0.2, tol = 1e-8, 3 physical steps, FP64.  One bench *step*
is one implicit physical time step (the PT iteration driven to err <= tol);
the K timed steps cycle through the problem's 3 steps, the state reset to H0
(untimed) at the start of every cycle.  The same line carries, as
sub-records, the 2D nonlinear 4096^2 problem (5 steps, nchk 100), the 1D
linear 512 problem, the batch of 256 step-diffusion grids and the 3D 256^3
adjoint.

Metric: T_eff = A_eff * iterations / time, with A_eff = (2*3+2)*nx*ny*8 bytes
per PT iteration in 2D and (2*4+2)*nx*ny*nz*8 in 3D -- the reference's own
effective-throughput definition (scripts/diff_2D_nonlin_perf.jl:107,
scripts/diff_3D/diff_3D_nonlin_perf.jl:114), in GB/s (1e9 bytes).

* ``value``: device-resident state, every physical step timed with CUDA
  events on the library's stream (every check and the stopping decision
  included), summed over the K steps.  The working set (9 fields of 1.07 GB)
  is far larger than L2, so no flush is needed.
* ``e2e``: the same metric through the C ABI call a driver makes,
  ``ptd_solve`` on pinned host buffers (H uploaded, one physical step solved,
  H downloaded) per step, wall clock.
* ``roofline``: the fused PT kernel alone (fixed iterations, the reference's
  perf protocol, scripts/diff_3D/diff_3D_nonlin_perf.jl:97-105), A_eff per
  launch over the mean launch time, against the measured HBM copy bandwidth.
* ``forms``: the same problem in the other arithmetic forms (DFH, DF64,
  FP32_RB, FP32_DC), timed over the same leading steps as FP64, with their
  iteration counts, their FP64-equivalent T_eff, their kernel's fraction of
  HBM, and their distance to the FP64 solution and to the converged implicit
  solution (an FP32_RB solve at tol/10).
* ``cpu_baseline`` / ``--impl reference``: the CPU restatement of the
  reference (oracle/, built for the host CPU, OpenMP on all host cores; the
  reference's own Julia Threads backend cannot run here: no Julia) on a
  bounded sample: the reference's perf protocol (a first physical step, then
  a fixed number of PT iterations of the second one timed), as T_eff.
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
GRID_WORKLOADS = ("3d_nonlin_512", "2d_nonlin_4096", "1d_lin_512")
DTYPES = {"fp64": "f64", "df64": "df64 (f32x2)", "dfh": "f64 state, df64 (f32x2) arithmetic",
          "fp32_dc": "f32 inner + f64 outer", "fp32_rb": "f32 changes on an f64 base"}
# ncu summaries holding the DRAM traffic per launch of a form's dominant kernel
TRAFFIC = {("3d_nonlin_512", "fp64"): "pt_kernel_3d_nonlin_512.md",
           ("2d_nonlin_4096", "fp64"): "pt_kernel_2d_nonlin_4096.md",
           ("2d_nonlin_4096", "fp32_rb"): "rb2d_tb2_pair_nonlin_4096.md",
           ("3d_nonlin_512", "fp32_rb"): "rb3d_nonlin_256.md"}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


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


def profile_traffic(summary: str):
    """DRAM bytes per launch of a kernel, from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", summary)
    try:
        with open(path) as fh:
            for ln in fh:
                if ln.startswith("traffic_bytes_per_launch:"):
                    return float(ln.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during a timed region."""

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


def dist_setup():
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


def _reduce(pg, v: float, op: str) -> float:
    if pg is None:
        return v
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=getattr(pg.ReduceOp, op))
    return float(t.item())


def reduce_max(pg, v: float) -> float:
    return _reduce(pg, v, "MAX")


def reduce_sum(pg, v: float) -> float:
    return _reduce(pg, v, "SUM")


def rel_l2(a, b) -> float:
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (CPU restatement of the reference), host-tuned build
def cpu_baseline(s, shape, budget_s=15.0):
    """The reference's perf protocol on the host cores (scripts/diff_3D/diff_3D_nonlin_perf.jl:97-113):
    a first physical step (here a few untimed PT iterations), Hold <- H, then a
    fixed number of PT iterations of the second step timed; T_eff from A_eff."""
    from oracle import oracle as O

    nth = os.cpu_count() or 1
    H0 = __import__("ptdiff").initial_condition(s, *shape)
    H = np.array(H0, order="F")
    q = [np.zeros_like(H) for _ in range(3)]
    t0 = time.perf_counter()
    O.iterate(s, H, H0, q, 2, nthreads=nth, native=True)      # stand-in for step 1
    t_probe = (time.perf_counter() - t0) / 2
    Hold = H.copy(order="F")                                  # assign!(Hold, H) at the end of step 1
    n = int(max(2, min(2000, budget_s / max(t_probe, 1e-9))))
    t0 = time.perf_counter()
    O.iterate(s, H, Hold, q, n, nthreads=nth, native=True)
    dt = time.perf_counter() - t0
    teff = a_eff_bytes(shape) * n / dt / 1e9
    return {"value": round(teff, 3), "unit": "GB/s", "cores": nth, "kind": "port",
            "sample": f"{n} fixed PT iterations (no checks) of physical step 2 of the {len(shape)}D problem "
                      f"{'x'.join(map(str, shape))}, {dt:.1f} s; CPU restatement of the reference "
                      f"(oracle/, OpenMP on {nth} threads, built for the host CPU, one pass per flux and "
                      f"update kernel like the reference); the reference's Julia Threads backend cannot run "
                      f"(no Julia)"}


def run_reference(args, world, rank, pg):
    import ptdiff

    if rank != 0:
        return 0
    wl = "3d_nonlin_512" if args.workload == "suite" else args.workload
    if wl not in ptdiff.scripts.CONFIGS:
        print(json.dumps({"impl": "reference", "unavailable": f"the reference has no {wl} "
                          "workload (batched and adjoint solvers are new here)"}), flush=True)
        return 0
    s = ptdiff.scripts.CONFIGS[wl]
    shape = (args.n or s.default_n,) * s.ndim
    budget = max(4.0, 60.0 / max(args.steps, 1))
    vals, times = [], []
    cb = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cb = cpu_baseline(s, shape, budget_s=budget)
        times.append(time.perf_counter() - t0)
        vals.append(cb["value"])
    value = statistics.median(vals) if vals else 0.0
    cb["value"] = value
    print(json.dumps({
        "impl": "reference", "metric": "T_eff", "value": value, "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(statistics.median(times) * 1e3, 3) if times else None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl, "shape": list(shape), "protocol": "fixed PT iterations of physical step 2"},
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)
    return 0


# ---------------------------------------------------------------------------
# One grid problem: K physical steps cycling through the problem's nt steps
class GridBench:
    def __init__(self, workload, shape, pg, nfix=100):
        import ptdiff

        self.ptdiff = ptdiff
        self.wl = workload
        self.s = ptdiff.scripts.CONFIGS[workload]
        self.shape = shape
        self.nt = max(self.s.nt, 1)
        self.A = a_eff_bytes(shape)
        self.cells = float(np.prod(shape))
        self.H0 = ptdiff.initial_condition(self.s, *shape)
        self.pg = pg
        self.nfix = nfix
        self.peak, self.peak_kind = read_peaks()

    def solver(self, precision, tol=None):
        return self.ptdiff.Solver(self.ptdiff.make_params(self.s, self.shape, nt=1, precision=precision, tol=tol))

    def timed(self, sol, K, W, keep_cycle=True):
        """W untimed physical steps, then K timed ones; step k is step (k mod nt)+1 of
        the problem, the state reset to H0 (untimed) at the start of every cycle.
        Every step timed with CUDA events on the library's stream."""
        import torch

        st = torch.cuda.ExternalStream(sol.stream)
        for k in range(W):
            if k % self.nt == 0:
                sol.set_state(self.H0)
            sol.step(1)
        sol.sync()
        barrier(self.pg)
        torch.cuda.synchronize()
        l0, i0 = sol.counters()
        times, iters, H_cycle = [], [], None
        for k in range(K):
            if k % self.nt == 0:
                sol.set_state(self.H0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            its, _ = sol.step(1)
            e1.record(st)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            iters.append(int(its[0]))
            if keep_cycle and k == min(K, self.nt) - 1:
                H_cycle = sol.get_state()
        torch.cuda.synchronize()
        barrier(self.pg)
        l1, i1 = sol.counters()
        return {"t": times, "iters": iters, "launches": l1 - l0, "iterations": i1 - i0, "H": H_cycle}

    def kernel_time(self, sol, n):
        """Mean time of one PT iteration of the fused kernel alone (fixed
        iterations, no checks): the time of 2n iterations minus that of n, over
        n, so that what a call does once (the rebased form's FP64 rebase around
        its FP32 iterations) drops out."""
        import torch

        st = torch.cuda.ExternalStream(sol.stream)
        sol.set_state(self.H0)
        sol.iterate(8)
        sol.sync()

        def run(k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            sol.iterate(k)
            e1.record(st)
            e1.synchronize()
            return e0.elapsed_time(e1) / 1e3

        return (run(2 * n) - run(n)) / n

    def e2e(self, precision, K, W):
        """ptd_solve on pinned host buffers, one physical step per call, wall clock."""
        import torch

        pin = torch.empty(self.H0.size, dtype=torch.float64, pin_memory=True)
        Hh = pin.numpy()
        sol = self.ptdiff.Solver(self.ptdiff.make_params(self.s, self.shape, nt=1, precision=precision))
        for k in range(W):
            if k % self.nt == 0:
                Hh[:] = np.ravel(self.H0, order="F")
            sol.solve(Hh)
        barrier(self.pg)
        t_tot, its_tot = 0.0, 0
        for k in range(K):
            if k % self.nt == 0:
                Hh[:] = np.ravel(self.H0, order="F")
            t0 = time.perf_counter()
            its, _, _ = sol.solve(Hh)
            t_tot += time.perf_counter() - t0
            its_tot += int(its.sum())
        sol.close()
        return reduce_max(self.pg, t_tot), its_tot

    def kernel_record(self, precision, t_launch):
        """The dominant kernel of a form against the HBM roofline: bytes per launch / launch time."""
        nd = self.s.ndim
        if precision == "fp32_rb":
            # one FP32 iteration reads delta, H_b (FP32), the fluxes omega_d, the
            # base flux defects t_b,d and R_b, writes delta and omega_d: (2+3nd+2)*4 B
            # per cell; a launch runs two iterations (temporal blocking) with an even
            # check cadence in 2D
            tb_ok = nd == 2   # 3D: one iteration per launch unless PTD_FLAG_RB_TBLOCK_3D
            ipl = 2 if tb_ok and self.s.nout % 2 == 0 else 1
            nbytes = (2 + 3 * nd + 2) * 4 * self.cells
            kname = {1: "rb1d_kernel", 2: "rb2d_kernel", 3: "rb3d_kernel"}[nd]
            if ipl == 2:
                kname = "rb2d_tb2_pair_kernel" if nd == 2 and self.s.model in (0, 2) else f"rb{nd}d_tb2_kernel"
            name = f"{kname} ({ipl} FP32 iteration{'s' if ipl > 1 else ''} per launch)"
        else:
            ipl, nbytes = 1, self.A
            name = f"pt{nd}d_kernel<{precision.upper()}> (fused PT iteration)"
        launch = t_launch * ipl
        ach = nbytes / launch / 1e9
        return {"kernel": name, "iterations_per_launch": ipl, "launch_us": round(launch * 1e6, 2),
                "algorithmic_bytes_per_launch": nbytes, "achieved_gbs": round(ach, 1),
                "frac": round(ach / self.peak, 4)}

    def form(self, precision, fp64, Kf, H_fp64, H_conv):
        """A form timed over the first Kf steps FP64 was timed on (one untimed warm-up step)."""
        sol = self.solver(precision)
        r = self.timed(sol, Kf, 1)
        t_launch = self.kernel_time(sol, self.nfix) if precision != "fp32_dc" else None
        sol.close()
        t_f = reduce_max(self.pg, sum(r["t"]))
        t_64 = sum(fp64["t"][:Kf])
        rec = {"ms_per_step": round(t_f / Kf * 1e3, 3), "speedup_vs_fp64": round(t_64 / t_f, 3),
               "steps": Kf, "rel_l2_vs_fp64": rel_l2(r["H"], H_fp64),
               "rel_l2_vs_converged": rel_l2(r["H"], H_conv) if H_conv is not None else None}
        if precision == "fp32_dc":
            rec["fp32_inner_iterations_per_step"] = r["iters"]
        else:
            its = r["iters"]
            rec.update({"pt_iterations_per_step": its, "same_iterations_as_fp64": its == fp64["iters"][:Kf],
                        "teff_fp64_equivalent_gbs": round(reduce_sum(self.pg, self.A * sum(its)) / t_f / 1e9, 2)})
            rec["kernel"] = self.kernel_record(precision, t_launch)
            tr = TRAFFIC.get((self.wl, precision))
            if tr:
                rec["kernel"]["traffic"] = profile_traffic(tr)
        return rec

    def run(self, K, W, forms=True, e2e=True, K_forms=None):
        import torch

        sol = self.solver("fp64")
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
        r = self.timed(sol, K, W)
        clk = clocks.stop()
        H_fp64 = r["H"]
        t_max = reduce_max(self.pg, sum(r["t"]))
        value = reduce_sum(self.pg, self.A * sum(r["iters"])) / t_max / 1e9
        t_launch = self.kernel_time(sol, self.nfix)
        sol.close()
        kr = self.kernel_record("fp64", t_launch)
        traffic = profile_traffic(TRAFFIC[(self.wl, "fp64")]) if (self.wl, "fp64") in TRAFFIC else None
        roofline = {"bound": "hbm", "achieved": kr["achieved_gbs"], "peak": self.peak, "unit": "GB/s",
                    "frac": kr["frac"], "traffic": traffic, "peak_kind": self.peak_kind, "kernel": kr["kernel"],
                    "launch_us": kr["launch_us"], "algorithmic_bytes_per_launch": self.A}
        # the native-FP64 kernel's own ceiling: FP64 instructions per cell x
        # cells / launch time against this GPU's FP64 FMA rate, measured now
        fp64_pipe = None
        per_cell = {2: 18, 3: 26}.get(self.s.ndim) if self.s.model == self.ptdiff.scripts.NONLIN else None
        if per_cell:
            rate = ctypes.c_double(0.0)
            self.ptdiff._abi.check(self.ptdiff._abi.lib().ptd_measure_fp64_rate(ctypes.byref(rate)),
                                   "ptd_measure_fp64_rate")
            ach = per_cell * self.cells / t_launch / 1e9
            fp64_pipe = {"bound": "fp64 pipe", "achieved": round(ach, 1), "peak": round(rate.value / 1e9, 1),
                         "unit": "G FP64 instr/s", "frac": round(ach / (rate.value / 1e9), 4),
                         "instr_per_cell": per_cell, "peak_kind": "measured live (DFMA chains)"}
        out = {"value": value, "t": t_max, "iters": r["iters"], "launches": r["launches"], "clocks": clk,
               "roofline": roofline, "fp64_pipe": fp64_pipe}
        Kf = min(K, K_forms or 2 * self.nt)
        if forms:
            # the converged implicit solution of the problem's nt steps: the
            # rebased form (FP64 counts and accuracy, no FP32 floor) at tol/10
            sc = self.solver("fp32_rb", tol=self.s.tol / 10)
            rc = self.timed(sc, self.nt, 0)
            sc.close()
            H_conv = rc["H"]
            out["fp64_rel_l2_vs_converged"] = rel_l2(H_fp64, H_conv)
            names = ["dfh", "fp32_rb", "fp32_dc"]
            if self.s.ndim == 3 or self.s.ndim == 1:
                names.insert(1, "df64")   # DF64's 48-bit H cannot reach tol on the fine 2D grid
            out["forms"] = {p: self.form(p, r, Kf, H_fp64, H_conv) for p in names}
            torch.cuda.synchronize()
        if e2e:
            t_e, its_e = self.e2e("fp64", K, 1)
            out["e2e"] = {"value": round(reduce_sum(self.pg, self.A * its_e) / t_e / 1e9, 2), "unit": "GB/s",
                          "h2d_bytes_per_step": int(self.H0.size * 8), "d2h_bytes_per_step": int(self.H0.size * 8)}
            if forms:
                t_rb, _ = self.e2e("fp32_rb", Kf, 1)
                t_64 = t_e / K * Kf   # FP64 e2e over the same number of steps
                out["forms"]["fp32_rb"]["e2e_ms_per_step"] = round(t_rb / Kf * 1e3, 3)
                out["forms"]["fp32_rb"]["e2e_speedup_vs_fp64"] = round(t_64 / t_rb, 3)
        return out


def grid_line(args, world, rank, pg, workload, K, W, forms=True, n=0):
    s = __import__("ptdiff").scripts.CONFIGS[workload]
    shape = (n or s.default_n,) * s.ndim
    gb = GridBench(workload, shape, pg, nfix=args.fixed_iters)
    res = gb.run(K, W, forms=forms and not args.no_forms, e2e=True)
    ws_gb = (2 * s.ndim + 3) * np.prod(shape) * 8 / 1e9
    pub = PUBLISHED.get(workload)
    rec = {
        "metric": "T_eff", "value": round(res["value"], 2), "unit": "GB/s",
        "ms_per_step": round(res["t"] / max(K, 1) * 1e3, 3),
        "vs_baseline": round(res["value"] / pub, 3) if pub else None,
        "config": {"workload": workload, "shape": list(shape), "precision": "fp64", "nt": s.nt, "nchk": s.nout,
                   "tol": s.tol, "dt": s.dt,
                   "step": f"one physical time step to tol; the timed steps cycle through the problem's {s.nt} "
                           "steps from H0",
                   "l2": f"inputs larger than L2 (working set {ws_gb:.2f} GB), no flush",
                   "parallelism": f"replicas x{world}"},
        "roofline": res["roofline"], "fp64_pipe": res["fp64_pipe"], "e2e": res["e2e"],
        "gpu_launches": int(res["launches"]), "clocks": res["clocks"], "pt_iterations_per_step": res["iters"]}
    if "forms" in res:
        rec["fp64_rel_l2_vs_converged"] = res["fp64_rel_l2_vs_converged"]
        rec["forms"] = res["forms"]
    return rec, gb


# ---------------------------------------------------------------------------
def run_c1(pg):
    """The 1D linear 512-cell problem (the CPU-runnable configuration): the full
    5-step solve on the GPU through ptd_solve and on the host cores through the
    oracle; the published count of the reference script it shifts is 2020
    (output/out_diff_1D_lin.txt:5)."""
    import ptdiff
    from oracle import oracle as O

    s = ptdiff.scripts.CONFIGS["1d_lin_512"]
    H0 = ptdiff.initial_condition(s, 512)
    sol = ptdiff.Solver(ptdiff.make_params(s, (512,)))
    H = H0.copy(order="F")
    sol.solve(H)   # warm-up
    times, its = [], None
    for _ in range(5):
        H = H0.copy(order="F")
        t0 = time.perf_counter()
        its, _, _ = sol.solve(H)
        times.append(time.perf_counter() - t0)
    sol.close()
    t0 = time.perf_counter()
    Hr, its_r, _, _ = O.solve(s, H0, nthreads=1)
    t_cpu = time.perf_counter() - t0
    return {"workload": "1d_lin_512", "shape": [512], "nt": s.nt, "nchk": s.nout,
            "pt_iterations_per_step": [int(v) for v in its], "pt_iterations_total": int(its.sum()),
            "published_total": 2020, "oracle_iterations_total": int(its_r.sum()),
            "gpu_ms_per_solve": round(statistics.median(times) * 1e3, 3),
            "cpu_ms_per_solve": round(t_cpu * 1e3, 3), "cpu_cores": 1,
            "rel_l2_vs_oracle": rel_l2(H, Hr)}


def _batch_run(prec, world, rank, pg, K, W):
    """K timed batch solves (one physical step each) of the 256-instance batch
    in one precision; the instances are sharded over the ranks by cell count
    (no collective on the data path).  value: the instances' H0 and D resident
    on the device (H0 copied device to device into the solve's fields inside
    the timed region); e2e: H0 and D from pinned host memory and H back into
    it, inside the timed region (the host refill of H0 between steps is not
    timed)."""
    import torch

    import ptdiff
    from ptdiff import dist as PD

    n = 256
    sizes, Hs, Ds = ptdiff.batch_instances(n, seed=0)
    mine = PD.shard_by_cells([int(s) ** 2 for s in sizes], world)[rank]
    sz = [int(sizes[i]) for i in mine]
    p = ptdiff.batch_params(len(mine), model=1, precision=prec, nt=1)
    b = ptdiff.BatchSolver(p, sz, sz)
    w, c, us = b.tune()
    depth = b.config()[2]
    flat = lambda a: torch.from_numpy(np.ravel(a, order="F").copy())
    H0d = [flat(Hs[i]).cuda() for i in mine]
    Dd = [flat(Ds[i]).cuda() for i in mine]
    Hd = [h.clone() for h in H0d]
    # pinned host fields for the end-to-end leg
    H0h = [flat(Hs[i]) for i in mine]
    Hh = [h.clone().pin_memory() for h in H0h]
    Dh = [flat(Ds[i]).pin_memory() for i in mine]

    def dev_step():
        for hd, h0 in zip(Hd, H0d):
            hd.copy_(h0)
        return b.solve(Hd, Dd)

    for _ in range(W):
        dev_step()
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    l0, i0 = b.counters()
    t0 = time.perf_counter()
    err = [0.0]
    iters = None
    for _ in range(K):
        iters, err = dev_step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    l1, i1 = b.counters()
    t_e2e = 0.0
    for _ in range(K):
        for hh, h0 in zip(Hh, H0h):
            hh.copy_(h0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        b.solve(Hh, Dh)
        torch.cuda.synchronize()
        t_e2e += time.perf_counter() - t1
    b.close()
    t_max = reduce_max(pg, dt)
    t_e2e = reduce_max(pg, t_e2e)
    total = reduce_sum(pg, len(mine) * K)
    cells = sum(int(v) ** 2 for v in sz)
    return {"value": round(total / t_max, 3), "ms_per_step": round(t_max / K * 1e3, 3), "steps": K, "warmup": W,
            "e2e": {"value": round(total / t_e2e, 3), "unit": "instances/s", "ms_per_step": round(t_e2e / K * 1e3, 3),
                    "h2d_bytes_per_step": 2 * 8 * cells, "d2h_bytes_per_step": 8 * cells},
            "tuned": {"warps": w, "chunk": c, "iterations_per_launch": depth, "us_per_iter": round(float(us), 2)},
            "gpu_launches": int(l1 - l0), "iterations": int(i1 - i0),
            "max_iterations_of_an_instance": int(np.max(iters)) if iters is not None else 0,
            "max_err_last": float(max(err)), "clocks": clk}


def run_batch_record(args, world, rank, pg, K=3, W=1):
    """The batched 2D step-diffusion workload: 256 instances, sides log-uniform
    in [128, 1024] (seeded), step-function D, tol 1e-8, one implicit step per
    solve.  Metric: instances solved per second.  The suite runs the rebased
    FP32 form (FP32_RB) and, for comparison, the FP32 + FP64 defect correction
    (FP32_DC)."""
    suite = args.workload == "suite"
    prec = args.precision if args.precision in ("fp64", "df64", "fp32_dc", "fp32_rb") and not suite else "fp32_rb"
    r = _batch_run(prec, world, rank, pg, K, W)
    rec = {"metric": "batch instances per second (one implicit step to tol)",
           "value": r["value"], "unit": "instances/s", "steps": K, "warmup": W,
           "ms_per_step": r["ms_per_step"], "dtype": DTYPES[prec],
           "config": {"workload": "batch_linstep_256", "instances": 256, "sides": "log-uniform 128..1024, seed 0",
                      "tol": 1e-8, "precision": prec, "tuned": r["tuned"]},
           "e2e": r["e2e"],
           "gpu_launches": r["gpu_launches"], "iterations": r["iterations"],
           "max_iterations_of_an_instance": r["max_iterations_of_an_instance"], "max_err_last": r["max_err_last"],
           "clocks": r["clocks"]}
    if suite and prec != "fp32_dc":
        d = _batch_run("fp32_dc", world, rank, pg, 2, 1)
        d["speedup_of_" + prec] = round(r["value"] / d["value"], 3) if d["value"] else None
        rec["fp32_dc"] = d
    return rec


def run_adjoint_record(args, world, rank, pg, K=2, W=1):
    """The adjoint workload: 3D D = exp(m) H^3 on 256^3, m a smooth Gaussian
    random field (correlation length 1, std 0.3, seeded), 10 implicit steps of
    dt = 0.1, L2 misfit of H^10 against a target from a perturbed m; one step
    = one gradient evaluation (forward with one checkpoint per physical step +
    adjoint), dL/dm and dL/dH0.  The gradient is checked against central finite
    differences (Richardson-combined) in random directions."""
    import torch

    import ptdiff
    from ptdiff import scripts as S

    n = args.adj_n
    shape = (n,) * 3
    s = S.SCRIPTS["diff_3D_nonlin_multixpu"].with_(
        name="adjoint_3d_256", model=S.NONLIN_EXPM, shift=1.0, dirichlet=1.0, ttot=1.0, dt=0.1,
        tol=args.adj_tol, itmax=20000, ic="linrange")
    H0 = S.initial_condition(s, *shape)
    m = S.log_coefficient_field(shape, seed=0)
    mt = m + S.log_coefficient_field(shape, seed=1)   # the perturbed coefficient of the target
    dev = lambda a: torch.from_numpy(np.ravel(a, order="F").copy()).cuda()
    out = {}
    Ht = None
    head = "fp32_rb"   # FP32 iterations on the change since an FP64 base
    clk = None
    for prec in (head, "df64", "fp64"):
        A = ptdiff.AdjointSolver(ptdiff.make_params(s, shape, precision=prec, nchk=10))
        if Ht is None:
            _, Ht = A.forward(H0, mt, H0, want_HN=True)
        H0d, md, Htd = dev(H0), dev(m), dev(Ht)
        gmd, ghd = torch.empty_like(H0d), torch.empty_like(H0d)
        for _ in range(W):
            A.forward(H0d, md, Htd)
            A.gradient(out_m=gmd, out_H0=ghd)
        torch.cuda.synchronize()
        barrier(pg)
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if prec == head else None
        l0, _ = A.counters()
        t_fwd = t_adj = 0.0
        nsteps = K if prec == head else 1
        fwd_iters = adj_iters = 0
        loss = None
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
        if clocks:
            clk = clocks.stop()
        l1, _ = A.counters()
        res_err, res_target = A.residuals()
        t_tot = reduce_max(pg, t_fwd + t_adj)
        rec = {"grads_per_s": round(world * nsteps / t_tot, 4), "ms_per_gradient": round(t_tot / nsteps * 1e3, 2),
               "forward_ms": round(t_fwd / nsteps * 1e3, 2), "adjoint_ms": round(t_adj / nsteps * 1e3, 2),
               "adjoint_over_forward": round(t_adj / t_fwd, 3),
               "forward_pt_iterations": fwd_iters // nsteps, "adjoint_pt_iterations": adj_iters // nsteps,
               "gpu_launches": int(l1 - l0), "loss": loss,
               "adjoint_final_rel_residual": [float(e / t * 1e-10) if t > 0 else 0.0
                                              for e, t in zip(res_err, res_target)]}
        log(f"adjoint {prec}: forward {rec['forward_ms']:.0f} ms, adjoint {rec['adjoint_ms']:.0f} ms")
        if prec == head:
            gm_h, gh_h = None, None
            t0 = time.perf_counter()
            for _ in range(nsteps):
                A.forward(H0, m, Ht)
                gm_h, gh_h = A.gradient()
            rec["e2e_grads_per_s"] = round(world * nsteps / reduce_max(pg, time.perf_counter() - t0), 4)
            rng = np.random.default_rng(7)
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
                rels.append(abs(fd - gv) / max(abs(gv), 1e-300))
            rec["fd_check"] = {"directions": len(rels), "eps": args.fd_eps,
                               "max_rel_err": max(rels) if rels else None,
                               "median_rel_err": float(np.median(rels)) if rels else None}
        out[prec] = rec
        A.close()
    d = out[head]
    return {"metric": "adjoint gradient evaluations per second", "value": d["grads_per_s"], "unit": "gradients/s",
            "steps": K, "warmup": W, "ms_per_step": d["ms_per_gradient"],
            "dtype": "f32 changes on an f64 base (rebased)",
            "config": {"workload": "adjoint_3d_256", "shape": list(shape), "nt": 10, "dt": 0.1, "tol": s.tol,
                       "model": "D = exp(m) H^3", "m": "Gaussian random field, corr 1, std 0.3, seed 0",
                       "target": "H^10 of m + a second such field (seed 1)", "checkpoints": "one per step"},
            "e2e": {"value": d["e2e_grads_per_s"], "unit": "gradients/s",
                    "h2d_bytes_per_step": int(3 * H0.size * 8), "d2h_bytes_per_step": int(2 * H0.size * 8)},
            "gpu_launches": d["gpu_launches"], "adjoint_over_forward": d["adjoint_over_forward"],
            "fd_check": d["fd_check"], "clocks": clk, "fp32_rb": d, "df64": out["df64"], "fp64": out["fp64"]}


# ---------------------------------------------------------------------------
def run_ours(args, world, rank, local, pg):
    import torch

    torch.cuda.set_device(local)
    wl = "3d_nonlin_512" if args.workload == "suite" else args.workload
    suite = args.workload == "suite"
    if wl == "batch_linstep_256":
        rec = run_batch_record(args, world, rank, pg, K=args.steps, W=args.warmup)
        if rank == 0:
            rec.update({"n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                        "data": "synthetic", "warmup": args.warmup})
            print(json.dumps(rec), flush=True)
        return 0
    if wl == "adjoint_3d_256":
        rec = run_adjoint_record(args, world, rank, pg, K=args.steps, W=args.warmup)
        if rank == 0:
            rec.update({"n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                        "data": "synthetic", "parallelism": f"replicas x{world}"})
            print(json.dumps(rec), flush=True)
        return 0
    if args.precision != "fp64":
        raise SystemExit("--precision other than fp64 is reported under `forms` of the grid workloads")
    t_start = time.perf_counter()
    rec, gb = grid_line(args, world, rank, pg, wl, args.steps, args.warmup, n=args.n)
    log(f"{wl}: {time.perf_counter() - t_start:.0f} s")
    cb = cpu_baseline(gb.s, gb.shape, budget_s=args.cpu_budget) if world == 1 and rank == 0 and not args.no_cpu \
        else None
    line = {"metric": "T_eff", "value": rec["value"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": rec["vs_baseline"], "dtype": "f64", "data": "synthetic", "config": rec["config"],
            "roofline": rec["roofline"], "fp64_pipe": rec["fp64_pipe"], "cpu_baseline": cb, "e2e": rec["e2e"],
            "gpu_launches": rec["gpu_launches"], "clocks": rec["clocks"],
            "pt_iterations_per_step": rec["pt_iterations_per_step"]}
    for k in ("fp64_rel_l2_vs_converged", "forms"):
        if k in rec:
            line[k] = rec[k]
    if suite and world == 1:
        t0 = time.perf_counter()
        c2, _ = grid_line(args, world, rank, pg, "2d_nonlin_4096", 5, 1)
        c2["steps"], c2["warmup"] = 5, 1
        line["c2_2d_nonlin_4096"] = c2
        log(f"2d_nonlin_4096: {time.perf_counter() - t0:.0f} s")
        t0 = time.perf_counter()
        line["c1_1d_lin_512"] = run_c1(pg)
        line["c4_batch_linstep_256"] = run_batch_record(args, world, rank, pg)
        log(f"1d + batch: {time.perf_counter() - t0:.0f} s")
        t0 = time.perf_counter()
        line["c5_adjoint_3d_256"] = run_adjoint_record(args, world, rank, pg)
        log(f"adjoint: {time.perf_counter() - t0:.0f} s")
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="suite",
                    choices=["suite", *GRID_WORKLOADS, "batch_linstep_256", "adjoint_3d_256"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "df64", "dfh", "fp32_dc", "fp32_rb"],
                    help="batch workload: its arithmetic (grid workloads report every form under `forms`)")
    ap.add_argument("--n", type=int, default=0, help="override the grid size of the headline problem (testing)")
    ap.add_argument("--fixed-iters", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the other arithmetic forms")
    ap.add_argument("--adj-n", type=int, default=256, help="adjoint workload: grid size")
    ap.add_argument("--adj-tol", type=float, default=1e-10, help="adjoint workload: PT tolerance of the solves")
    ap.add_argument("--fd-directions", type=int, default=20, help="adjoint workload: finite-difference checks")
    ap.add_argument("--fd-eps", type=float, default=1e-3, help="adjoint workload: finite-difference step")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    world, rank, local, pg = dist_setup()
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank, pg)
        return run_ours(args, world, rank, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
