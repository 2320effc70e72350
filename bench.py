"""Benchmark: ms to relative residual 1e-10 on the 2D 1024^2 and 3D 256^3 random-coefficient problems.

One step = one complete solve (coefficient hierarchy + cycles until
||rhs - L_h phi||_2 / ||rhs||_2 <= 1e-10) of the seeded synthetic problem
``jsolver_gb300.workloads.random_2d(1024, seed)``: D_xx, D_yy = exp(GRF sigma 1, corr.
length 0.05), lambda ~ U[0, 10], rhs = L_h sin(pi x) sin(2 pi y). The default run also
measures the 3D half of the metric, ``workload_3d``: ``random_3d(256, seed)`` (D = exp(GRF
sigma 1.2, l 0.08) per axis, lambda = exp(GRF) scaled to [0, 50], rhs = smooth GRF noise
+ a Gaussian source), F-cycles, with the same keys as the 2D line.

Forms (``--form``): ``fp64`` plain FP64 multigrid from phi0 = 0; ``mixed`` FP32 cycles in
FP64 iterative refinement; ``learned`` / ``learned-mixed`` the same from the learned
network's initial guess, whose computation is inside every timed step. ``--outer``:
``richardson`` iterates the cycle as the reference does; ``fcg`` uses the same cycle as
the preconditioner of flexible CG. The default is the headline form, mixed precision
with FCG; every run also times the reference's plain FP64 iteration of the same problem
the same way and reports it under ``plain_fp64``, and in 2D the same form from the
learned guess under ``learned_guess_form`` (the learned + FP32 vs plain FP64 pairing).

Our arm (default): ``value`` is the device time of a solve with inputs resident in HBM,
through the C ABI (jmg_solve), timed with CUDA events on the solving stream; L2 is
flushed (256 MB write) before every timed solve. ``e2e`` is the same solve through the
public API (solve_2d / solve_3d on CUDA tensors) with the host->device copies of the
inputs from pinned memory and the device->host copy of phi and the count inside the
timed region. ``roofline`` is the kernel with the largest share of the solve in the
committed launch list (profiles/launch_shares.json) among those bench.py times alone with
CUDA events: the level-0 sweep, the level-0 fused smooth + restrict (2D), the coarse block
and the FCG step's FP64 residual; ``roofline_others`` holds the rest. ``cpu_baseline`` is the median
time of full solves of the C oracle on all host cores. ``--gpus N`` under torchrun runs
N independent replicas (the path does not shard).

Reference arm (``--impl reference``): the reference's CPU path cannot run here (JAX is
absent), so the oracle's C/OpenMP restatement of it is timed on the host cores, full
solves, same workload and metric (and one full 3D solve under ``workload_3d``).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RTOL = 1e-10
WORKLOADS = {  # name -> (dimension, default resolution, default cycle)
    "2d": (2, 1024, "V"),  # 2D 1024^2 random-coefficient problem (arrays 1027^2 float64)
    "3d": (3, 256, "F"),   # 3D 256^3 random-coefficient problem (arrays 259^3 float64)
    "adjoint": (2, 512, "V"),  # reverse mode: 2D 512^2, fixed 12 V-cycles, loss sum(w phi)
    "adjoint3d": (3, 64, "V"),  # reverse mode: 3D 64^3, fixed 12 V-cycles, loss sum(w phi)
    "batch": (2, 256, "V"),  # many independent 2D 256^2 problems in one batched call
}


def metric_name(dim, m):
    return f"ms to rel. residual 1e-10 ({dim}D {m}^{dim} random-coefficient problem)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "fp64", "mixed", "learned", "learned-mixed"])
    ap.add_argument("--no-compare", action="store_true", help="skip the plain FP64 comparison solve")
    ap.add_argument("--inner-cycles", type=int, default=None,
                    help="FP32 cycles per refinement / FCG step (mixed forms; default 2 with FCG, else 1)")
    ap.add_argument("--outer", default="auto", choices=["auto", "richardson", "fcg"],
                    help="iterate the cycle (reference) or use it as the preconditioner of flexible CG; "
                         "auto: fcg for the mixed and learned forms, richardson for fp64")
    ap.add_argument("--workload", default="2d", choices=sorted(WORKLOADS))
    ap.add_argument("--cycle", default=None, choices=["V", "W", "F"])
    ap.add_argument("--nu1", type=int, default=None,
                    help="pre-smoothing sweeps of the timed form (reference: 1; mixed + FCG default: 1)")
    ap.add_argument("--nu2", type=int, default=None,
                    help="post-smoothing sweeps of the timed form (reference: 1; mixed + FCG default: 5 in 2D, "
                         "3 in 3D)")
    ap.add_argument("--m", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-3d", action="store_true", help="default run: skip the 3D 256^3 block (workload_3d)")
    ap.add_argument("--batch", type=int, default=64, help="problems per step of the batch workload")
    ap.add_argument("--iters", type=int, default=12, help="fixed cycles of the adjoint workload")
    ap.add_argument("--dxy", action="store_true", help="adjoint workload: with D_xy (2D 9-point stencil)")
    ap.add_argument("--lanes", type=int, default=8, help="concurrent lanes of the batch workload")
    a = ap.parse_args()
    dim, m, cyc = WORKLOADS[a.workload]
    a.dim = dim
    a.m = a.m or m
    a.cycle = a.cycle or cyc
    if a.form == "auto":
        a.form = "mixed"
    if a.outer == "auto":
        a.outer = "richardson" if a.form == "fp64" else "fcg"
    if a.inner_cycles is None:
        a.inner_cycles = 1
    return a


def form_nu(args, dim):
    """(nu1, nu2) of the timed form. The mixed + FCG form runs one cycle per FCG step with
    nu1 = 1 and nu2 = 5 in 2D, 3 in 3D: the fastest of a measured sweep (2D 1024^2 V:
    5.75 ms, against 5.79 with (1, 4), 5.88 with (1, 3), 6.25 with two (1, 1) cycles per
    step; 3D 256^3 F: 81.1 ms with (1, 3), (2, 2) or (2, 4), 81.6 with (1, 4), 94.8 with two
    (1, 1) cycles). Every other form keeps the reference's (1, 1); --nu1 / --nu2 override."""
    fcg_mixed = args.outer == "fcg" and args.form in ("mixed", "learned-mixed")
    nu1 = args.nu1 if args.nu1 is not None else 1
    nu2 = args.nu2 if args.nu2 is not None else ((5 if dim == 2 else 3) if fcg_mixed else 1)
    return nu1, nu2


# kernel launches of one learned guess: input pooling, RMS, packing (3); 12 convolutions,
# 3 poolings, 3 up-adds; the output interpolation (1)
GUESS_LAUNCHES = 22


def make_problem(args, seed):
    from jsolver_gb300 import workloads
    return workloads.random_2d(args.m, seed=seed) if args.dim == 2 else workloads.random_3d(args.m, seed=seed)


def coeff_names(dim):
    return ["D_xx", "D_yy"] if dim == 2 else ["D_xx", "D_yy", "D_zz"]


def cycle_kw(c):
    return {"V": {}, "W": {"gamma": 2}, "F": {"fcycle": True}}[c]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """SM clock and clock-event reasons of the GPU, sampled during the timed region.

    NVML is read from a background thread every 5 ms (the timed regions last tens of
    milliseconds); where the NVML library cannot be loaded, nvidia-smi samples every 100 ms.
    Only read-only queries are made: no setting of the GPU is touched. The GPU is found by
    its UUID, so a remapped CUDA_VISIBLE_DEVICES still names the right one."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    POLL_S = 0.005
    NVML_CLOCK_SM = 1
    # nvmlClocksEventReason* bit masks of nvml.h
    REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                   0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index, uuid=None):
        self.index, self.uuid = index, uuid
        self.p = self.nvml = self.thread = None
        self.sm, self.smax, self.reasons, self.out = [], None, set(), ""

    def _nvml_open(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        rc = (nv.nvmlDeviceGetHandleByUUID(f"GPU-{self.uuid}".encode(), ctypes.byref(h)) if self.uuid else 1)
        if rc != 0 and nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
            nv.nvmlShutdown()
            return False
        self.reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if nv.nvmlDeviceGetMaxClockInfo(h, self.NVML_CLOCK_SM, ctypes.byref(mx)) == 0:
            self.smax = float(mx.value)
        self.nvml, self.h = nv, h
        return True

    def _nvml_sample(self):
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        if self.nvml.nvmlDeviceGetClockInfo(self.h, self.NVML_CLOCK_SM, ctypes.byref(clk)) == 0:
            self.sm.append(float(clk.value))
        if self.reasons_fn(self.h, ctypes.byref(rs)) == 0:
            self.reasons.update(n for b, n in self.REASON_BITS.items() if rs.value & b)

    def _nvml_loop(self):
        while not self.stop.wait(self.POLL_S):
            self._nvml_sample()

    def __enter__(self):
        import threading
        try:
            ok = self._nvml_open()
        except (OSError, AttributeError):
            ok = False
        if ok:
            self._nvml_sample()  # one sample before the region starts, so the record is never empty
            self.stop = threading.Event()
            self.thread = threading.Thread(target=self._nvml_loop, daemon=True)
            self.thread.start()
            return self
        self.nvml = None
        try:
            ident = f"GPU-{self.uuid}" if self.uuid else str(self.index)
            self.p = subprocess.Popen(["nvidia-smi", f"--id={ident}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.thread is not None:
            self.stop.set()
            self.thread.join()
            self.nvml.nvmlShutdown()
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out = ""
        return False

    def summary(self):
        if self.nvml is None and self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        if self.p is not None:
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for line in self.out.splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    self.sm.append(float(f[1]))
                    self.smax = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        self.reasons.add(n)
        return {"sm_mhz": float(np.median(self.sm)) if self.sm else None, "sm_max_mhz": self.smax,
                "min_sm_mhz": min(self.sm) if self.sm else None, "reasons": sorted(self.reasons),
                "samples": len(self.sm), "source": "nvml" if self.nvml is not None else "nvidia-smi"}


def gpu_uuid(dev):
    """The CUDA device's UUID as hex digits and dashes (NVML and nvidia-smi take it with
    a 'GPU-' prefix), or None where torch does not report one."""
    import torch
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid).strip()
    except (AttributeError, RuntimeError):
        return None
    u = u[4:] if u.startswith("GPU-") else u
    return u if u and all(c in "0123456789abcdefABCDEF-" for c in u) else None


def cpu_full_solves(p, dim, m, kw, runs, budget_s):
    """Median time of full solves (phi0 = 0 to rel. residual 1e-10, plain FP64 cycles: the
    reference's algorithm) of the C oracle on all host cores: `runs` solves, or fewer once
    `budget_s` seconds have been spent (at least one)."""
    from oracle import c_oracle
    from oracle.grid import OracleGrid1D
    g = OracleGrid1D(m)
    nthreads = os.cpu_count() or 1
    times, counts, rr = [], [], None
    t_start = time.perf_counter()
    for _ in range(max(1, runs)):
        t0 = time.perf_counter()
        _, cnt, rr = c_oracle.solve((g,) * dim, p["phi0"], p["rhs"], p["lam"], tuple(p[k] for k in coeff_names(dim)),
                                    stop="residual", rtol=RTOL, nthreads=nthreads, **kw)
        times.append((time.perf_counter() - t0) * 1e3)
        counts.append(cnt)
        if time.perf_counter() - t_start > budget_s:
            break
    return float(np.median(times)), len(times), counts[-1], rr, nthreads


def cpu_baseline(p, dim, m, kw, runs, budget_s):
    """The reported CPU baseline: the full-solve median of cpu_full_solves."""
    ms, n, cycles, rr, nthreads = cpu_full_solves(p, dim, m, kw, runs, budget_s)
    return {"value": ms, "unit": "ms", "cores": nthreads, "kind": "port",
            "sample": f"median of {n} full solve(s) to rel. residual 1e-10 ({cycles} plain FP64 "
                      f"{'V' if not kw else 'F' if kw.get('fcycle') else 'W'}-cycles from phi0 = 0), C/OpenMP "
                      f"restatement of the reference algorithm (oracle/jmg_oracle.c), {nthreads} threads"}


def reference_arm(args):
    """The reference's algorithm on the host cores: full solves of the C oracle."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    p = make_problem(args, args.seed)
    nthreads = os.cpu_count() or 1
    kw = cycle_kw(args.cycle)
    from oracle import c_oracle
    from oracle.grid import OracleGrid1D
    g = OracleGrid1D(args.m)
    times, counts, rr = [], [], None
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, cnt, rr = c_oracle.solve((g,) * args.dim, p["phi0"], p["rhs"], p["lam"],
                                    tuple(p[k] for k in coeff_names(args.dim)), stop="residual", rtol=RTOL,
                                    nthreads=nthreads, **kw)
        dt = (time.perf_counter() - t0) * 1e3
        if it >= args.warmup:
            times.append(dt)
            counts.append(cnt)
    ms = float(np.median(times))
    line = {
        "metric": metric_name(args.dim, args.m), "value": ms, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded GRF coefficients, manufactured rhs)", "impl": "reference",
        "config": {"workload": workload_name(args.dim, args.m),
                   "cycle": args.cycle, "stop": f"rel. residual <= {RTOL}", "cycles": counts[-1]},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} full solves (median), C/OpenMP restatement of the reference "
                                   f"algorithm (oracle/jmg_oracle.c), {nthreads} threads; the reference's own JAX "
                                   "path cannot run without JAX"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "final_rel_residual": rr,
    }
    if args.workload == "2d" and not args.no_3d:
        # the 3D half of the metric: one full solve (about 25 s on 16 cores)
        dim3, m3, cyc3 = WORKLOADS["3d"]
        from jsolver_gb300 import workloads
        p3 = workloads.random_3d(m3, seed=args.seed)
        ms3, n3, c3, rr3, _ = cpu_full_solves(p3, dim3, m3, cycle_kw(cyc3), 1, 0.0)
        line["workload_3d"] = {
            "metric": metric_name(dim3, m3), "value": ms3, "unit": "ms", "steps": n3, "warmup": 0,
            "config": {"workload": workload_name(dim3, m3), "cycle": cyc3, "stop": f"rel. residual <= {RTOL}",
                       "cycles": c3},
            "cpu_baseline": {"value": ms3, "unit": "ms", "cores": nthreads, "kind": "port",
                             "sample": f"{n3} full solve, C/OpenMP restatement (oracle/jmg_oracle.c), "
                                       f"{nthreads} threads"},
            "e2e": {"value": ms3, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "final_rel_residual": rr3,
        }
    print(json.dumps(line), flush=True)


def max_over_ranks(value, device):
    """The job's time: the maximum of one float over all ranks (every rank gets it)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(seed, rank):
    """Each replica solves its own seeded problem: no data is exchanged between ranks."""
    return seed + rank


def workload_name(dim, m):
    return f"{dim}d-{m}^{dim}-random-coeff (arrays {m + 3}^{dim} float64)"


def adjoint_bench(args):
    """Reverse mode of the fixed-mode solve: forward (--iters V-cycles, 12 by default) and
    backward (the hand-written adjoint) device times, their ratio and the peak device memory
    of one forward + backward, loss = sum(w phi) with seeded Gaussian weights w: the 2D
    random-coefficient problem at 512^2 (workload adjoint; --dxy adds a D_xy field of
    |D_xy| <= 0.3 min(D_xx, D_yy)), or the 3D one at 64^3 (workload adjoint3d)."""
    import torch
    from jsolver_gb300 import workloads
    from jsolver_gb300.grid_1d import grid_1D
    from jsolver_gb300.solver_2d import solve_2d
    from jsolver_gb300.solver_3d import solve_3d
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    m, iters, dim = args.m, args.iters, args.dim
    p = make_problem(args, args.seed)
    g = grid_1D(m)
    w = torch.from_numpy(np.random.default_rng(args.seed + 1).standard_normal(p["rhs"].shape)).to(dev)
    names = ["phi0", "rhs", "lam"] + coeff_names(dim)
    dxy = dim == 2 and args.dxy
    if dxy:
        u = np.random.default_rng(args.seed + 2).uniform(-1, 1, p["rhs"].shape)
        p["D_xy"] = 0.3 * np.minimum(p["D_xx"], p["D_yy"]) * u
        names.append("D_xy")

    def solve(x, **kw):
        if dim == 3:
            return solve_3d(g, g, g, *x, **kw)
        return solve_2d(g, g, *x[:5], D_xy=x[5] if dxy else None, **kw)

    def inputs(grad):
        return [torch.from_numpy(p[k]).to(dev).requires_grad_(grad and k != "phi0") for k in names]

    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    fwd, bwd = [], []
    for it in range(args.warmup + args.steps):
        x = inputs(False)
        e0, e1 = ev(), ev()
        e0.record()
        with torch.no_grad():
            solve(x, fixed=True, max_iters_outer=iters)
        e1.record()
        x = inputs(True)
        phi, _ = solve(x, fixed=True, max_iters_outer=iters)
        loss = (phi * w).sum()
        e2, e3 = ev(), ev()
        e2.record()
        loss.backward()
        e3.record()
        torch.cuda.synchronize()
        if it >= args.warmup:
            fwd.append(e0.elapsed_time(e1))
            bwd.append(e2.elapsed_time(e3))
    # the library keeps the solve's and the adjoint's workspaces across calls: release
    # them so that the measured peak includes both
    from jsolver_gb300 import _engine
    torch.cuda.synchronize()
    _engine.CACHE.ws.clear()
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats(dev)
    base = torch.cuda.memory_allocated(dev)
    x = inputs(True)
    phi, _ = solve(x, fixed=True, max_iters_outer=iters)
    (phi * w).sum().backward()
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated(dev) - base
    f, b = float(np.median(fwd)), float(np.median(bwd))
    stencil = " with D_xy" if dxy else ""
    line = {"metric": f"backward/forward time ratio, reverse mode of the fixed-mode {dim}D solve{stencil} "
                      f"({m}^{dim}, {iters} V-cycles)",
            "value": b / f, "unit": "ratio", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded GRF coefficients, manufactured rhs)",
            "config": {"workload": f"{dim}d-{m}^{dim}-random-coeff{stencil} fixed {iters} V-cycles, "
                                   f"loss = sum(w phi)",
                       "gradients": ", ".join(names[1:]) + " (and phi0)"},
            "forward_ms": f, "backward_ms": b, "peak_device_memory_mb": peak / 2 ** 20,
            "array_mb": p["rhs"].nbytes / 2 ** 20}
    print(json.dumps(line), flush=True)


def batch_bench(args):
    """Many independent solves: ``--batch`` 2D random-coefficient problems at ``--m``
    (256 by default; seeds seed..seed+B-1), each to rel. residual 1e-10, in one
    solve_2d_batched call with ``--lanes`` concurrent lanes, against the same problems
    solved one after another with solve_2d. Inputs resident on the device, L2 flushed
    before every timed step, CUDA events on the calling stream."""
    import torch
    from jsolver_gb300 import workloads
    from jsolver_gb300.grid_1d import grid_1D
    from jsolver_gb300.solver_2d import solve_2d, solve_2d_batched
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    m, nb = args.m, args.batch
    g = grid_1D(m)
    probs = [workloads.random_2d(m, seed=args.seed + b) for b in range(nb)]
    keys = ("phi0", "rhs", "lam", "D_xx", "D_yy")
    X = [torch.from_numpy(np.stack([p[k] for p in probs])).to(dev) for k in keys]
    precision = "mixed" if args.form in ("mixed", "learned-mixed") else "fp64"
    opts = dict(stop="residual", rtol=RTOL, precision=precision, max_iters_outer=20000, outer=args.outer,
                nu1=form_nu(args, 2)[0], nu2=form_nu(args, 2)[1], **cycle_kw(args.cycle))
    if precision == "mixed":
        opts["inner_cycles"] = args.inner_cycles
    flush = torch.empty(256 * 2 ** 20, dtype=torch.uint8, device=dev)

    def timed(fn):
        out = []
        for it in range(args.warmup + args.steps):
            flush.fill_(it & 0xFF)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            torch.cuda.synchronize()
            if it >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return float(np.median(out)), r

    t_b, (phi_b, cnt_b) = timed(lambda: solve_2d_batched(g, g, *X, lanes=args.lanes, **opts))

    def sequential():
        res = [solve_2d(g, g, *[x[b] for x in X], **opts) for b in range(nb)]
        return res

    t_s, res_s = timed(sequential)
    same = all(torch.equal(phi_b[b], res_s[b][0]) and int(cnt_b[b]) == int(res_s[b][1]) for b in range(nb))
    line = {"metric": f"solves/s, {nb} independent 2D {m}^2 random-coefficient problems to rel. residual 1e-10",
            "value": nb / (t_b / 1e3), "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "dtype": "f32+f64" if precision == "mixed" else "f64",
            "data": "synthetic (seeded GRF coefficients, manufactured rhs)",
            "config": {"workload": f"batch of {nb} 2d-{m}^2-random-coeff, {args.cycle}-cycles, "
                                   f"{precision}, outer {args.outer}", "lanes": args.lanes,
                       "nu1": form_nu(args, 2)[0], "nu2": form_nu(args, 2)[1], "inner_cycles": args.inner_cycles,
                       "l2": "flushed (256 MB write) before every step"},
            "ms_per_batch": t_b, "sequential_ms": t_s, "sequential_solves_per_s": nb / (t_s / 1e3),
            "speedup_vs_sequential": t_s / t_b, "cycles_mean": float(cnt_b.double().mean()),
            "identical_to_single_solves": bool(same)}
    print(json.dumps(line), flush=True)


def load_json(name):
    try:
        with open(os.path.join(ROOT, *name.split("/"))) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def level_points(dim, m, levels):
    return [(((m >> l) + 3) ** dim) for l in range(levels)]


def coarse_alg_bytes(dim, m, levels, start, gamma, nu1, nu2, elem):
    """Algorithmic bytes of one coarse sub-cycle launch (a plain cycle from `start` down to
    the deepest level, L-2): per sweep (d+4)*s*N (phi, rhs, d faces, 1/A_cc read; phi
    written), per defect + restriction (d+3)*s*N + s*N_c, per prolongation 2*s*N + s*N_c,
    summed over the recursion's visits (solver_2d.py:582-614)."""
    N = level_points(dim, m, levels)
    last = levels - 2
    sweep = lambda l: (dim + 4) * elem * N[l]  # noqa: E731

    def cyc(l):
        if l == last:
            return (nu1 + nu2) * sweep(l)
        return (nu1 + nu2) * sweep(l) + (dim + 3) * elem * N[l] + 2 * elem * N[l + 1] + 2 * elem * N[l] + \
            gamma * cyc(l + 1)
    return cyc(start)


def timed_alone(fn, stream, flush, n):
    """Mean CUDA-event time (ms) of fn(stream) over n launches, L2 flushed before each."""
    import torch
    evs = []
    for _ in range(n):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn(stream)
        e1.record(stream)
        evs.append((e0, e1))
    stream.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in evs]))


def measure(args, dim, m, cycle, steps, warmup, plain_steps, ws_n, rank, local, dev, learned_cmp_on=True):
    """One workload's line: the form's solve (value, e2e), the plain FP64 comparison, the
    roofline of the dominant kernel and of the other timed kernels, and the CPU baseline."""
    import torch
    import torch.distributed as dist
    from jsolver_gb300 import _engine, _lib, workloads
    from jsolver_gb300.grid_1d import grid_1D
    from jsolver_gb300.solver_2d import solve_2d
    from jsolver_gb300.solver_3d import solve_3d

    cn = coeff_names(dim)
    seed = replica_seed(args.seed, rank)
    p = workloads.random_2d(m, seed=seed) if dim == 2 else workloads.random_3d(m, seed=seed)
    g = grid_1D(m)
    kw = cycle_kw(cycle)
    learned = args.form.startswith("learned") and dim == 2
    precision = "mixed" if args.form in ("mixed", "learned-mixed") else "fp64"
    nu1, nu2 = form_nu(args, dim)
    opts = dict(stop="residual", rtol=RTOL, precision=precision, max_iters_outer=20000, outer=args.outer,
                nu1=nu1, nu2=nu2, **kw)
    if precision == "mixed":
        opts["inner_cycles"] = args.inner_cycles
    lib = _lib.load()
    grid = _engine.make_grid((g,) * dim)
    plan = _lib.Plan(grid, _engine.make_config(**opts))
    stream = torch.cuda.Stream(dev)
    d = {k: torch.from_numpy(p[k]).to(dev) for k in ["phi0", "rhs", "lam"] + cn}
    out = torch.empty_like(d["phi0"])
    start = torch.empty_like(d["phi0"])  # the learned guess
    count = torch.zeros((), dtype=torch.int64, device=dev)
    wsb = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device=dev)
    coeffs = _lib.JmgCoeffs()
    coeffs.lam = d["lam"].data_ptr()
    for k, name in enumerate(cn):
        coeffs.D[k] = d[name].data_ptr()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    vp = ctypes.c_void_p
    net = None
    if learned:
        from jsolver_gb300.learned import GuessNet, WEIGHTS
        net = GuessNet.load(WEIGHTS, device=dev)

    def solve_dev(s, pl=plan, ws=wsb, use_net=learned):
        phi0 = d["phi0"]
        if use_net:
            _lib.check(lib.jmg_net_guess_2d(net.handle, ctypes.byref(grid), ctypes.byref(coeffs),
                                            vp(d["rhs"].data_ptr()), ctypes.c_float(net.out_scale),
                                            vp(start.data_ptr()), vp(s.cuda_stream)))
            phi0 = start
        _lib.check(lib.jmg_solve(pl.handle, vp(phi0.data_ptr()), vp(d["rhs"].data_ptr()), ctypes.byref(coeffs),
                                 vp(out.data_ptr()), vp(count.data_ptr()), vp(ws.data_ptr()),
                                 ctypes.c_size_t(ws.numel()), vp(s.cuda_stream)))

    def timed(fn, n_steps, n_warm):
        for _ in range(n_warm):
            fn(stream)
        stream.synchronize()
        if ws_n > 1:
            dist.barrier()
        torch.cuda.synchronize()
        evs = []
        for _ in range(n_steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(stream)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        if ws_n > 1:
            dist.barrier()
        t_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        return max_over_ranks(t_ms, dev) if ws_n > 1 else t_ms

    def rel_residual(pl, ws):
        rr_t = torch.empty((), dtype=torch.float64, device=dev)
        _lib.check(lib.jmg_rel_residual(pl.handle, vp(out.data_ptr()), vp(d["rhs"].data_ptr()), vp(rr_t.data_ptr()),
                                        vp(ws.data_ptr()), ctypes.c_size_t(ws.numel()), vp(stream.cuda_stream)))
        stream.synchronize()
        return float(rr_t.item())

    with torch.cuda.stream(stream):
        plain = None
        if not args.no_compare and (args.form != "fp64" or args.outer != "richardson"):
            # the plain FP64 multigrid from phi0 = 0 on the same problem, timed the same way
            plan64 = _lib.Plan(grid, _engine.make_config(**dict(opts, precision="fp64", inner_cycles=1,
                                                                outer="richardson", nu1=1, nu2=1)))
            ws64 = torch.empty(plan64.workspace_bytes, dtype=torch.uint8, device=dev)
            f64 = lambda s: solve_dev(s, plan64, ws64, False)  # noqa: E731
            ms64 = timed(f64, plain_steps, max(3, min(warmup, 3)))
            plain = {"ms": ms64, "cycles": int(count.item()), "final_rel_residual": rel_residual(plan64, ws64),
                     "steps": plain_steps}
            del ws64
        with Clocks(local, gpu_uuid(dev)) as clk:
            ms = timed(solve_dev, steps, warmup)
        cycles = int(count.item())
        rel_res = rel_residual(plan, wsb)
        guess_rel_res = None
        if learned:
            solve_dev(stream)  # leaves the guess in `start`
            out.copy_(start)
            guess_rel_res = rel_residual(plan, wsb)
            solve_dev(stream)
        err_exact = (float(np.abs(out.cpu().numpy() - p["phi_exact"]).max()) if "phi_exact" in p else None)
        # the metric's other pairing, learned guess + the same form, timed the same way (2D:
        # the network is 2D); its guess is computed inside every timed solve
        learned_cmp = None
        if learned_cmp_on and not args.no_compare and dim == 2 and not learned:
            from jsolver_gb300.learned import GuessNet, WEIGHTS
            if os.path.exists(WEIGHTS):
                net = GuessNet.load(WEIGHTS, device=dev)
                ms_l = timed(lambda s_: solve_dev(s_, plan, wsb, True), steps, warmup)
                learned_cmp = {"form": f"learned guess + {args.form}", "ms": ms_l,
                               "cycles": int(count.item()) * (args.inner_cycles if precision == "mixed" else 1),
                               "final_rel_residual": rel_residual(plan, wsb),
                               "speedup_vs_plain_fp64": (plain["ms"] / ms_l) if plain else None,
                               "gain_vs_zero_guess": ms / ms_l}
                solve_dev(stream, plan, wsb, False)  # leave the zero-guess form's arrays in the workspace

        # The fine-level red-black sweep of the form's cycles (FP64, or FP32 in the mixed
        # forms; one launch per sweep where the level sweeps in one pass, else colour
        # launches) and the coarse sub-cycle, each timed alone with CUDA events on its
        # stream, L2 flushed before every timed interval. One-pass sweeps alternate two
        # buffers, so they run in pairs.
        fp32 = 1 if precision == "mixed" else 0
        elem = 4 if fp32 else 8
        smooth = lib.jmg_op_smooth32_ws if fp32 else lib.jmg_op_smooth_ws
        launches_per_sweep = lib.jmg_plan_sweep_launches(plan.handle, 0, fp32)
        per = 2 if launches_per_sweep == 1 else 1
        wsa = (vp(wsb.data_ptr()), ctypes.c_size_t(wsb.numel()))
        _lib.check(smooth(plan.handle, 0, 2 * per, *wsa, vp(stream.cuda_stream)))
        sweep_ms = timed_alone(lambda s_: _lib.check(smooth(plan.handle, 0, per, *wsa, vp(s_.cuda_stream))),
                               stream, flush, 20) / per
        n0 = (m + 3) ** dim
        alg_sweep = (dim + 4) * elem * n0  # (d+4)*s*N0: phi, rhs, d faces, 1/A_cc read; phi written
        # the one-pass FP32 3D sweep is k_sweep_tma3d (TMA plane copies) unless JMG_SWEEP3D=regs
        tma = dim == 3 and fp32 and launches_per_sweep == 1 and os.environ.get("JMG_SWEEP3D") != "regs"
        traffic = load_json("profiles/traffic.json").get(
            f"sweep_{'fp32' if fp32 else 'fp64'}_{dim}d_{m}" +
            ("_tma" if tma else "_onepass" if launches_per_sweep == 1 else ""))
        peaks = load_json("MEASURED_PEAKS.json")
        peak = float(peaks.get("hbm_gbs", 6800.0))
        peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
        sweep_kernel = (f"{('k_sweep_tma3d' if tma else 'k_sweep_fused3d') if dim == 3 else 'k_sweep_onepass2d'}"
                        f"<{'float' if fp32 else 'double'}> "
                        "(fine level; one launch per sweep)" if launches_per_sweep == 1 else
                        f"k_sweep_color{dim}d<{'float' if fp32 else 'double'}> (fine level; "
                        f"{launches_per_sweep} launches per sweep)")
        roof_sweep = {"bound": "hbm", "kernel": sweep_kernel,
                      "achieved": alg_sweep / launches_per_sweep / (sweep_ms / launches_per_sweep * 1e-3) / 1e9,
                      "peak": peak, "unit": "GB/s", "peak_source": peak_src,
                      "alg_bytes_per_launch": alg_sweep / launches_per_sweep,
                      "launch_ms": sweep_ms / launches_per_sweep, "traffic": traffic}
        roof_sweep["frac"] = roof_sweep["achieved"] / peak
        cands = {"sweep": roof_sweep}
        if dim == 2 and lib.jmg_plan_level_fused(plan.handle, 0, fp32):
            # level 0 runs the fused pairs: time its smooth + restrict launch (reads phi, rhs,
            # the two face arrays, 1/A_cc and A_cc; writes phi's second buffer and the coarse
            # rhs and phi: (7 N0 + 2 Nc) * s bytes)
            sr = lambda s_: _lib.check(lib.jmg_op_smooth_restrict_ws(plan.handle, 0, fp32, *wsa,  # noqa: E731
                                                                     vp(s_.cuda_stream)))
            sr(stream)
            sr_ms = timed_alone(sr, stream, flush, 20)
            alg_sr = (7 * n0 + 2 * (m // 2 + 3) ** 2) * elem
            cands["smooth_restrict"] = {
                "bound": "hbm", "kernel": f"k_smooth_restrict2d<{'float' if fp32 else 'double'}> (level 0: "
                                          "last pre-sweep + defect + restriction, one launch)",
                "achieved": alg_sr / (sr_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s", "peak_source": peak_src,
                "alg_bytes_per_launch": alg_sr, "launch_ms": sr_ms,
                "traffic": load_json("profiles/traffic.json").get(f"smooth_restrict_{'fp32' if fp32 else 'fp64'}_2d_{m}")}
        if args.outer == "fcg" and precision == "mixed":
            # the exact FP64 residual that ends every FCG step: reads x, rhs, the d face
            # arrays and A_cc (FP64), writes the FP32 residual: ((d + 3) * 8 + 4) * N0 bytes;
            # its d + 4 FP64 operations per point make it FP64-issue-bound as much as
            # bandwidth-bound on GB300
            fr = lambda s_: _lib.check(lib.jmg_op_fcg_residual_ws(plan.handle, *wsa, vp(s_.cuda_stream)))  # noqa: E731
            fr(stream)
            fr_ms = timed_alone(fr, stream, flush, 20)
            alg_fr = ((dim + 3) * 8 + 4) * n0
            cands["fcg_residual"] = {
                "bound": "hbm", "kernel": f"k_fcg32_init<{dim}> (FP64 residual of the FCG step, FP32 copy, "
                                          "partial norms; one launch)",
                "achieved": alg_fr / (fr_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s", "peak_source": peak_src,
                "alg_bytes_per_launch": alg_fr, "launch_ms": fr_ms,
                "traffic": load_json("profiles/traffic.json").get(f"fcg_residual_{dim}d_{m}")}
        for v in cands.values():
            v["frac"] = v["achieved"] / peak
        # the coarse sub-cycle (one launch from the first coarse level down)
        lib.jmg_op_coarse_ws(plan.handle, fp32, *wsa, vp(stream.cuda_stream))
        cstart = lib.jmg_plan_coarse_start(plan.handle)
        coarse_ms = timed_alone(lambda s_: _lib.check(lib.jmg_op_coarse_ws(plan.handle, fp32, *wsa,
                                                                           vp(s_.cuda_stream))), stream, flush, 20)
        cf = _engine.make_config(**opts)
        alg_coarse = coarse_alg_bytes(dim, m, plan.levels, cstart, max(cf.gamma, 1), max(cf.nu1, 0), max(cf.nu2, 0),
                                      elem)
        coarse_name = "k_coarse_cycle" if os.environ.get("JMG_COARSE") else "k_coarse_staged"
        roof_coarse = {"bound": "hbm", "kernel": f"{coarse_name}<{'float' if fp32 else 'double'}, {dim}> "
                                                 f"(1 block: levels {m >> cstart}^{dim} ... {m >> (plan.levels - 2)}"
                                                 f"^{dim} in one launch, staged in shared memory; latency-bound)",
                       "achieved": alg_coarse / (coarse_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                       "peak_source": peak_src, "alg_bytes_per_launch": alg_coarse, "launch_ms": coarse_ms,
                       "traffic": load_json("profiles/traffic.json").get(
                           f"coarse_{'fp32' if fp32 else 'fp64'}_{dim}d_{m}")}
        roof_coarse["frac"] = roof_coarse["achieved"] / peak
        cands["coarse"] = roof_coarse

        # end to end through the public API from pinned host buffers
        host = {k: torch.from_numpy(p[k]).pin_memory() for k in ["phi0", "rhs", "lam"] + cn}
        dst = {k: torch.empty_like(d[k]) for k in host}
        phi_host = torch.empty(out.shape, dtype=torch.float64).pin_memory()
        cnt_host = torch.empty((), dtype=torch.int64).pin_memory()

        def e2e_step(marks=None):
            for k in host:
                dst[k].copy_(host[k], non_blocking=True)
            if marks:
                marks[0].record(stream)
            solve = solve_2d if dim == 2 else solve_3d
            extra = {"guess": net} if learned else {}
            phi, cnt = solve(*((g,) * dim), dst["phi0"], dst["rhs"], dst["lam"], *[dst[k] for k in cn], **opts,
                             **extra)
            if marks:
                marks[1].record(stream)
            phi_host.copy_(phi, non_blocking=True)
            cnt_host.copy_(cnt, non_blocking=True)

        for _ in range(0 if args.no_e2e else 2):
            e2e_step()
        stream.synchronize()
        e2e_t, e2e_parts = [], []
        for _ in range(0 if args.no_e2e else steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            marks = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e0.record(stream)
            e2e_step(marks)
            e1.record(stream)
            e1.synchronize()
            e2e_t.append(e0.elapsed_time(e1))
            e2e_parts.append((e0.elapsed_time(marks[0]), marks[0].elapsed_time(marks[1]), marks[1].elapsed_time(e1)))
        e2e_ms = float(np.mean(e2e_t)) if e2e_t else None
        # mean device time of each part of the end-to-end step: the input copies, the
        # solve call, the result copies
        e2e_split = ({"h2d_ms": float(np.mean([t[0] for t in e2e_parts])),
                      "solve_ms": float(np.mean([t[1] for t in e2e_parts])),
                      "d2h_ms": float(np.mean([t[2] for t in e2e_parts]))} if e2e_parts else None)
        h2d = sum(t.numel() * 8 for t in host.values())
        d2h = phi_host.numel() * 8 + 8

    fixed_n, per_cycle = ctypes.c_int64(), ctypes.c_int64()
    lib.jmg_plan_launch_counts(plan.handle, ctypes.byref(fixed_n), ctypes.byref(per_cycle))
    launches = steps * (fixed_n.value + per_cycle.value * cycles + (GUESS_LAUNCHES if learned else 0))

    # the kernel with the largest share of the solve in the committed launch list (shares
    # per candidate: the level-0 sweep, the level-0 smooth + restrict, the coarse block, the
    # FCG residual); the others beside it
    shares = load_json("profiles/launch_shares.json").get(
        f"{dim}d_{m}_{args.form}_{args.outer}_{cycle}_nu{nu1}{nu2}_x{args.inner_cycles}", {})
    dominant = max(cands, key=lambda k: shares.get(k, 0.0))
    roof = dict(cands[dominant], launch_share=shares.get(dominant))
    roof_others = {k: dict(v, launch_share=shares.get(k)) for k, v in cands.items() if k != dominant}

    line = {
        "metric": metric_name(dim, m), "value": ms, "unit": "ms", "n_gpus": ws_n, "steps": steps,
        "warmup": warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "mixed": "f32+f64", "learned": "bf16+f64", "learned-mixed": "bf16+f32+f64"}[args.form],
        "data": "synthetic (seeded GRF coefficients, manufactured rhs; no dataset in the reference)",
        "config": {"workload": workload_name(dim, m), "cycle": cycle,
                   "form": args.form, "stop": f"rel. residual <= {RTOL}",
                   "cycles": cycles * (args.inner_cycles if precision == "mixed" else 1),
                   "inner_cycles": args.inner_cycles if precision == "mixed" else None, "outer": args.outer,
                   "nu1": nu1, "nu2": nu2,
                   "l2": "flushed (256 MB write) before every timed solve", "parallelism": f"replicas x{ws_n}"},
        "solves_per_s": 1e3 / ms * ws_n,
        "final_rel_residual": rel_res,
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (plain["ms"] / ms) if plain else None,
        "guess_rel_residual": guess_rel_res,
        "learned_guess_form": learned_cmp,
        "max_err_vs_exact_discrete": err_exact,
        "roofline": roof,
        "roofline_others": roof_others,
        "e2e": ({"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                 "split": e2e_split} if e2e_ms is not None else None),
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        # the reference's algorithm (plain FP64 cycles from phi0 = 0), full solves, median;
        # 3D 256^3 takes ~25 s per solve on 16 cores, so one solve there
        line["cpu_baseline"] = cpu_baseline(p, dim, m, kw, runs=3 if dim == 2 else 1, budget_s=20.0)
    return line


def main():
    args = parse()
    if args.workload in ("adjoint", "adjoint3d"):
        return adjoint_bench(args)
    if args.workload == "batch":
        return batch_bench(args)
    if args.impl == "reference":
        return reference_arm(args)
    import torch
    import torch.distributed as dist
    ws_n, rank, local = dist_env()
    if ws_n > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    line = measure(args, args.dim, args.m, args.cycle, args.steps, args.warmup, args.steps, ws_n, rank, local, dev)
    if args.workload == "2d" and not args.no_3d:
        # the 3D half of the metric (3D 256^3, F-cycles, the same form); its plain FP64
        # comparison (about 1.3 s a solve) is timed over at most 5 steps
        dim3, m3, cyc3 = WORKLOADS["3d"]
        torch.cuda.empty_cache()
        line["workload_3d"] = measure(args, dim3, m3, cyc3, args.steps, args.warmup, min(args.steps, 5), ws_n, rank,
                                      local, dev, learned_cmp_on=False)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws_n > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
