#!/usr/bin/env python
"""bench.py — SSA velocity solves per second and latency on GB300, mixed precision vs FP64.

Workload: the serving stream.  512 SSA velocity-solve requests arrive as a Poisson process at 200 requests/s,
with grid sizes drawn uniformly from 128x64, 256x128, 512x256 and 1024x512.  Every size covers the same
512 km x 256 km marine ice sheet (dx = 4, 2, 1, 0.5 km).  Each request has a seeded random bed, a Weertman
friction coefficient from its own seed (1000 + request index), Glen n = 3, free-slip walls and a subgrid
grounded fraction.  It is solved with Picard to 1e-6 relative velocity change around multigrid PCG to 1e-8
(coarsening stops at 32 cells; 2 + 2 point sweeps, 20 on the coarsest level), starting from zero.  The mixed
solver runs the multigrid in FP32 under FP64 flexible CG.  The plain FP64 solver runs the multigrid in FP64.

One step is one batch of B consecutive requests of the stream (B = --batch, default 32).  The timed steps
walk the stream from its first request and wrap around after 512.  The warm-up steps come from its end.

  value     solves/s of the mixed solver with every request's inputs staged in HBM before the timed region.
            Up to B solves are in flight on B streams.  A finished solve frees its resident problem for the
            next request at once (continuous batching).  Time runs from the first solve's start event to the
            last one's end event.  Requests of up to 1024x512 keep the working set far above L2, so L2 is not
            flushed.
  batched   with --batch-slots S > 1 (default 8), the same timed requests in batches of up to S requests of one
            grid size (nk_batch: one launch per kernel for the whole batch), beside the headline.
  e2e       the same requests through the C ABI serving loop (nk_server_*) from host buffers, submitted at
            their Poisson arrival times.  Covers upload, geometry, solve and read-back of u and v; host wall
            clock.  p50 and p99 latency run from arrival to result; a second pass over the first requests at 0.8x
            the measured capacity gives the latency at a sustainable arrival rate.
  fp64      the plain FP64 solver one solve at a time, timed on one request of each size.  Its stream rate is
            the stream's size mix divided by those times.
  roofline  the fine-level FP32 l1-Jacobi sweep (the most frequent kernel) on a 2048x1024 grid with L2
            flushed before each launch, against the measured HBM copy bandwidth.  The FP64 CG operator is
            given with its FP64-pipe bound.
  published_scaling  the reference's published multigrid scaling benchmark (one SSA solve to 1e-8 at six grid
            spacings, diagonal and multigrid PCG): iterations and GPU device time beside the published CPU and H200
            times.
  halfpipe_adjoint  the STREAMICE halfpipe adjoint (the reference's gradient benchmark): ∂J/∂xx through three DIVA
            time steps with a partial-cell front by nk_checkpointed_gradient, beside centred differences of the
            library's forward steps and STREAMICE's published cost and gradient; wall times of the gradient and of
            one forward run.
  cpu_baseline  the FP64 CPU restatement of the reference solve (the oracle) on all host cores: one solve of the
            first timed request of each grid size, weighted by the stream's size counts.  The same solves give
            the mixed solver's relative L2 velocity error against the FP64 oracle for every grid size.

`--impl reference` times that CPU restatement alone, on the same stream and config: one FP64 solve per step, the
grid sizes taken in turn, weighted by the stream's size counts.
Multi-GPU: replicas only.  Each rank serves its own copy of the stream; there is no collective on the data
path."""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "nunatak.jl_gb300"))
# concurrent solves use one stream each: 32 hardware work queues instead of 8 (before any CUDA context exists)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "SSA solves/s & p99 latency, mixed vs FP64 on GB300 at <=1e-6 rel velocity error"
WORKLOAD = ("serving stream: 512 marine-sheet SSA solve requests, Poisson arrivals at 200/s, grids uniform over "
            "128x64 / 256x128 / 512x256 / 1024x512 on 512x256 km, friction seed 1000+k per request; Picard reltol 1e-6 x "
            "multigrid PCG reltol 1e-8 (coarsest >= 32 cells); mixed precision (FP32 multigrid, FP64 outer CG / Picard); "
            "steps of {B} consecutive requests")
N_REQUESTS = 512
ARRIVAL_RATE = 200.0
# How the CPU restatement's speed compares with the reference's own CPU code, on the reference's published scaling
# benchmark (docs/src/model/numerics.md:47-48, one thread each, same iteration counts).
ORACLE_CALIBRATION = ("one oracle thread takes 3.7-5.6x the reference's published single-thread time on its multigrid "
                      "scaling benchmark (1 km: 0.85 / 0.55 s diagonal / multigrid against 0.22 / 0.10 s; 0.5 km: 7.0 / 2.4 s "
                      "against 1.9 / 0.43 s; a 2.7 GHz Xeon core against an AMD EPYC 9745 core)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nunatak", choices=["nunatak", "reference"])
    ap.add_argument("--batch", type=int, default=32, help="requests per step, and solves in flight at once")
    ap.add_argument("--batch-slots", type=int, default=8,
                    help="slots of the batched leg reported beside the headline (nk_batch: requests of one grid size solved "
                         "together); 0 or 1: no batched leg")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the oracle solves (CPU baseline and the mixed-vs-oracle errors of every grid size)")
    ap.add_argument("--no-scaling", action="store_true", help="skip the reference's published scaling benchmark rows")
    ap.add_argument("--no-halfpipe", action="store_true", help="skip the STREAMICE halfpipe adjoint of the default line")
    ap.add_argument("--rate", type=float, default=ARRIVAL_RATE,
                    help="Poisson arrival rate of the e2e leg, requests/s (the workload's is 200)")
    ap.add_argument("--profile", choices=["solve", "smoother", "operator", "enthalpy"], default=None,
                    help="profiling runs for ncu: 'solve' = warm-up solves then one timed solve of the workload; "
                         "'smoother' / 'operator' = the roofline kernel on the 2048x1024 grid, 3 launches; "
                         "'enthalpy' = the column energy step on the 1024x512 DIVA sheet (Nσ = 10), 3 launches")
    ap.add_argument("--adjoint", action="store_true",
                    help="the adjoint workload instead: gradient of a velocity misfit with respect to log C on the "
                         "512x256 marine sheet by the fixed-point Picard adjoint, checked against centred differences")
    ap.add_argument("--fd-cells", type=int, default=32, help="cells of the finite-difference check (--adjoint)")
    ap.add_argument("--diva", action="store_true",
                    help="the DIVA workload instead: one solve of the 2048x1024 DIVA sheet (Nσ = 10, Arrhenius A, "
                         "regularised Coulomb drag) in mixed precision and in FP64, from rest")
    ap.add_argument("--timestep", action="store_true",
                    help="the time-step kernels (thickness stage, WENO limiter, energy step) at 2048x1024 against HBM")
    ap.add_argument("--scaling", action="store_true",
                    help="the reference's published multigrid scaling benchmark instead: iterations and device time of "
                         "one SSA solve to 1e-8 at six grid spacings, beside the published numbers")
    ap.add_argument("--halfpipe-adjoint", action="store_true",
                    help="the STREAMICE halfpipe adjoint instead (benchmarks/halfpipe_streamice_adjoint.jl): the gradient "
                         "through three DIVA time steps with a partial-cell front, beside centred differences and STREAMICE's "
                         "published cost and gradient")
    ap.add_argument("--time-gradient", action="store_true",
                    help="the gradient through time steps at scale instead: four steps of the 1024x512 marine sheet "
                         "(mixed precision, a Picard solve after every stage) forward alone and through "
                         "nk_checkpointed_gradient")
    ap.add_argument("--profile-grid", type=int, nargs=2, default=[256, 128], metavar=("NX", "NY"),
                    help="grid of the marine-sheet solve that --profile solve runs")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def rel_l2(ua, va, ub, vb):
    import numpy as np
    return float(math.sqrt(np.sum((ua - ub) ** 2) + np.sum((va - vb) ** 2)) / math.sqrt(np.sum(ub ** 2) + np.sum(vb ** 2)))


def workload(precision, member=0, grid=(256, 128)):
    from nunatak_gb300 import workloads
    return workloads.marine_sheet(grid[0], grid[1], seed=1, seed_friction=1000 + member, precision=precision)


def stream_requests(n, batch, steps, warmup, rate=ARRIVAL_RATE):
    """(warm-up requests, timed requests) of the serving stream: timed steps walk the stream from its start,
    wrapping after N_REQUESTS; warm-up steps take the batches before the stream's end."""
    from nunatak_gb300 import workloads
    stream = workloads.serving_stream(n_requests=n, rate=rate)
    timed = [stream[k % n] for k in range(steps * batch)]
    warm = [stream[(n - warmup * batch + k) % n] for k in range(warmup * batch)]
    return warm, timed


def build_cases(requests, precision):
    """serving_case of every request, built on a thread pool (the FFT filters release the GIL)."""
    import concurrent.futures as cf
    from nunatak_gb300 import workloads
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(lambda r: workloads.serving_case(r, precision), requests))


def cpu_solve(case, threads):
    """One full FP64 solve of the CPU restatement (the oracle) with `threads` OpenMP threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import nunatak_oracle
    used = nunatak_oracle.set_threads(threads)
    P = case.problem(nunatak_oracle.OracleProblem)
    t0 = time.perf_counter()
    st = P.picard_solve()
    dt = time.perf_counter() - t0
    return dt, st, P.get("u"), P.get("v"), used


def replica_throughput(requests, span_ms, world, device):
    """Whole-job solves/s of `world` replicas that each served `requests`: the slowest replica's span (max over
    ranks, one all-reduce of the timing only) divides the requests of all ranks.  Returns (value, span_ms)."""
    if world > 1:
        import torch
        t = torch.tensor([span_ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        span_ms = float(t.item())
    return world * requests / (span_ms / 1e3), span_ms


def stream_config(B, timed_reqs, world):
    """The `config` of both arms' lines: the workload, its timed requests and their grid sizes."""
    count = {}
    for r in timed_reqs:
        key = "%dx%d" % r["size"]
        count[key] = count.get(key, 0) + 1
    return {"workload": WORKLOAD.format(B=B), "requests": len(timed_reqs), "batch": B, "in_flight": B,
            "grids": {k: count[k] for k in sorted(count, key=lambda k: int(k.split("x")[0]))},
            "parallelism": f"replicas{world}",
            "l2": "not flushed: inputs larger than L2 (up to 32 resident 1024x512 problems in flight)"}


def stream_rate(count, seconds_per_solve):
    """Solves/s of the stream's size mix: its requests over the sum of count x seconds per solve of each size."""
    return sum(count.values()) / sum(count[k] * seconds_per_solve[k] for k in count)


def size_rotation(timed_reqs, n):
    """n requests of the timed stream with the grid sizes taken in turn (smallest first): the k-th step of the
    reference arm solves the (k // 4)-th timed request of the (k % 4)-th size."""
    by_size = {}
    for r in timed_reqs:
        by_size.setdefault(r["size"], []).append(r)
    sizes = sorted(by_size)
    return [by_size[sizes[k % len(sizes)]][(k // len(sizes)) % len(by_size[sizes[k % len(sizes)]])] for k in range(n)]


def run_reference(args, rank):
    """`--impl reference`: the reference's CPU path (restated as the FP64 oracle) on all host threads, on the same
    stream, config and metric as the GPU arm.  Every step is one FP64 solve of a timed request, the grid sizes taken
    in turn (128x64, 256x128, 512x256, 1024x512, 128x64, ...), so that every size is timed; the value is the stream's
    size mix over those times (stream_rate).  Warm-up steps solve 128x64 requests."""
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    import __graft_entry__
    from nunatak_gb300 import workloads
    __graft_entry__.build()
    threads = os.cpu_count() or 1
    warm_reqs, timed_reqs = stream_requests(N_REQUESTS, args.batch, args.steps, args.warmup, args.rate)
    config = stream_config(args.batch, timed_reqs, dist_env()[1])
    smallest = [r for r in timed_reqs if r["size"] == workloads.SERVING_SIZES[0]]
    used = threads
    for k in range(args.warmup):
        cpu_solve(workloads.serving_case(smallest[k % len(smallest)], "fp64"), threads)
    times, per_size = [], {}
    for r in size_rotation(timed_reqs, args.steps):
        dt, st, _, _, used = cpu_solve(workloads.serving_case(r, "fp64"), threads)
        times.append(dt)
        per_size.setdefault("%dx%d" % r["size"], []).append(dt)
    mean_s = {k: statistics.mean(v) for k, v in per_size.items()}
    count = {k: n for k, n in config["grids"].items() if k in mean_s}
    value = stream_rate(count, mean_s)
    one_thread = {}
    if args.steps:
        dt1, _, _, _, _ = cpu_solve(workloads.serving_case(smallest[0], "fp64"), 1)
        one_thread = {"128x64_s_per_solve": dt1, "note": "one 128x64 request on one thread (untimed extra)"}
    sample = (f"{args.steps} FP64 solves (oracle restatement of the reference solve, multigrid PCG) of the timed stream's "
              f"requests, one per step, grid sizes in turn ({', '.join(sorted(per_size, key=lambda k: int(k.split('x')[0])))}); "
              f"value = the stream's size mix over the mean time per size")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / max(1, len(times)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded marine ice sheets, no dataset)",
            "config": config,
            "seconds_per_solve": mean_s,
            "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * max(times),
                           "note": "one solve at a time: latency is the solve time"},
            "one_thread": one_thread,
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": used, "kind": "port", "sample": sample,
                             "calibration": ORACLE_CALIBRATION},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# FP64 instructions (DADD + DMUL + DFMA) per cell of the operator apply, from the ncu counts of
# smsp__sass_thread_inst_executed_op_{dadd,dmul,dfma}_pred_on on the 2048x1024 k_apply, regular-grid walk
# (14.0 + 6.4 + 4.5; profiles/operator_fp64_2048x1024.md).
FP64_OPERATOR_INSTR_PER_CELL = 24.9
FP64_INSTR_PER_SM_CLOCK = 2      # GB300 FP64 pipe: 2 thread instructions per SM per clock
SMS = 152


def profile_traffic(name):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from a committed ncu summary's
    `traffic_bytes_per_launch:` line, or None."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    return None


def roofline_problem(nk, workloads, ctx):
    """2048 x 1024 mixed-precision marine sheet with the multigrid state of one short solve."""
    big = workloads.marine_sheet(2048, 1024, seed=1, precision="mixed",
                                 velocity_solver=nk.StressBalanceSolver(
                                     linear_iteration_control=nk.FixedIterations(2), picard_iteration_control=nk.FixedIterations(1),
                                     preconditioner=nk.StressBalanceMultigridPreconditioner(minimum_coarse_size=32), precision="mixed"))
    Pb = big.problem(nk.Problem, context=ctx)
    Pb.picard_solve()
    return Pb


def profile(args, nk, workloads, ctx):
    import numpy as np
    if args.profile == "solve":
        P = workload("mixed", grid=tuple(args.profile_grid)).problem(nk.Problem, context=ctx)
        zu, zv = np.zeros(P.shape("u")), np.zeros(P.shape("v"))
        for _ in range(max(1, args.warmup) + 1):
            P.set("u", zu)
            P.set("v", zv)
            st = P.picard_solve()
        print(json.dumps({"profile": "solve", "picard_iterations": st.picard_iterations, "cg_iterations": st.linear_iterations_total,
                          "device_ms": st.device_ms}))
    elif args.profile == "enthalpy":
        from nunatak_gb300 import model as M
        solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(5), picard_iteration_control=M.FixedIterations(2),
                                       preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=32), precision="mixed")
        case = workloads.diva_sheet(1024, 512, dx=2e3, velocity_solver=solver)
        P = case.problem(nk.Problem, context=ctx)
        P.picard_solve()
        P.velocity_profile()
        P.set("E", 2009.0 * (case.temperature - 223.15))
        ms, by = P.time_kernel("step_enthalpy", repeats=3, flush_bytes=512 << 20)
        P.close()
        print(json.dumps({"profile": "enthalpy", "ms_per_launch": ms, "bytes_per_launch": by}))
    else:
        Pb = roofline_problem(nk, workloads, ctx)
        kernel = "smoother" if args.profile == "smoother" else "operator_fp64"
        ms, by = Pb.time_kernel(kernel, repeats=3, flush_bytes=512 << 20)
        print(json.dumps({"profile": kernel, "ms_per_launch": ms, "bytes_per_launch": by}))


class ResidentPool:
    """Resident mixed-precision problems keyed by grid size.  A request takes a free problem of its size (or a
    new one) and gives it back when its solve has finished."""

    def __init__(self, nk, ctx):
        self.nk, self.ctx, self.free, self.created = nk, ctx, {}, 0

    def take(self, case):
        lst = self.free.setdefault((case.grid.Nx, case.grid.Ny), [])
        if lst:
            return lst.pop()
        self.created += 1
        return case.problem(self.nk.Problem, context=self.ctx)

    def give(self, P):
        self.free[(P.grid.Nx, P.grid.Ny)].append(P)

    def close(self):
        for lst in self.free.values():
            for P in lst:
                P.close()
        self.free = {}


class BatchPool:
    """Resident batches (nk_batch) of `slots` mixed-precision problems keyed by grid size."""

    def __init__(self, nk, ctx, slots):
        self.nk, self.ctx, self.slots, self.free, self.created = nk, ctx, slots, {}, 0

    def take(self, case):
        lst = self.free.setdefault((case.grid.Nx, case.grid.Ny), [])
        if lst:
            return lst.pop()
        self.created += 1
        return self.nk.Batch(case.grid, case.descriptors(), self.slots, context=self.ctx)

    def give(self, B):
        self.free[(B.grid.Nx, B.grid.Ny)].append(B)

    def close(self):
        for lst in self.free.values():
            for B in lst:
                B.close()
        self.free = {}


def stage(cases):
    """Every request's input fields copied to HBM (float64 CUDA tensors), plus zero velocities per grid size."""
    import torch
    staged = [{k: torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)).cuda() for k, v in c.fields.items()}
              for c in cases]
    zeros = {}
    for c in cases:
        key = (c.grid.Nx, c.grid.Ny)
        if key not in zeros:
            nfx, nfy = c.grid.face_count(0), c.grid.face_count(1)
            zeros[key] = (torch.zeros(c.grid.Ny * nfx, dtype=torch.float64, device="cuda"),
                          torch.zeros(nfy * c.grid.Nx, dtype=torch.float64, device="cuda"))
    torch.cuda.synchronize()
    return staged, zeros


def run_resident(pool, cases, staged, zeros, in_flight, keep=()):
    """Continuous batching of `cases` through resident problems: up to `in_flight` solves on the device, the
    next request started as soon as a solve finishes.  Inputs come from HBM (set_field from device memory).
    Returns the per-request stats and the (u, v) of the requests in `keep`."""
    order = list(range(len(cases)))
    running, stats, kept = {}, [None] * len(cases), {}

    def start(k):
        P = pool.take(cases[k])
        for name, t in staged[k].items():
            P.set_device(name, t.data_ptr())
        P.compute_geometry()
        zu, zv = zeros[(cases[k].grid.Nx, cases[k].grid.Ny)]
        P.set_device("u", zu.data_ptr())
        P.set_device("v", zv.data_ptr())
        P.picard_solve_async()
        running[id(P)] = (P, k)

    while order or running:
        while order and len(running) < in_flight:
            start(order.pop(0))
        finished = [(P, k) for P, k in running.values() if P.query()]
        for P, k in finished:
            stats[k] = P.wait()
            if k in keep:
                kept[k] = (P.get("u"), P.get("v"))
            del running[id(P)]
            pool.give(P)
        if not finished:
            time.sleep(0.0002)
    return stats, kept


def run_batched(pool, cases, staged, zeros, in_flight, keep=()):
    """run_resident with batches: the oldest queued request and the next queued ones of its grid size (up to the
    batch's slots and the requests allowed in flight) share one batched solve; a finished batch takes the next group
    at once.  Returns the per-request stats and the (u, v) of the requests in `keep`."""
    queue = list(range(len(cases)))
    running, stats, kept, n_running = {}, [None] * len(cases), {}, 0
    size = lambda k: (cases[k].grid.Nx, cases[k].grid.Ny)

    def start(ks):
        B = pool.take(cases[ks[0]])
        for slot, k in enumerate(ks):
            P = B.problem(slot)
            for name, t in staged[k].items():
                P.set_device(name, t.data_ptr())
            P.compute_geometry()
            zu, zv = zeros[size(k)]
            P.set_device("u", zu.data_ptr())
            P.set_device("v", zv.data_ptr())
        B.picard_solve_async(list(range(len(ks))))
        running[id(B)] = (B, ks)

    while queue or running:
        while queue and n_running < in_flight:
            room = min(pool.slots, in_flight - n_running)
            key = size(queue[0])
            ks = [k for k in queue if size(k) == key][:room]
            for k in ks:
                queue.remove(k)
            start(ks)
            n_running += len(ks)
        finished = [(B, ks) for B, ks in running.values() if B.query()]
        for B, ks in finished:
            st = B.wait()
            for slot, k in enumerate(ks):
                stats[k] = st[slot]
                if k in keep:
                    kept[k] = (B.problem(slot).get("u"), B.problem(slot).get("v"))
            del running[id(B)]
            n_running -= len(ks)
            pool.give(B)
        if not finished:
            time.sleep(0.0002)
    return stats, kept


def arrival_times(requests, rate=ARRIVAL_RATE):
    """Arrival of each request in seconds; a wrapped pass of the stream arrives after the previous one."""
    from nunatak_gb300 import workloads
    period = workloads.serving_stream(n_requests=N_REQUESTS, rate=rate)[-1]["arrival"] + 1.0 / rate
    out, passes, last = [], 0, -1
    for r in requests:
        if r["index"] <= last:
            passes += 1
        last = r["index"]
        out.append(r["arrival"] + passes * period)
    return out


def run_server(S, cases, arrivals):
    """Submit each case at its arrival time (host clock), drive the serving loop, collect every result.
    Returns (throughput solves/s, latencies ms from arrival to result, stats)."""
    t_host0 = time.perf_counter()
    t_srv0 = S.clock()
    tickets = []
    for case, t in zip(cases, arrivals):
        while time.perf_counter() - t_host0 < t:
            S.progress()
            time.sleep(0.0002)
        tickets.append(S.submit(case))
    res = [S.wait(tk) for tk in tickets]
    done = [r[3][2] - t_srv0 for r in res]
    lat = [1e3 * (d - t) for d, t in zip(done, arrivals)]
    return len(cases) / (max(done) - arrivals[0]), lat, [r[2] for r in res]


def cost_difference(up, vp, um, vm, uo, vo, mu_u, mu_v):
    """J(+) - J(-) for J = ½ Σ_ice (u - u_obs)² + (v - v_obs)², written as ½ Σ (u₊ - u₋)(u₊ + u₋ - 2 u_obs): the two
    costs are never formed, so the difference keeps the digits that subtracting two rounded sums of 10⁵ terms loses."""
    du, dv = (up - um) * mu_u, (vp - vm) * mu_v
    return 0.5 * (float(np.sum(du * (up + um - 2 * uo) * mu_u)) + float(np.sum(dv * (vp + vm - 2 * vo) * mu_v)))


def fd_cells(grad, n, seed, floor=1e-3):
    """n seeded cells among those whose adjoint gradient is at least `floor` of the largest: a centred difference
    can only resolve a cell whose gradient stands above the solver's and the arithmetic's noise."""
    cand = np.argwhere(np.abs(grad) >= floor * np.max(np.abs(grad)))
    rng = np.random.default_rng(seed)
    return [tuple(int(c) for c in cand[k]) for k in rng.choice(len(cand), size=min(n, len(cand)), replace=False)]


def run_adjoint(args, nk, workloads, ctx):
    """The adjoint workload: J = ½ Σ_ice (u - u_obs)² + (v - v_obs)² in (m/yr)² on the 512x256 (1 km) marine sheet,
    u_obs from a solve with friction seed 2000 plus 1 % Gaussian noise; ∂J/∂log C at every cell by nk_picard_adjoint
    (mixed precision: FP32 multigrid inside FP64 CG); centred differences of converged solves at 32 seeded cells
    whose gradient is at least 1e-3 of the largest, each cell's relative error reported, with the workload's step
    ε = 1e-6 and with ε = 1e-3.  Solves use Picard 1e-14 and CG 1e-14 (the adjoint 1e-12), so that the perturbed
    solves leave less noise than the differences resolve: at ε = 1e-6 a cell's velocities move by about 1e-6 of its
    share of the response, close to what FP64 solves can separate, so ε = 1e-3 is the resolved comparison."""
    import torch
    from nunatak_gb300 import model as M
    nx, ny = 512, 256
    yr2 = workloads.YEAR ** 2
    tight = nk.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-14, maxiter=5000),
                                   picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=1000),
                                   preconditioner=nk.StressBalanceMultigridPreconditioner(minimum_coarse_size=32), precision="mixed")
    case = workloads.marine_sheet(nx, ny, seed=1, seed_friction=1000, velocity_solver=tight)
    obs = workloads.marine_sheet(nx, ny, seed=1, seed_friction=2000, velocity_solver=tight).problem(nk.Problem, context=ctx)
    obs.picard_solve()
    rng = np.random.default_rng(3)
    uo, vo = obs.get("u"), obs.get("v")
    uo = uo * (1 + 0.01 * rng.standard_normal(uo.shape))
    vo = vo * (1 + 0.01 * rng.standard_normal(vo.shape))
    obs.close()
    P = case.problem(nk.Problem, context=ctx)
    mu = P.get("ice_mask")
    mu_u = (np.maximum(np.pad(mu, ((0, 0), (1, 0)), mode="edge"), np.pad(mu, ((0, 0), (0, 1)), mode="edge")) > 0).astype(float)
    mu_v = (np.maximum(np.pad(mu, ((1, 0), (0, 0)), mode="edge"), np.pad(mu, ((0, 1), (0, 0)), mode="edge")) > 0).astype(float)

    P.picard_solve()
    zu, zv = np.zeros(P.shape("u")), np.zeros(P.shape("v"))
    P.set("u", zu)
    P.set("v", zv)
    fwd = P.picard_solve()
    xs = (P.get("u"), P.get("v"))
    du, dv = (xs[0] - uo) * mu_u, (xs[1] - vo) * mu_v
    J0 = 0.5 * yr2 * (float(np.sum(du * du)) + float(np.sum(dv * dv)))
    ub, vb = yr2 * du, yr2 * dv                           # ∂J/∂u, ∂J/∂v with J in (m/yr)²
    control = M.Convergence(reltol=1e-12, maxiter=1000)
    P.picard_adjoint(ub, vb, control)                 # warm-up (graph capture of the linear solve)
    torch.cuda.synchronize()
    _, _, grad, _, ast = P.picard_adjoint(ub, vb, control)
    cells = fd_cells(grad, args.fd_cells, 5)
    ad = [float(grad[c]) for c in cells]
    scale = float(np.max(np.abs(grad)))
    checks = {}
    for eps in (1e-6, 1e-3):
        probs = []
        for cell in cells:
            for sgn in (1.0, -1.0):
                Q = case.problem(nk.Problem, context=ctx)
                C = case.fields["C"].copy()
                C[cell] *= math.exp(sgn * eps)
                Q.set("C", C)
                Q.set("u", xs[0])
                Q.set("v", xs[1])
                probs.append(Q)
        vel = []
        for k in range(0, len(probs), 32):
            batch = probs[k:k + 32]
            for Q in batch:
                Q.picard_solve_async()
            for Q in batch:
                Q.wait()
                vel.append((Q.get("u"), Q.get("v")))
                Q.close()
        fd = [yr2 * cost_difference(*vel[2 * n], *vel[2 * n + 1], uo, vo, mu_u, mu_v) / (2 * eps) for n in range(len(cells))]
        rel = [abs(a - f) / abs(a) for a, f in zip(ad, fd)]
        checks["eps=%g" % eps] = {"max_rel_err_per_cell": max(rel), "median_rel_err_per_cell": float(np.median(rel)),
                                  "cells_within_1e-4": int(sum(r <= 1e-4 for r in rel)),
                                  "cells": [[int(c[0]), int(c[1]), a, f, r] for c, a, f, r in zip(cells, ad, fd, rel)]}
    print(json.dumps({
        "metric": "adjoint gradient of the velocity misfit w.r.t. log C (fixed-point Picard adjoint) vs centred differences",
        "config": {"workload": "marine_sheet 512x256 dx=1km, u_obs from friction seed 2000 + 1% noise, J over ice points in (m/yr)^2",
                   "precision": "mixed (FP32 multigrid, FP64 CG and adjoint residual)", "fd_cells": len(cells),
                   "cell_selection": "seeded among cells with |dJ/dlog C| >= 1e-3 max|dJ/dlog C|",
                   "fd_formula": "(J+ - J-) / 2 eps with J+ - J- = 1/2 sum (u+ - u-)(u+ + u- - 2 u_obs)",
                   "tolerances": "Picard 1e-14, CG 1e-14, adjoint 1e-12"},
        "forward_ms": fwd.device_ms, "forward_picard_iterations": fwd.picard_iterations,
        "adjoint_ms": ast.device_ms, "adjoint_iterations": ast.picard_iterations, "adjoint_cg_iterations": ast.linear_iterations_total,
        "adjoint_status": ast.status, "J": J0, "max_abs_gradient": scale, "finite_differences": checks}), flush=True)


def run_diva(nk, workloads, ctx):
    """The DIVA workload: the 2048x1024 (1 km) DIVA sheet with Nσ = 10, the Arrhenius rate factor of the seeded
    temperature field, regularised Coulomb drag (α² = 0.5, m = 1/3) and a front at x = 1900 km, solved from rest
    with Picard 1e-6 x multigrid PCG 1e-8, once in mixed precision and once in FP64 (after a first solve that
    captures the CUDA graph).  Reports device time per solve, iterations, the mixed-vs-FP64 velocity error and the
    transition speed (α² N / C)^(1/m) that the reference's regularised Coulomb law implies at grounded cells."""
    nx, ny = 2048, 1024
    res, vel = {}, {}
    for prec in ("mixed", "fp64"):
        P = workloads.diva_sheet(nx, ny, precision=prec).problem(nk.Problem, context=ctx)
        zu, zv = np.zeros(P.shape("u")), np.zeros(P.shape("v"))
        P.picard_solve()                                  # graph capture and warm-up
        P.set("u", zu)
        P.set("v", zv)
        st = P.picard_solve()
        res[prec] = {"ms_per_solve": st.device_ms, "picard_iterations": st.picard_iterations,
                     "cg_iterations": st.linear_iterations_total, "status": st.status}
        vel[prec] = (P.get("u"), P.get("v"))
        if prec == "fp64":
            N, C, phi, H = P.get("N"), P.get("C"), P.get("phi"), P.get("H")
            grounded = (phi > 0.5) & (H > 0) & (N > 0)
            ut = (0.5 * N[grounded] / C[grounded]) ** 3 * workloads.YEAR
            transition = {"p10": float(np.percentile(ut, 10)), "median": float(np.median(ut)), "p90": float(np.percentile(ut, 90))}
        P.close()
    (um, vm), (u6, v6) = vel["mixed"], vel["fp64"]
    err = float(np.sqrt(np.sum((um - u6) ** 2) + np.sum((vm - v6) ** 2)) / np.sqrt(np.sum(u6 ** 2) + np.sum(v6 ** 2)))
    print(json.dumps({
        "metric": "DIVA velocity solve time on GB300, mixed vs FP64",
        "config": {"workload": "diva_sheet 2048x1024 dx=1km, Nsigma=10 (faces (k/10)^2), Arrhenius A from T(zeta) = 270 - 17 zeta "
                               "+ 3 K x seeded field, regularised Coulomb (alpha^2 = 0.5, m = 1/3), front at x = 1900 km; "
                               "Picard 1e-6 x multigrid PCG 1e-8, from rest"},
        "mixed": res["mixed"], "fp64": res["fp64"], "speedup_mixed_vs_fp64": res["fp64"]["ms_per_solve"] / res["mixed"]["ms_per_solve"],
        "rel_error_mixed_vs_fp64": err, "max_speed_m_per_yr": float(np.max(np.abs(u6)) * workloads.YEAR),
        "coulomb_transition_speed_m_per_yr": transition}), flush=True)


def halfpipe_adjoint(nk, workloads, ctx):
    """The STREAMICE halfpipe adjoint (benchmarks/halfpipe_streamice_adjoint.jl:66-99) with the benchmark's tolerances
    (Picard 1e-8, CG 1e-10, the adjoint at the Picard control): J and ∂J/∂xx at the four centreline cells from
    nk_checkpointed_gradient, centred differences of the library's forward steps with the benchmark's ε = 0.1 m/yr, and
    STREAMICE's published values (tests/golden/halfpipe_streamice.json).  Times: one gradient call and one forward run
    (the three steps alone), wall clock on the host."""
    with open(os.path.join(ROOT, "tests", "golden", "halfpipe_streamice.json"), encoding="utf-8") as f:
        spec = json.load(f)
    weights = spec["control_weights"]
    cells = [(j - 1, i - 1) for i, j in spec["check_cells_julia"]]
    P, year, st = workloads.halfpipe_problem(nk.Problem, spec, context=ctx)
    t0 = time.perf_counter()
    g = P.checkpointed_gradient(workloads.halfpipe_cost(year), 0.2 * year, 3, melt_weights=weights)
    t_grad = time.perf_counter() - t0

    def cost(control=None):
        Q, _, _ = workloads.halfpipe_problem(nk.Problem, spec, context=ctx)
        return workloads.halfpipe_forward_cost(Q, year, weights, control)

    t0 = time.perf_counter()
    J = cost()
    t_fwd = time.perf_counter() - t0
    rows = []
    for k, cell in enumerate(cells):
        xx = np.zeros((spec["Ny"], spec["Nx"]))
        xx[cell] = 0.1
        fd = (cost(xx) - cost(-xx)) / 0.2
        ad = float(g["melt"][cell] / year)
        sad, sfd = spec["streamice_adjoint_gradient"][k], spec["streamice_finite_difference"][k]
        rows.append({"cell_julia": list(spec["check_cells_julia"][k]), "adjoint": ad, "finite_difference": fd,
                     "rel_adjoint_vs_fd": (ad - fd) / abs(fd), "streamice_adjoint": sad, "streamice_finite_difference": sfd,
                     "ratio_to_streamice_adjoint": ad / sad})
    return {"metric": "STREAMICE halfpipe adjoint: dJ/dxx through 3 DIVA time steps with a partial-cell front",
            "J": g["J"], "J_forward": J, "streamice_cost": spec["streamice_cost"],
            "ratio_to_streamice_cost": g["J"] / spec["streamice_cost"], "rows": rows,
            "gradient_wall_s": t_grad, "forward_wall_s": t_fwd, "gradient_over_forward": t_grad / t_fwd,
            "stats": g["stats"]}


def run_halfpipe_adjoint(nk, workloads, ctx):
    print(json.dumps(halfpipe_adjoint(nk, workloads, ctx)), flush=True)


def run_time_gradient(nk, workloads, ctx, nx=1024, ny=512, steps=4):
    """The gradient through time steps at scale: the 1024x512 marine sheet in mixed precision (Picard 1e-6 x multigrid
    PCG 1e-8), a surface mass balance of 0.3 m/yr and a basal melt of 1 m/yr under floating ice, four steps of half the
    advective time scale of the first solve's velocities (the sheet's margin is fast), with a Picard solve after every
    stage, J = Σ H² after the last.  Times (host wall clock, the device synchronised):
    the forward steps alone from the same state, and one nk_checkpointed_gradient call (its forward, the segments'
    re-runs and the reverse sweep with a Picard adjoint per solve); the gradient's magnitude per field."""
    case = workloads.marine_sheet(nx, ny, precision="mixed")
    year = workloads.YEAR
    weights = None

    def fresh():
        P = case.problem(nk.Problem, context=ctx)
        P.energy_set("surface_mass_balance", 0.3 / year)
        P.energy_set("basal_melt_rate", 1.0 / year)
        P.energy_set("clipped_thickness", 0.0)
        st = P.picard_solve()
        return P, st

    P, st0 = fresh()
    dx, dy = 512e3 / nx, 256e3 / ny
    u, v = np.abs(P.get("u")), np.abs(P.get("v"))
    dt = 0.5 / float(np.max(u[:, :nx] / dx + v[:ny, :] / dy))
    t0 = time.perf_counter()
    for _ in range(steps):
        for stage in (1, 2, 3):
            P.step_thickness_stage(dt, stage)
            P.picard_solve()
    H = P.get("H")
    t_fwd = time.perf_counter() - t0
    J_fwd = float(np.sum(H * H))
    P.close()
    P, _ = fresh()

    def cost(step, H, u, v, mask):
        return (float(np.sum(H * H)), 2 * H, None, None) if step == steps else None

    t0 = time.perf_counter()
    g = P.checkpointed_gradient(cost, dt, steps, melt_weights=weights)
    t_grad = time.perf_counter() - t0
    print(json.dumps({
        "metric": "gradient through time steps at scale (nk_checkpointed_gradient)",
        "config": {"workload": "marine_sheet %dx%d (500 m), mixed precision, Picard 1e-6 x multigrid PCG 1e-8, a 0.3 m/yr, "
                               "m 1 m/yr (floating), %d steps of %.4g yr (half the advective time scale), a Picard solve after "
                               "every stage, J = sum H^2" % (nx, ny, steps, dt / year)},
        "forward_wall_s": t_fwd, "gradient_wall_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
        "J": g["J"], "J_forward": J_fwd, "rel_J_difference": abs(g["J"] - J_fwd) / J_fwd,
        "max_abs": {k: float(np.max(np.abs(g[k]))) for k in ("H", "u", "v", "smb", "melt", "log_C", "log_A")},
        "stats": g["stats"]}), flush=True)


def run_scaling(nk, workloads, ctx, problem_cls=None, rows=None, quiet=False):
    """The reference's published multigrid scaling benchmark (benchmarks/multigrid_scaling.jl; its table in
    docs/src/model/numerics.md:42-49, kept in tests/golden/reference_scaling.json): the MISMIP+-like ice stream
    at six spacings, five Picard iterations of multigrid PCG to 1e-6 from rest, then one SSA solve of the last
    coefficients from zero to 1e-8 with the diagonal and with the multigrid preconditioner (FP64, and the
    multigrid also in mixed precision).  Each timed solve follows an untimed one of the same system (graph
    capture).  Reports device milliseconds and iterations per row beside the published H200 seconds."""
    from nunatak_gb300 import model as M
    cls = problem_cls or nk.Problem
    with open(os.path.join(ROOT, "tests", "golden", "reference_scaling.json"), encoding="utf-8") as f:
        table = json.load(f)["rows"]
    out = []
    for row in table if rows is None else [r for r in table if r["dx_m"] in rows]:
        case = workloads.mismip_stream(row["dx_m"])
        P = case.problem(cls, context=ctx) if ctx is not None else case.problem(cls)
        P.picard_solve()
        coefficients = {k: P.get(k) for k in ("eta_H", "eta_H_ff", "beta_u", "beta_v")}
        tau = P.get("tau_u"), P.get("tau_v")
        P.close()
        entry = {"dx_m": row["dx_m"], "grid": [row["nx"], row["ny"]],
                 "published": {"diagonal_iterations": row["diagonal_iterations"], "diagonal_cpu_gpu_s": row["diagonal_cpu_gpu_s"],
                               "multigrid_iterations": row["multigrid_iterations"], "multigrid_cpu_gpu_s": row["multigrid_cpu_gpu_s"]}}
        for name, pre, prec in (("diagonal", M.StressBalanceDiagonalPreconditioner(), "fp64"),
                                ("multigrid", M.StressBalanceMultigridPreconditioner(), "fp64"),
                                ("multigrid_mixed", M.StressBalanceMultigridPreconditioner(), "mixed")):
            solver = M.StressBalanceSolver(preconditioner=pre, precision=prec, picard_iteration_control=M.FixedIterations(1),
                                           linear_iteration_control=M.Convergence(reltol=1e-8, maxiter=100_000))
            c2 = workloads.Case("mismip_stream", case.grid, dict(case.config, velocity_solver=solver), case.fields)
            Q = c2.problem(cls, context=ctx) if ctx is not None else c2.problem(cls)
            for k, value in coefficients.items():
                Q.set(k, value)
            for _ in range(2):                           # the first solve captures the graph
                Q.set("u", 0.0)
                Q.set("v", 0.0)
                st = Q.linear_solve(*tau)
            entry[name] = {"iterations": st.linear_iterations_last, "device_ms": st.device_ms, "status": st.status}
            Q.close()
        out.append(entry)
    if quiet:
        return out
    print(json.dumps({
        "metric": "one SSA solve from zero to 1e-8 (reference multigrid scaling benchmark): CG iterations and device time",
        "config": {"workload": "MISMIP+-like ice stream of benchmarks/multigrid_scaling.jl (640 x 80 km, bed and thickness "
                               "formulas of the benchmark, calving front at 600 km), coefficients after 5 Picard iterations "
                               "of multigrid PCG to 1e-6 from rest",
                   "published": "docs/src/model/numerics.md:42-49: CPU = one thread of an AMD EPYC 9745, GPU = one H200"},
        "rows": out}), flush=True)
    return out


def timestep_kernels(nk, workloads, ctx, peak):
    """The time-step kernels on the 2048x1024 DIVA sheet (Nσ = 10, the workload's geometry, temperature and drag) after
    a short solve and its velocity profile, L2 flushed before each launch: one Runge-Kutta stage of the thickness step
    with first-order upwinding and with the default bounded WENO-5, the bounded WENO's limiter, and the column energy
    step from the enthalpy of the seeded temperature.  Algorithmic bytes per launch over CUDA-event time against the
    measured HBM bandwidth."""
    from nunatak_gb300 import model as M
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(5), picard_iteration_control=M.FixedIterations(2),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=32), precision="mixed")
    case = workloads.diva_sheet(2048, 1024, velocity_solver=solver)
    P = case.problem(nk.Problem, context=ctx)
    P.picard_solve()
    P.velocity_profile()
    P.set("E", 2009.0 * (case.temperature - 223.15))
    out = {}
    for name, kernel, adv in (("thickness_stage_upwind1", "thickness_stage", M.UpwindBiased(order=1)),
                              ("thickness_stage_weno5_bounded", "thickness_stage", M.default_thickness_advection()),
                              ("thickness_faces_weno5", "thickness_faces", M.default_thickness_advection()),
                              ("thickness_limiter", "thickness_limiter", M.default_thickness_advection()),
                              ("step_enthalpy", "step_enthalpy", None)):
        if adv is not None:
            P.set_thickness_advection(adv)
        P.time_kernel(kernel, repeats=2, flush_bytes=0)
        ms, by = P.time_kernel(kernel, repeats=10, flush_bytes=512 << 20)
        gbs = by / (ms * 1e-3) / 1e9
        out[name] = {"ms_per_launch": ms, "bytes_per_launch": by, "achieved_gbs": gbs, "frac_of_hbm": gbs / peak}
    P.close()
    return {"grid": "2048x1024, Nsigma = 10 (DIVA sheet), L2 flushed before each launch", "kernels": out}


# Algorithmic bytes per cell of the solve's repeated work (each array a kernel touches, once, at its precision):
# the FP64 flexible CG iteration (operator 65 B, update 104 B, dots after the V-cycle 32 B, xpby 48 B), the FP32
# V-cycle (about 62 four-byte words per fine cell, times 4/3 for the coarse levels) and the SSA coefficient update
# of each Picard iteration (15 eight-byte words).
CG_BYTES_PER_CELL = 65 + 104 + 32 + 48
VCYCLE_BYTES_PER_CELL = int(round(62 * 4 / 3 * 4))
COEF_BYTES_PER_CELL = 15 * 8


def stream_algorithmic_bytes(cells, picard_iterations, cg_iterations):
    """Σ over requests of cells × (Picard iterations × coefficient bytes + CG iterations × (CG + V-cycle bytes))."""
    return float(sum(n * (p * COEF_BYTES_PER_CELL + c * (CG_BYTES_PER_CELL + VCYCLE_BYTES_PER_CELL))
                     for n, p, c in zip(cells, picard_iterations, cg_iterations)))


def main():
    args = parse()
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    sys.path.insert(0, ROOT)
    import numpy as np
    import torch
    import __graft_entry__
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local_rank)
    __graft_entry__.build()
    import nunatak_gb300 as nk
    from nunatak_gb300 import library, workloads

    ctx = library.Context(local_rank)
    if args.profile:
        profile(args, nk, workloads, ctx)
        return
    if args.adjoint:
        if rank == 0:
            run_adjoint(args, nk, workloads, ctx)
        return
    if args.diva:
        if rank == 0:
            run_diva(nk, workloads, ctx)
        return
    if args.scaling:
        if rank == 0:
            run_scaling(nk, workloads, ctx)
        return
    if args.halfpipe_adjoint:
        if rank == 0:
            run_halfpipe_adjoint(nk, workloads, ctx)
        return
    if args.time_gradient:
        if rank == 0:
            run_time_gradient(nk, workloads, ctx)
        return
    if args.timestep:
        if rank == 0:
            print(json.dumps({"metric": "time-step kernels vs HBM", **timestep_kernels(nk, workloads, ctx, measured_peaks()[0])}), flush=True)
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    B = args.batch
    warm_reqs, timed_reqs = stream_requests(N_REQUESTS, B, args.steps, args.warmup, args.rate)
    warm_cases = build_cases(warm_reqs, "mixed")
    cases = build_cases(timed_reqs, "mixed")
    config = stream_config(B, timed_reqs, world)
    count = config["grids"]
    first_of_size = {}
    for k, c in enumerate(cases):
        first_of_size.setdefault("%dx%d" % (c.grid.Nx, c.grid.Ny), k)

    # ---- value: the timed requests with inputs staged in HBM, continuous batching of B in flight --------------
    def stream_leg(pool, runner, warm, timed):
        """One pass over the timed requests (after one over the warm-up requests) with inputs staged in HBM."""
        w_staged, w_zeros = stage(warm)
        runner(pool, warm, w_staged, w_zeros, B)
        del w_staged, w_zeros
        staged, zeros = stage(timed)
        barrier()
        created0 = pool.created
        launches0 = library.launch_count()
        with ClockSampler(local_rank) as clocks:
            t0 = time.perf_counter()
            stats, kept = runner(pool, timed, staged, zeros, B, keep=set(first_of_size.values()))
            barrier()
            wall = time.perf_counter() - t0
        launches = library.launch_count() - launches0
        span_ms = max(x.device_end_ms for x in stats) - min(x.device_start_ms for x in stats)
        value, span_ms = replica_throughput(len(timed), span_ms, world, "cuda")
        leg = {"value": value, "span_ms": span_ms, "stats": stats, "kept": kept, "clocks": clocks, "wall": wall,
               "launches": launches, "service": [x.device_end_ms - x.device_start_ms for x in stats],
               "created": pool.created - created0}
        pool.close()
        del staged, zeros
        torch.cuda.empty_cache()
        return leg

    def leg_summary(leg, mode):
        return {"value": leg["value"], "unit": "solves/s", "ms_per_step": leg["span_ms"] / args.steps, "wall_s": leg["wall"],
                "gpu_launches": int(leg["launches"]),
                "latency_ms": {"p50": statistics.median(leg["service"]), "p99": float(np.percentile(leg["service"], 99))},
                "cg_iterations_per_solve": {"min": min(x.linear_iterations_total for x in leg["stats"]),
                                            "max": max(x.linear_iterations_total for x in leg["stats"])},
                "mode": mode}

    head = stream_leg(ResidentPool(nk, ctx), run_resident, warm_cases, cases)
    batched = None
    if args.batch_slots > 1:
        # the same requests in batches: requests of one grid size share one batched graph (nk_batch)
        b_leg = stream_leg(BatchPool(nk, ctx, args.batch_slots), run_batched, warm_cases, cases)
        batched = leg_summary(b_leg, f"requests of one grid size solved together, up to {args.batch_slots} per batched graph "
                                     f"(nk_batch; one launch per kernel for every slot), {B} requests in flight")
        batched["rel_error_vs_headline"] = {key: rel_l2(*b_leg["kept"][k], *head["kept"][k]) for key, k in first_of_size.items()}
        del b_leg
    value, span_ms, stats, kept, clocks = head["value"], head["span_ms"], head["stats"], head["kept"], head["clocks"]
    wall, launches, service, created_timed = head["wall"], head["launches"], head["service"], head["created"]

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    # ---- fp64: the plain FP64 solver one solve at a time, one request of each size ----------------------------
    fp64_ms, rel_err = {}, {}
    for key, k in first_of_size.items():
        P64 = workloads.serving_case(timed_reqs[k], "fp64").problem(nk.Problem, context=ctx)
        zu, zv = np.zeros(P64.shape("u")), np.zeros(P64.shape("v"))
        P64.picard_solve()                  # warm-up: graph capture
        P64.set("u", zu)
        P64.set("v", zv)
        st = P64.picard_solve()
        fp64_ms[key] = st.device_ms
        um, vm = kept[k]
        rel_err[key] = rel_l2(um, vm, P64.get("u"), P64.get("v"))
        P64.close()
    fp64_value = stream_rate(count, {k: fp64_ms[k] / 1e3 for k in count})

    # ---- e2e: the same requests through the serving loop of the C ABI, host buffers, Poisson arrivals ---------
    from nunatak_gb300.server import Server
    S = Server(max_in_flight=B, memory_cap_bytes=64 << 30, context=ctx)
    for c in warm_cases:
        S.submit(c)
    S.wait_all()
    arrivals = arrival_times(timed_reqs, args.rate)
    e2e_value, e2e_lat, e2e_stats = run_server(S, cases, arrivals)
    # the same server at a sustainable arrival rate (0.8 x the capacity just measured) on the first requests, so that
    # the latency describes the server and not the queue of an overloaded stream
    sus_rate = 0.8 * e2e_value
    n_sus = min(len(cases), max(B, int(round(10.0 * sus_rate))))
    sus_arrivals = arrival_times(timed_reqs[:n_sus], sus_rate)
    _, sus_lat, _ = run_server(S, cases[:n_sus], sus_arrivals)
    sinfo = S.info()
    S.close()
    h2d = sum(sum(np.asarray(v).nbytes for v in c.fields.values()) for c in cases) / args.steps
    d2h = sum(8 * (c.grid.Ny * c.grid.face_count(0) + c.grid.face_count(1) * c.grid.Nx) for c in cases) / args.steps
    e2e_err = max(abs(a.picard_iterations - b.picard_iterations) for a, b in zip(stats, e2e_stats))

    piters = [x.picard_iterations for x in stats]
    citers = [x.linear_iterations_total for x in stats]
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": span_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (multigrid) + f64 (CG, Picard)", "data": "synthetic (seeded marine ice sheets, no dataset)",
        "config": config,
        "timing": {"wall_s": wall, "problems_created_in_timed_region": created_timed},
        "batched": batched,
        "latency_ms": {"p50": statistics.median(service), "p99": float(np.percentile(service, 99)),
                       "note": "device time of each solve (start to end event) while sharing the GPU with the others"},
        "picard_iterations": {"min": min(piters), "max": max(piters)},
        "cg_iterations_per_solve": {"min": min(citers), "max": max(citers)},
        "fp64": {"value": fp64_value, "unit": "solves/s", "ms_per_solve": fp64_ms,
                 "mode": "plain FP64 solver (FP64 multigrid PCG) one solve at a time; stream rate from one timed solve "
                         "of each grid size weighted by the stream's size counts"},
        "speedup_mixed_vs_fp64": value / world / fp64_value,
        "speedup_e2e_vs_fp64": e2e_value / fp64_value,
        "rel_error_mixed_vs_fp64_gpu": rel_err,
        "roofline": None,
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "latency_ms": {"p50": statistics.median(e2e_lat), "p99": float(np.percentile(e2e_lat, 99)),
                               "note": f"arrival (Poisson, {args.rate:g}/s) to result on the host; arrivals exceed capacity, "
                                       "so this is mostly queueing"},
                "latency_ms_sustainable": {"rate_per_s": sus_rate, "requests": n_sus,
                                           "p50": statistics.median(sus_lat), "p99": float(np.percentile(sus_lat, 99)),
                                           "note": "the first requests of the stream at Poisson arrivals of 0.8 x the "
                                                   "measured e2e capacity, arrival to result on the host"},
                "path": "nk_server_submit / nk_server_wait (host inputs, upload, geometry, solve, read-back)",
                "picard_iteration_mismatch_vs_resident": e2e_err, "server": sinfo},
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }

    # ---- roofline of the most frequent kernel on a grid larger than L2 ----------------------------------------
    peak, peak_kind = measured_peaks()
    Pb = roofline_problem(nk, workloads, ctx)
    Pb.time_kernel("smoother", repeats=3, flush_bytes=0)
    sm_ms, sm_bytes = Pb.time_kernel("smoother", repeats=20, flush_bytes=512 << 20)
    op_ms, op_bytes = Pb.time_kernel("operator_fp64", repeats=20, flush_bytes=512 << 20)
    Pb.close()
    achieved = sm_bytes / (sm_ms * 1e-3) / 1e9
    sm_mhz = line["clocks"].get("sm_mhz") or 2070.0
    fp64_rate = FP64_OPERATOR_INSTR_PER_CELL * 2048 * 1024 / (op_ms * 1e-3) / 1e9
    fp64_peak = FP64_INSTR_PER_SM_CLOCK * SMS * sm_mhz * 1e6 / 1e9
    line["roofline"] = {
        "bound": "hbm", "kernel": "fine-level FP32 l1-Jacobi sweep (k_smooth_point<float>), 2048x1024, L2 flushed",
        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
        "traffic": profile_traffic("smoother_fp32_2048x1024.md"), "bytes_per_launch": sm_bytes, "ms_per_launch": sm_ms,
        "operator_fp64": {"kernel": "k_apply (FP64 operator, 2048x1024, L2 flushed)", "ms_per_launch": op_ms,
                          "achieved_gbs": op_bytes / (op_ms * 1e-3) / 1e9, "bound": "fp64 pipe",
                          "fp64_ginstr_per_s": fp64_rate, "fp64_peak_ginstr_per_s": fp64_peak, "frac": fp64_rate / fp64_peak,
                          "traffic": profile_traffic("operator_fp64_2048x1024.md")}}
    # ---- the stream as a whole: algorithmic bytes of every request's iterations over the device span ------------
    stream_bytes = stream_algorithmic_bytes([c.grid.Nx * c.grid.Ny for c in cases], piters, citers)
    stream_gbs = stream_bytes / (span_ms * 1e-3) / 1e9 * world
    line["roofline_stream"] = {
        "achieved": stream_gbs, "peak": peak, "unit": "GB/s", "frac": stream_gbs / (peak * world), "peak_source": peak_kind,
        "bytes": stream_bytes,
        "model": "per request and cell: Picard iterations x %d B (SSA coefficient update, 15 words FP64) + CG iterations x "
                 "(%d B FP64 flexible CG iteration + %d B FP32 V-cycle, 62 words x 4/3 levels)"
                 % (COEF_BYTES_PER_CELL, CG_BYTES_PER_CELL, VCYCLE_BYTES_PER_CELL)}
    line["roofline_timestep"] = timestep_kernels(nk, workloads, ctx, peak)
    # ---- the reference's published scaling benchmark: GPU device times beside the published H200 and CPU times ----
    if not args.no_scaling:
        line["published_scaling"] = run_scaling(nk, workloads, ctx, quiet=True)
    # ---- the reference's gradient benchmark through the time steps ----
    if not args.no_halfpipe:
        line["halfpipe_adjoint"] = halfpipe_adjoint(nk, workloads, ctx)
    # ---- the FP64 CPU restatement (the oracle): one solve of each size, the parity of the mixed solves against it and
    # the CPU baseline of the stream's size mix -----------------------------------------------------------------------
    if not args.no_cpu_baseline:
        cpu_s, errs, used = {}, {}, 1
        for key, k in first_of_size.items():
            dt, _, uo, vo, used = cpu_solve(workloads.serving_case(timed_reqs[k], "fp64"), os.cpu_count() or 1)
            cpu_s[key] = dt
            errs[key] = rel_l2(kept[k][0], kept[k][1], uo, vo)
        line["cpu_baseline"] = {"value": stream_rate(count, cpu_s), "unit": "solves/s", "cores": used, "kind": "port",
                                "calibration": ORACLE_CALIBRATION, "seconds_per_solve": cpu_s,
                                "sample": "one FP64 solve (oracle restatement, multigrid PCG, OpenMP on all host cores) of the "
                                          "first timed request of each grid size; value = the stream's size mix over those times"}
        line["rel_error_mixed_vs_fp64_oracle"] = {key: errs[key] for key in errs}
        line["rel_error_mixed_vs_fp64_oracle_requests"] = {key: int(timed_reqs[k]["index"]) for key, k in first_of_size.items()}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()


if __name__ == "__main__":
    main()
