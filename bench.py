#!/usr/bin/env python
"""bench.py — SSA velocity solves per second on GB300 (mixed precision vs FP64).

Workload: the marine ice sheet on a 256 x 128 grid at 2 km (seeded random bed, Weertman friction with a
seeded random coefficient, Glen n = 3, free-slip walls, subgrid grounded fraction), Picard to 1e-6 relative
velocity change around multigrid PCG to 1e-8 (levels 256x128, 128x64, 64x32, 32x32; 2 + 2 point sweeps, 20
on the coarsest).  One step solves a batch of B ensemble members (the same geometry, friction seeds 1000+k)
from a zero initial guess.  The mixed solver runs the multigrid preconditioner in FP32 under FP64 flexible
conjugate gradients, the B members concurrently on B streams; the plain FP64 solver is timed on the same
members one solve at a time.

  value     solves/s of the mixed solver, inputs resident in HBM, CUDA events (first start to last end of the
            batch), L2 flushed (256 MiB write) between steps; latency p50 / p99 of the individual solves
  e2e       the same batch through the serving loop of the C ABI (nk_server_*) from host buffers: upload of
            H, bed, C, A, geometry, solve, read-back of u and v, host wall clock
  roofline  the dominant kernel (the fine-level FP32 ℓ1-Jacobi sweep) timed with CUDA events on a 2048 x 1024
            grid with L2 flushed before each launch, against the measured HBM copy bandwidth
  cpu_baseline  the FP64 CPU restatement of the reference solve (the oracle) on the host cores, one full solve

`--impl reference` times that CPU restatement alone (all host threads, full solves of the same workload).
Multi-GPU: replicas only (each rank solves its own batch; no collective on the data path)."""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "nunatak.jl_gb300"))
# concurrent solves use one stream each: 32 hardware work queues instead of 8 (before any CUDA context exists)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "SSA solves/s & p99 latency, mixed vs FP64 on GB300 at <=1e-6 rel velocity error"
WORKLOAD = ("marine_sheet 256x128 dx=2km (seeded bed + Weertman C), ensemble batch of {B} friction seeds per step, "
            "Picard reltol 1e-6 x multigrid PCG reltol 1e-8, 4 levels, mixed precision (FP32 multigrid, FP64 outer CG / Picard)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nunatak", choices=["nunatak", "reference"])
    ap.add_argument("--batch", type=int, default=32, help="ensemble members solved concurrently per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", choices=["solve", "smoother", "operator"], default=None,
                    help="profiling runs for ncu: 'solve' = warm-up solves then one timed solve of the workload; "
                         "'smoother' / 'operator' = the roofline kernel on the 2048x1024 grid, 3 launches")
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


def run_reference(args, rank):
    """`--impl reference`: the reference's CPU path (restated as the FP64 oracle) on all host threads."""
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    import __graft_entry__
    __graft_entry__.build()
    threads = os.cpu_count() or 1
    case = workload("fp64")
    for _ in range(args.warmup):
        cpu_solve(case, threads)
    times = []
    used = threads
    for _ in range(args.steps):
        dt, st, _, _, used = cpu_solve(case, threads)
        times.append(dt)
    total = sum(times)
    value = args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded marine ice sheet)",
            "config": {"workload": WORKLOAD.replace("mixed precision (FP32 multigrid, FP64 outer CG / Picard)", "FP64 throughout"),
                       "grid": [256, 128]},
            "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * max(times)},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": used, "kind": "port",
                             "sample": f"{args.steps} full FP64 solves (oracle restatement of the reference solve)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    else:
        Pb = roofline_problem(nk, workloads, ctx)
        kernel = "smoother" if args.profile == "smoother" else "operator_fp64"
        ms, by = Pb.time_kernel(kernel, repeats=3, flush_bytes=512 << 20)
        print(json.dumps({"profile": kernel, "ms_per_launch": ms, "bytes_per_launch": by}))


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

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    B = args.batch
    cases = [workload("mixed", k) for k in range(B)]
    probs = [c.problem(nk.Problem, context=ctx) for c in cases]
    zu, zv = np.zeros(probs[0].shape("u")), np.zeros(probs[0].shape("v"))

    def batch_step(ps):
        """Solve every problem of `ps` concurrently from zero; returns (device span ms, per-solve stats)."""
        for p in ps:
            p.set("u", zu)
            p.set("v", zv)
        flush.random_(0, 255)
        torch.cuda.synchronize()
        for p in ps:
            p.picard_solve_async()
        st = [p.wait() for p in ps]
        span = max(x.device_end_ms for x in st) - min(x.device_start_ms for x in st)
        return span, st

    for _ in range(args.warmup):
        batch_step(probs)

    # ---- timed region: K batches of B mixed-precision solves on resident inputs ----------------------
    spans, solves = [], []
    barrier()
    launches0 = library.launch_count()
    with ClockSampler(local_rank) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            span, st = batch_step(probs)
            spans.append(span)
            solves.extend(st)
        barrier()
        wall = time.perf_counter() - t0
    launches = library.launch_count() - launches0
    busy = sum(spans) / 1e3
    if world > 1:
        t = torch.tensor([busy], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        busy = float(t.item())
    value = world * args.steps * B / busy
    lat = [x.device_ms for x in solves]
    u_mixed, v_mixed = probs[0].get("u"), probs[0].get("v")

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    # ---- the plain FP64 solver, one solve at a time, on the same members -----------------------------------
    n64 = min(B, 4)
    s64 = []
    P64s = [workload("fp64", k).problem(nk.Problem, context=ctx) for k in range(n64)]
    for k, P64 in enumerate(P64s):
        P64.set("u", zu)
        P64.set("v", zv)
        if k == 0:
            P64.picard_solve()          # warm-up (graph capture)
            P64.set("u", zu)
            P64.set("v", zv)
        flush.random_(0, 255)
        torch.cuda.synchronize()
        s64.append(P64.picard_solve())
    fp64_value = len(s64) / (sum(x.device_ms for x in s64) / 1e3)
    u64, v64 = P64s[0].get("u"), P64s[0].get("v")
    del P64s

    # ---- end to end through the serving loop with host buffers --------------------------------------------
    from nunatak_gb300.server import Server
    S = Server(max_in_flight=B, memory_cap_bytes=8 << 30, context=ctx)
    for c in cases[:2]:
        S.wait(S.submit(c))             # warm-up: resident problems and their graphs
    e2e_times, e2e_lat = [], []
    for _ in range(args.steps):
        flush.random_(0, 255)
        torch.cuda.synchronize()
        t = time.perf_counter()
        tickets = [S.submit(c) for c in cases]
        res = [S.wait(tk) for tk in tickets]
        e2e_times.append(time.perf_counter() - t)
        e2e_lat.extend(1e3 * (r[3][2] - r[3][0]) for r in res)
    e2e_value = args.steps * B / sum(e2e_times)
    sinfo = S.info()
    S.close()
    h2d = B * sum(np.asarray(v).nbytes for v in cases[0].fields.values())
    d2h = B * (zu.nbytes + zv.nbytes)

    # ---- roofline of the dominant kernel on a grid larger than L2 ---------------------------------------
    peak, peak_kind = measured_peaks()
    Pb = roofline_problem(nk, workloads, ctx)
    Pb.time_kernel("smoother", repeats=3, flush_bytes=0)
    sm_ms, sm_bytes = Pb.time_kernel("smoother", repeats=20, flush_bytes=512 << 20)
    op_ms, op_bytes = Pb.time_kernel("operator_fp64", repeats=20, flush_bytes=512 << 20)
    achieved = sm_bytes / (sm_ms * 1e-3) / 1e9
    del Pb

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * busy / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (multigrid) + f64 (CG, Picard)", "data": "synthetic (seeded marine ice sheet, no dataset)",
        "config": {"workload": WORKLOAD.format(B=B), "grid": [256, 128], "dx_m": 2000.0, "batch": B,
                   "parallelism": f"replicas{world}", "l2": "flushed between steps (256 MiB write outside the timed events)",
                   "wall_s": wall},
        "latency_ms": {"p50": statistics.median(lat), "p99": float(np.percentile(lat, 99)), "max": max(lat),
                       "note": "per solve, device events; all B members start together"},
        "picard_iterations": solves[-1].picard_iterations, "cg_iterations_per_solve": solves[-1].linear_iterations_total,
        "fp64": {"value": fp64_value, "unit": "solves/s", "ms_per_solve": 1e3 / fp64_value, "solves_timed": len(s64),
                 "mode": "plain FP64 solver (FP64 multigrid PCG), one solve at a time",
                 "picard_iterations": s64[-1].picard_iterations, "cg_iterations_per_solve": s64[-1].linear_iterations_total},
        "speedup_mixed_vs_fp64": value / world / fp64_value,
        "rel_error_mixed_vs_fp64_gpu": rel_l2(u_mixed, v_mixed, u64, v64),
        "roofline": {"bound": "hbm", "kernel": "fine-level FP32 l1-Jacobi sweep (k_smooth_point<float>), 2048x1024, L2 flushed",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": None, "bytes_per_launch": sm_bytes, "ms_per_launch": sm_ms,
                     "operator_fp64": {"ms_per_launch": op_ms, "achieved_gbs": op_bytes / (op_ms * 1e-3) / 1e9}},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "latency_ms": {"p50": statistics.median(e2e_lat), "p99": float(np.percentile(e2e_lat, 99))},
                "path": "nk_server_submit / nk_server_wait (host inputs, upload, geometry, solve, read-back)",
                "server": sinfo},
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    if not args.no_cpu_baseline:
        dt, st, uo, vo, used = cpu_solve(workload("fp64", 0), os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": used, "kind": "port",
                                "sample": "one full FP64 solve of the same workload (oracle restatement, multigrid PCG)"}
        line["rel_error_vs_fp64_oracle"] = rel_l2(u_mixed, v_mixed, uo, vo)
        line["fp64_rel_error_vs_fp64_oracle"] = rel_l2(u64, v64, uo, vo)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()


if __name__ == "__main__":
    main()
