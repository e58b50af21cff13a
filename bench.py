#!/usr/bin/env python
"""Benchmark of the explicit FVM residual + stage update on one GB300.

Workload (the configuration the headline metric is quoted on): 3D ideal-gas
blast on a 256^3 grid with reflective (Symmetry) walls, FP64 state,
background rho = 1 (+-1% seeded noise), p = 0.1, sphere of radius 0.1 at the
centre with p = 10; limited linear reconstruction (Linear2psLim, Barth-
Jespersen), Roe flux, RK1 (the reference's only stage), CFL 0.4.  A "step" is
one RK step over the whole grid; one cell-update is one cell advanced by one
stage.  The state (687 MB FP64 per copy) is larger than L2, so no flush is
needed between steps.

Lines printed (rank 0, one JSON line):
  --impl ours       value  = cell-updates/s with the state resident in HBM,
                             device-timed with CUDA events on the library stream
                    e2e    = same metric through the C ABI with host buffers
                             (pinned H2D of the initial state, K steps, D2H of
                             the final state) timed on the host
                    roofline, cpu_baseline (oracle port on this host's cores),
                    clocks, fp64 plain-path rate and mixed-vs-FP64 errors
                    workloads: the other configurations measured in the same
                    run (2D shear layer 1024^2, the 4096 batched tubes, a
                    10 s sample of the served stream), each with its own
                    e2e, roofline, CPU baseline and mixed-vs-FP64 error
  --impl reference  the reference algorithm's CPU implementation (the
                    oracle port, all host threads) on the same workload: each
                    step is one RK step over the whole 256^3 blast, whose
                    initial state the oracle builds itself (the product
                    library is not loaded).
With torchrun (N>1) every rank advances its own replica (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
N_DEFAULT = 256
BLAST = [1.0, 0.1, 10.0, 0.1, 0.01]  # rho, p_out, p_in, radius, noise
SEED = 2024
BYTES_PER_CELL_UPDATE = 80  # one FP64 read + one FP64 write of the 5 conserved values


def workload_case(capi, n, nz=None, periodic_z=False):
    sym = (capi.BC_SYMMETRY, 0.0, (0.0, 0.0, 0.0), 0.0)
    return capi.make_case(ndims=3, nx=n, ny=n, nz=nz or n, periodic=(0, 0, 1 if periodic_z else 0),
                          recon=capi.RECON_LINEAR2_LIM, limiter=capi.LIM_BJ, solver=capi.RS_ROE, cfl=0.4,
                          eps=0.0, max_iter=200, max_time=1e30, bc=[sym] * 6)


def workload_config(n):
    """The workload, identical on both arms (the arithmetic of each arm is in
    its `dtype` and `precision` keys)."""
    return {"workload": f"3D ideal-gas blast {n}^3, Symmetry walls, Linear2psLim(BJ)+Roe, RK1, CFL 0.4",
            "grid": [n, n, n], "cells": n ** 3, "seed": SEED,
            "state": f"FP64, {n}^3 cells ({n ** 3 * 40 / 1e6:.0f} MB per copy)",
            "l2": "inputs larger than L2 (129 MB); no flush needed", "parallelism": "replicas"}


def dist_init():
    """(rank, world size, local rank, torch.distributed or None) from the
    torchrun environment: one independent replica per GPU over NCCL (gloo on
    hosts without CUDA, where only the host-side logic runs)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(lr)
        dist.init_process_group("nccl")
    else:
        dist.init_process_group("gloo")
    return dist.get_rank(), ws, lr, dist


def _reduce(x, dist, op):
    if dist is None:
        return float(x)
    import torch
    dev = f"cuda:{torch.cuda.current_device()}" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def rank_max(x, dist):
    """The largest x over the ranks (the slowest replica's time)."""
    return _reduce(x, dist, dist.ReduceOp.MAX if dist is not None else None)


def rank_sum(x, dist):
    """The sum of x over the ranks (the units every replica processed)."""
    return _reduce(x, dist, dist.ReduceOp.SUM if dist is not None else None)


def replica_rate(units, seconds, dist):
    """Whole-job rate of independent replicas: the units all ranks processed
    divided by the slowest rank's time (the timed regions are bracketed by
    barriers)."""
    return rank_sum(units, dist) / rank_max(seconds, dist)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = uuid
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(", ") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        rows = [r for r in rows if len(r) >= 9 and (self.uuid is None or r[0].strip() in self.uuid)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].strip().replace(".", "").isdigit() else None,
                "samples": len(rows), "reasons": reasons}


def gpu_uuid(dev):
    try:
        import torch
        u = torch.cuda.get_device_properties(dev).uuid
        return "GPU-" + str(u)
    except Exception:
        return None


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(workload, kernel, cells):
    """DRAM bytes per launch of `kernel` over `cells` cells in `workload`: the
    committed ncu capture's bytes per cell (dram__bytes_read.sum +
    dram__bytes_write.sum over the captured launch's cells) times the cell
    count, or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            rec = json.load(f).get(workload)
        return float(rec["bytes_per_cell"]) * cells if rec and rec["kernel"] == kernel else None
    except Exception:
        return None


def oracle_sample_rate(steps, warmup, threads, n=N_DEFAULT):
    """The reference algorithm on the CPU (oracle port, OpenMP over `threads`
    host threads): cell-updates/s of RK steps over the whole n^3 blast with
    Symmetry walls, the same workload as the GPU arm; the oracle builds the
    initial state itself (its restatement of the scenario, bit-identical to
    the library's)."""
    from oracle import oracle as O
    from turbostructred_gb300 import capi  # the plain-Python case description only
    case = workload_case(capi, n)
    ic = O.fill_scenario(case, O.SCENARIO_BLAST, SEED, BLAST, threads=threads)
    full = O.embed(case, ic)
    del ic
    if warmup:
        full, _ = O.advance(case, full, warmup, threads=threads)
    t0 = time.perf_counter()
    full, info = O.advance(case, full, steps, threads=threads)
    dt = time.perf_counter() - t0
    return n ** 3 * steps / dt, dt, f"{steps} RK step(s) over the whole {n}^3 blast (Symmetry walls) after {warmup} warm-up step(s)"


def _cpu_job(job):
    """One problem advanced by the oracle port on one host core: (case, interior
    state, steps or -1 for the Run loop) -> (cell-updates, seconds)."""
    import numpy as np

    from oracle import oracle as O
    case, ic, steps = job
    full = O.embed(case, np.asarray(ic))
    t0 = time.perf_counter()
    _, info = O.advance(case, full, steps, threads=1)
    cells = case["nx"] * (case["ny"] if case["ndims"] > 1 else 1) * (case["nz"] if case["ndims"] > 2 else 1)
    return cells * info["iteration"], time.perf_counter() - t0


def cpu_pool_rate(jobs, procs):
    """Aggregate cell-updates/s of independent CPU jobs over `procs` processes
    (spawned: no process forks after the GPU is initialised)."""
    import multiprocessing as mp
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(_cpu_job, jobs, chunksize=1)
    wall = time.perf_counter() - t0
    return sum(r[0] for r in res) / wall, wall


def tubes_cpu_sample(every=8, cap=4000, seed=4096):
    from oracle import oracle as O
    from turbostructred_gb300 import workloads
    probs = workloads.tubes(4096, seed=seed, fill=O.fill_scenario)
    jobs = []
    for k in range(0, len(probs), every):
        c, ic = probs[k]
        c = dict(c, max_iter=cap)
        jobs.append((c, ic, -1))
    desc = (f"every {every}th of the 4096 tubes ({len(jobs)} tubes), each run to t_end or {cap} stages, "
            "one process per host core, oracle port (the reference's algorithm restated)")
    return jobs, desc


def served_cpu_sample(n_req=48, steps=16, seed=200):
    from oracle import oracle as O
    from turbostructred_gb300 import workloads
    reqs = workloads.stream(200.0, 60.0, seed=seed)[:n_req]
    jobs = [(c, workloads.stream_state(c, p, s, fill=O.fill_scenario), steps) for _, c, p, s in reqs]
    desc = (f"the first {n_req} requests of the stream, {steps} RK steps each (of 500), one process per host "
            "core, oracle port")
    return jobs, desc


def run_reference(args, rank, ws):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    if args.workload in ("tubes", "served"):
        jobs, sample = tubes_cpu_sample() if args.workload == "tubes" else served_cpu_sample()
        rate, secs = cpu_pool_rate(jobs, threads)
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "cell-updates/s", "n_gpus": ws,
                "steps": 1, "warmup": 0, "ms_per_step": 1e3 * secs, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": args.workload, "sample": sample},
                "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.workload in ("shear2d", "batch2d", "rows"):
        # the reference algorithm (oracle port, OpenMP over all host threads)
        # on the same 2D grids: the 1024^2 shear layer, one 512^2 quadrant
        # problem of the batch, or the 512^2 viscous channel of the rows
        # line, for a bounded number of steps
        from oracle import oracle as O
        from turbostructred_gb300 import capi, workloads
        if args.workload == "shear2d":
            case = capi.make_case(ndims=2, nx=1024, ny=1024, periodic=(1, 1, 1), recon=capi.RECON_LINEAR2_LIM,
                                  solver=capi.RS_HLLC, cfl=0.4, max_iter=10**6, max_time=1e30)
            ic = O.fill_scenario(case, O.SCENARIO_SHEAR_LAYER, 7, [2.0, 1.0, 0.5, 2.5, 0.01])
            steps, sample = 60, "60 RK steps of the 1024^2 shear layer"
        elif args.workload == "rows":
            nat = (capi.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
            wall = (capi.BC_WALL, 0.0, (0.0, 0.0, 0.0), 0.0)
            movw = (capi.BC_MOVING_WALL, 0.0, (0.3, 0.0, 0.0), 0.0)
            case = capi.make_case(ndims=2, nx=512, ny=512, periodic=(1, 0, 1), recon=capi.RECON_LINEAR2_LIM,
                                  solver=capi.RS_ROE, cfl=0.4, viscous=True, viscosity=1e-3, max_iter=10**6,
                                  max_time=1e30, bc=[nat, nat, wall, movw, nat, nat])
            ic = O.fill_scenario(case, O.SCENARIO_SHEAR_LAYER, 5, [2.0, 1.0, 0.5, 2.5, 0.05])
            steps, sample = 200, "200 RK steps of the 512^2 viscous channel"
        else:
            case = workloads.quadrant_case(512, capi.RS_ROE, 10**6)
            ic = workloads.stream_state(case, [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03,
                                               0.53, 0.0, 1.2, 0.3], 1, fill=O.fill_scenario)
            steps, sample = 120, "120 RK steps of one 512^2 quadrant problem of the batch"
        full = O.embed(case, ic)
        full, _ = O.advance(case, full, 2, threads=threads)
        t0 = time.perf_counter()
        O.advance(case, full, steps, threads=threads)
        secs = time.perf_counter() - t0
        cells = case["nx"] * case["ny"]
        rate = cells * steps / secs
        line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "cell-updates/s", "n_gpus": ws,
                "steps": steps, "warmup": 2, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": args.workload, "sample": sample},
                "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    rate, secs, sample = oracle_sample_rate(args.steps, args.warmup, threads, n=args.n)
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "precision": "fp64",
            "data": "synthetic (seeded blast initial state built by the oracle, no dataset)",
            "config": workload_config(args.n),
            "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def rel_errors(a, b):
    import numpy as np
    out = {}
    for name, v in (("rho", 0), ("mom", slice(1, 4)), ("E", 4)):
        x, y = a[..., v], b[..., v]
        out[f"L1_{name}"] = float(np.abs(x - y).sum() / max(np.abs(y).sum(), 1e-300))
        out[f"Linf_{name}"] = float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))
    return out


def run_ours(args, rank, ws, lr, dist):
    import numpy as np
    import torch

    from turbostructred_gb300 import build, capi
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    n = args.n
    case = workload_case(capi, n)
    ic = capi.fill_scenario(case, capi.SCENARIO_BLAST, SEED + rank, BLAST)
    cells = n ** 3

    # the fused mixed-precision step is the measured path; "fp64" times the
    # bit-exact FP64 path instead (an error, not a fallback, if a path fails)
    precision = "mixed" if args.precision == "auto" else args.precision
    prec_id = capi.PRECISION_MIXED if precision == "mixed" else capi.PRECISION_FP64

    solver = capi.Solver(case, prec_id, device=lr)
    solver.set_state(ic)
    if args.warmup:
        solver.step(args.warmup)
    solver.synchronize()
    uuid = gpu_uuid(lr)
    sampler = ClockSampler(uuid)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    info, timing = solver.step_timed(args.steps)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    t_ms = rank_max(timing["total_ms"], dist)
    value = replica_rate(cells * args.steps, t_ms / 1e3, dist)

    # roofline of the dominant kernel
    kernels = timing["kernels"]
    top = max(kernels, key=kernels.get)
    top_ms = kernels[top]
    peak, peak_kind = measured_peak()
    if precision == "mixed":
        alg = BYTES_PER_CELL_UPDATE * cells
        alg_note = "80 B x cells per launch (one fused launch advances every cell one stage)"
    else:
        alg = BYTES_PER_CELL_UPDATE * cells
        alg_note = "80 B x cells per step, charged to the dominant kernel of the FP64 path"
    achieved = alg / (top_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profile_traffic("blast3d", top, cells) if precision == "mixed" else None, "kernel": top,
                "kernel_ms": top_ms,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "algorithmic_bytes": alg, "algorithmic_note": alg_note,
                "step_kernels_ms": kernels}

    extra = {}
    # FP64 plain path at the same size (short run) and mixed-vs-FP64 error
    if precision == "mixed" and not args.skip_fp64:
        fp = capi.Solver(case, capi.PRECISION_FP64, device=lr)
        fp.set_state(ic)
        fp.step(2)
        _, tfp = fp.step_timed(args.fp64_steps)
        fp64_rate = cells * args.fp64_steps / (tfp["total_ms"] / 1e3)
        extra["fp64_value"] = fp64_rate
        extra["mixed_over_fp64"] = value / ws / fp64_rate
        # accuracy: same IC, same steps
        fp.set_state(ic)
        fp.set_info(iteration=0, time=0.0, dt=0.0)
        fp.step(args.err_steps)
        ref = fp.get_state()
        mx = capi.Solver(case, capi.PRECISION_MIXED, device=lr)
        mx.set_state(ic)
        mx.step(args.err_steps)
        got = mx.get_state()
        extra["mixed_error_vs_fp64"] = dict(steps=args.err_steps, **rel_errors(got, ref))
        fp.close()
        mx.close()

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.skip_e2e:
        host_in = torch.from_numpy(ic.reshape(-1)).pin_memory()
        host_out = torch.empty(ic.size, dtype=torch.float64).pin_memory()
        lib = capi.load()
        import ctypes as C
        P = C.POINTER(C.c_double)
        e2e_steps = args.steps
        times = []
        for job in range(args.e2e_jobs + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            capi.check(lib.ts_set_state(solver.h, C.cast(host_in.data_ptr(), P), capi.LAYOUT_INTERIOR))
            solver.set_info(iteration=0, time=0.0, dt=0.0)
            solver.step(e2e_steps)
            capi.check(lib.ts_get_state(solver.h, C.cast(host_out.data_ptr(), P), capi.LAYOUT_INTERIOR))
            t1 = time.perf_counter()
            if job > 0:
                times.append(t1 - t0)
        tj = statistics.median(times)
        state_bytes = ic.size * 8
        e2e = {"value": replica_rate(cells * e2e_steps, tj, dist), "unit": "cell-updates/s",
               "h2d_bytes_per_step": state_bytes / e2e_steps, "d2h_bytes_per_step": state_bytes / e2e_steps,
               "job": f"H2D of the {n}^3 initial state from pinned host memory, {e2e_steps} steps, D2H of the final state",
               "h2d_bytes_per_job": state_bytes, "d2h_bytes_per_job": state_bytes, "seconds_per_job": tj}
    solver.close()

    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        threads = os.cpu_count() or 1
        rate, secs, sample = oracle_sample_rate(args.cpu_steps, 1, threads, n=n)
        cpu = {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port", "sample": sample,
               "seconds": secs}

    # the other configurations, measured in the same run (one GPU only: under
    # torchrun each replica would repeat them)
    workloads = None
    if ws == 1 and not args.skip_workloads:
        workloads = other_workloads(args, rank, lr)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 flux" if precision == "mixed" else "f64",
                "precision": precision,
                "data": "synthetic (seeded blast initial state, no dataset)",
                "config": workload_config(n), "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": timing["launches"] * ws,
                "step_info": {"iteration": info["iteration"], "time": info["time"], "dt": info["dt"],
                              "health": info["health"]}}
        line.update(extra)
        if workloads is not None:
            line["workloads"] = workloads
        print(json.dumps(line), flush=True)


def other_workloads(args, rank, lr):
    """The 2D shear layer (C2), the batched tubes (C4) and a sample of the
    served stream (C5), each through its own bench function with its
    defaults, summarised for the default bench line."""
    import copy

    def sub(**kw):
        a = copy.copy(args)
        a.steps, a.warmup = None, None
        for k, v in kw.items():
            setattr(a, k, v)
        return a

    keep = ("workload", "value", "unit", "steps", "warmup", "ms_per_step", "e2e", "roofline", "cpu_baseline",
            "mixed_error_vs_fp64", "fp64_value", "mixed_over_fp64", "clocks", "gpu_launches", "config", "batch",
            "latency_ms", "admission_wait_ms", "offered_cell_updates_per_s", "step_info")
    out = {}
    for key, fn, a in (("shear2d_1024", run_shear, sub(steps=args.shear_steps, warmup=5)),
                       ("tubes_4096", run_tubes, sub(steps=3, warmup=3)),
                       ("served_stream", run_served, sub(seconds=args.served_sample_seconds, warmup=0))):
        line = fn(a, rank, 1, lr, None, emit=False)
        if line is not None:
            out[key] = {k: line[k] for k in keep if k in line}
    if "served_stream" in out:
        out["served_stream"]["sample"] = (f"the first {args.served_sample_seconds:g} s of the {args.rate:g} req/s "
                                          "stream (python bench.py --workload served runs the full 60 s)")
    return out


def tubes_cell_updates(infos, probs):
    return float(sum(c["nx"] * inf["iteration"] for (c, _), inf in zip(probs, infos)))


def run_tubes(args, rank, ws, lr, dist, emit=True):
    """Batched 1D tubes: one step = the whole batch solved to t_end."""
    import torch

    steps = args.steps or 3
    warmup = 3 if args.warmup is None else args.warmup

    from turbostructred_gb300 import build, capi, workloads
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    probs = workloads.tubes(args.tubes, seed=4096 + rank)
    budget = int(1.5 * sum(capi.batch_problem_bytes(c) for c, _ in probs)) + (64 << 20)
    cells = sum(c["nx"] for c, _ in probs)

    def solve(subset, tune):
        b = capi.Batch(budget, device=lr)
        t0 = time.perf_counter()
        ids = [b.add(c, v) for c, v in subset]
        t1 = time.perf_counter()
        choice = b.autotune(args.tune_stages) if tune else None
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        left = b.run()
        t3 = time.perf_counter()
        outs = [b.get(i) for i in ids]
        t4 = time.perf_counter()
        st = b.stats()
        b.close()
        assert left == 0
        return dict(add_s=t1 - t0, run_s=t3 - t2, get_s=t4 - t3, stats=st, choice=choice,
                    infos=[o[1] for o in outs], states=outs)

    for _ in range(warmup):
        solve(probs[:128], False)
    uuid = gpu_uuid(lr)
    sampler = ClockSampler(uuid)
    if dist is not None:
        dist.barrier()
    runs = [solve(probs, args.tune_stages > 0) for _ in range(steps)]
    clocks = sampler.stop()
    run_s = max(r["run_s"] for r in runs) if steps == 1 else statistics.median(r["run_s"] for r in runs)
    cu = tubes_cell_updates(runs[0]["infos"], probs)
    value = replica_rate(cu, run_s, dist)
    e2e_s = statistics.median(r["add_s"] + r["run_s"] + r["get_s"] for r in runs)
    e2e_value = replica_rate(cu, e2e_s, dist)
    health = sum(1 for inf in runs[0]["infos"] if inf["health"])
    iters = [inf["iteration"] for inf in runs[0]["infos"]]
    st = runs[0]["stats"]
    # accuracy: a sample of tubes against the FP64 plain path
    errs = []
    for k in range(0, len(probs), max(1, len(probs) // args.err_tubes)):
        c, ic = probs[k]
        with capi.Solver(c, capi.PRECISION_FP64, device=lr) as s:
            s.set_state(ic)
            inf = s.run()
            ref = s.get_state()
        got = runs[0]["states"][k][0]
        if inf["iteration"] == iters[k]:
            errs.append(rel_errors(got, ref))
    err = {k: max(e[k] for e in errs) for k in errs[0]} if errs else None
    bytes_in = sum(v.size * 8 for _, v in probs)
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL_UPDATE * cu / run_s / 1e9
    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": steps,
                "warmup": warmup, "ms_per_step": 1e3 * run_s, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64 state / f32 flux", "data": "synthetic (seeded tubes, no dataset)",
                "config": {"workload": f"{len(probs)} batched 1D shock tubes to t_end 0.1 (sizes 64-4096 "
                                       "log-uniform, half stiffened gas, PWC/Linear2psLim mixed, Roe, CFL 0.5)",
                           "tubes": len(probs), "cells": cells, "step": "the whole batch solved to t_end",
                           "warmup_step": "the first 128 tubes solved to t_end",
                           "l2": "state resident in HBM; each stage touches every active tube once",
                           "tile": runs[0]["choice"]},
                "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": bytes_in,
                        "d2h_bytes_per_step": bytes_in, "seconds_per_job": e2e_s},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": profile_traffic("tubes", "k_mix_step", cu),
                             "kernel": "k_mix_step (batched, one-row 1D tiles) and k_mix_tail",
                             "kernel_ms": None, "algorithmic_bytes": BYTES_PER_CELL_UPDATE * cu,
                             "basis": "80 B x the batch's cell-updates over the whole solve's wall time (stage "
                                      "kernels, finish kernels, the cluster tail kernel and launch gaps): a lower "
                                      "bound of the kernels' own rate",
                             "peak_source": peak_kind},
                "clocks": clocks, "gpu_launches": st["launches"],
                "batch": {"stages": st["stages"], "launches": st["launches"], "cell_updates": cu,
                          "max_iterations": max(iters), "unhealthy": health, "add_s": runs[0]["add_s"],
                          "get_s": runs[0]["get_s"]},
                "mixed_error_vs_fp64": {"tubes_sampled": len(errs), **(err or {})}}
        if ws == 1 and not args.skip_cpu:
            jobs, sample = tubes_cpu_sample()
            procs = os.cpu_count() or 1
            rate, secs = cpu_pool_rate(jobs, procs)
            line["cpu_baseline"] = {"value": rate, "unit": "cell-updates/s", "cores": procs, "kind": "port",
                                    "sample": sample, "seconds": secs}
        if emit:
            print(json.dumps(line), flush=True)
    return line


def run_served(args, rank, ws, lr, dist, emit=True):
    """Served stream: Poisson arrivals of 2D quadrant problems."""
    import threading

    from turbostructred_gb300 import build, capi, workloads
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    reqs = workloads.stream(args.rate, args.seconds, seed=200 + rank, steps=args.served_steps)
    order = capi.SERVE_SHORTEST_FIRST if args.order == "shortest" else capi.SERVE_FIFO
    srv = capi.Server(int(args.budget_gb * 2**30), chunk_ms=args.chunk_ms, device=lr, order=order,
                      max_cells=int(args.max_cells))
    # warm-up: a few solves of each size through the same server
    for side in workloads.SIDES:
        c = workloads.quadrant_case(side, capi.RS_ROE, 20)
        srv.wait(srv.submit(c, workloads.stream_state(c, [1.0, 0.0, 0.0, 1.0] * 4, 1), keep_state=False))
    st0 = srv.stats()
    ids = []
    lat = []
    done = threading.Event()

    # served results kept for the error against the FP64 path: every 40th
    # request of side <= 256
    sample = {k for k, (_, c, _, _) in enumerate(reqs) if k % 40 == 0 and c["nx"] <= 256}
    kept = {}

    def collector():
        k = 0
        while not (done.is_set() and k >= len(ids)):
            if k >= len(ids):
                time.sleep(0.001)
                continue
            state, info, t = srv.wait(ids[k])
            lat.append((t["submit_s"], t["admit_s"], t["finish_s"], info["iteration"]))
            if k in sample:
                kept[k] = (state, info)
            k += 1

    th = threading.Thread(target=collector)
    th.start()
    sampler = ClockSampler(gpu_uuid(lr))
    t0 = time.perf_counter()
    late = 0.0
    for at, case, params, seed in reqs:
        ic = workloads.stream_state(case, params, seed)
        now = time.perf_counter() - t0
        if now < at:
            time.sleep(at - now)
        else:
            late = max(late, now - at)
        ids.append(srv.submit(case, ic, keep_state=True))
    done.set()
    th.join()
    t_end = time.perf_counter() - t0
    clocks = sampler.stop()
    st = srv.stats()
    srv.close()
    lat_ms = [1e3 * (f - s) for s, a, f, it in lat]
    wait_ms = [1e3 * (a - s) for s, a, f, it in lat]
    if dist is not None:
        # every replica's requests count in the percentiles
        parts = [None] * ws
        dist.all_gather_object(parts, (lat_ms, wait_ms))
        lat_ms = [x for p in parts for x in p[0]]
        wait_ms = [x for p in parts for x in p[1]]
    lat_ms.sort()
    wait_ms.sort()

    def pct(v, p):
        import math
        return v[min(len(v), max(1, math.ceil(p / 100 * len(v)))) - 1] if v else None

    cu = st["cell_updates"] - st0["cell_updates"]
    first = min(s for s, a, f, it in lat)
    last = max(f for s, a, f, it in lat)
    value = replica_rate(cu, last - first, dist)
    bytes_io = sum(c["nx"] * c["ny"] * 40 for _, c, _, _ in reqs)
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL_UPDATE * cu / (last - first) / 1e9
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": len(reqs),
                "warmup": len(workloads.SIDES), "ms_per_step": 1e3 * (last - first) / max(1, len(reqs)),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 flux",
                "data": "synthetic (seeded Poisson stream of quadrant problems, no dataset)",
                "config": {"workload": f"served stream: Poisson {args.rate:g} req/s for {args.seconds:g} s of 2D "
                                       f"quadrant Riemann problems, sides {list(workloads.SIDES)}, Roe/HLLC at "
                                       f"random, {args.served_steps} RK steps each, HBM budget {args.budget_gb:g} GB",
                           "requests": len(reqs), "step": "one served request", "chunk_ms": args.chunk_ms,
                           "admission": {"order": args.order, "max_cells_in_flight": int(args.max_cells)}},
                "latency_ms": {"p50": pct(lat_ms, 50), "p99": pct(lat_ms, 99), "max": lat_ms[-1] if lat_ms else None},
                "admission_wait_ms": {"p50": pct(wait_ms, 50), "p99": pct(wait_ms, 99)},
                "mixed_error_vs_fp64": served_errors(reqs, kept, lr),
                "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": bytes_io / max(1, len(reqs)),
                        "d2h_bytes_per_step": bytes_io / max(1, len(reqs)),
                        "note": "latency and throughput are end to end: host submit (copy of the initial state) "
                                "to the final state back in host memory"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": profile_traffic("batch2d", "k_mix_step", cu),
                             "kernel": "k_mix_step (batched, one-row 2D tiles)", "kernel_ms": None,
                             "algorithmic_bytes": BYTES_PER_CELL_UPDATE * cu,
                             "basis": "80 B x the served cell-updates over the wall time from the first "
                                      "submission to the last result (includes uploads, read-backs and idle "
                                      "gaps): a lower bound of the kernel's own rate",
                             "peak_source": peak_kind},
                "server": {k: st[k] for k in ("submitted", "completed", "rejected", "stages", "launches", "busy_s",
                                              "admit_s", "retire_s")},
                "offered_cell_updates_per_s": sum(c["nx"] * c["ny"] * args.served_steps for _, c, _, _ in reqs)
                / args.seconds, "client_max_lateness_s": late, "wall_s": t_end,
                "clocks": clocks, "gpu_launches": st["launches"] - st0["launches"]}
        if ws == 1 and not args.skip_cpu:
            jobs, sample = served_cpu_sample()
            procs = os.cpu_count() or 1
            rate, secs = cpu_pool_rate(jobs, procs)
            line["cpu_baseline"] = {"value": rate, "unit": "cell-updates/s", "cores": procs, "kind": "port",
                                    "sample": sample, "seconds": secs}
        if emit:
            print(json.dumps(line), flush=True)
        return line


def served_errors(reqs, kept, lr):
    """Largest L1/Linf errors of sampled served results against the same
    requests run alone on the FP64 path."""
    from turbostructred_gb300 import capi, workloads
    errs = []
    for k, (state, info) in sorted(kept.items()):
        _, case, params, seed = reqs[k]
        with capi.Solver(case, capi.PRECISION_FP64, device=lr) as s:
            s.set_state(workloads.stream_state(case, params, seed))
            ref_info = s.run()
            ref = s.get_state()
        if ref_info["iteration"] == info["iteration"]:
            errs.append(rel_errors(state.reshape(ref.shape), ref))
    if not errs:
        return None
    return {"requests_sampled": len(errs), **{key: max(e[key] for e in errs) for key in errs[0]}}


SHEAR = [2.0, 1.0, 0.5, 2.5, 0.01]  # rho_in, rho_out, u, p, noise


def shear_case(capi, n, steps):
    return capi.make_case(ndims=2, nx=n, ny=n, periodic=(1, 1, 1), recon=capi.RECON_LINEAR2_LIM, limiter=capi.LIM_BJ,
                          solver=capi.RS_HLLC, cfl=0.4, max_iter=steps, max_time=1e30)


def shear_cpu_rate(threads, steps=60, n=1024):
    """The oracle port (all host threads) on the same shear layer, inputs built
    by the oracle: (rate, seconds, sample)."""
    from oracle import oracle as O
    from turbostructred_gb300 import capi  # plain-Python case description only
    case = shear_case(capi, n, 10**6)
    full = O.embed(case, O.fill_scenario(case, O.SCENARIO_SHEAR_LAYER, 7, SHEAR, threads=threads))
    full, _ = O.advance(case, full, 2, threads=threads)
    t0 = time.perf_counter()
    O.advance(case, full, steps, threads=threads)
    secs = time.perf_counter() - t0
    return n * n * steps / secs, secs, f"{steps} RK steps of the {n}^2 shear layer after 2 warm-up steps"


def e2e_jobs(capi, solver, ic, steps, jobs=2):
    """Median host time of jobs through the C ABI with host buffers: H2D of
    the initial state from pinned memory, `steps` steps, D2H of the final
    state (the first job is a warm-up)."""
    import ctypes as C

    import torch
    host_in = torch.from_numpy(ic.reshape(-1)).pin_memory()
    host_out = torch.empty(ic.size, dtype=torch.float64).pin_memory()
    lib = capi.load()
    P = C.POINTER(C.c_double)
    times = []
    for job in range(jobs + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(lib.ts_set_state(solver.h, C.cast(host_in.data_ptr(), P), capi.LAYOUT_INTERIOR))
        solver.set_info(iteration=0, time=0.0, dt=0.0)
        solver.step(steps)
        capi.check(lib.ts_get_state(solver.h, C.cast(host_out.data_ptr(), P), capi.LAYOUT_INTERIOR))
        t1 = time.perf_counter()
        if job > 0:
            times.append(t1 - t0)
    return statistics.median(times), ic.size * 8


def run_shear(args, rank, ws, lr, dist, emit=True):
    """2D shear layer 1024^2, periodic, Linear2psLim(BJ) + HLLC, 1000 steps:
    the mixed path timed, the plain FP64 path beside it, and the mixed-vs-FP64
    error after the same 1000 steps."""
    from turbostructred_gb300 import build, capi
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    n = 1024
    steps = args.steps or args.shear_steps
    warmup = 5 if args.warmup is None else args.warmup
    case = shear_case(capi, n, steps)
    ic = capi.fill_scenario(case, capi.SCENARIO_SHEAR_LAYER, 7 + rank, SHEAR)
    cells = n * n
    out = {}
    for prec, name in ((capi.PRECISION_MIXED, "mixed"), (capi.PRECISION_FP64, "fp64")):
        with capi.Solver(case, prec, device=lr) as s:
            s.set_state(ic)
            s.step(warmup)
            s.set_state(ic)
            s.set_info(iteration=0, time=0.0, dt=0.0)
            sampler = ClockSampler(gpu_uuid(lr)) if name == "mixed" else None
            info, tm = s.step_timed(steps)
            clocks = sampler.stop() if sampler else None
            out[name] = dict(state=s.get_state(), info=info, ms=tm["total_ms"], kernels=tm["kernels"], clocks=clocks,
                             launches=tm["launches"])
            if name == "mixed" and not args.skip_e2e:
                out["e2e"] = e2e_jobs(capi, s, ic, steps)
    t_ms = rank_max(out["mixed"]["ms"], dist)
    value = replica_rate(cells * steps, t_ms / 1e3, dist)
    kernels = out["mixed"]["kernels"]
    top = max(kernels, key=kernels.get)
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL_UPDATE * cells / (kernels[top] / 1e3) / 1e9
    err = rel_errors(out["mixed"]["state"], out["fp64"]["state"])
    e2e = None
    if "e2e" in out:
        tj, nbytes = out["e2e"]
        e2e = {"value": replica_rate(cells * steps, tj, dist), "unit": "cell-updates/s",
               "h2d_bytes_per_step": nbytes / steps, "d2h_bytes_per_step": nbytes / steps,
               "job": f"H2D of the {n}^2 initial state from pinned host memory, {steps} steps, D2H of the final state",
               "seconds_per_job": tj}
    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        threads = os.cpu_count() or 1
        rate, secs, sample = shear_cpu_rate(threads)
        cpu = {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port", "sample": sample,
               "seconds": secs}
    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": steps,
                "warmup": warmup, "ms_per_step": t_ms / steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 flux", "precision": "mixed",
                "data": "synthetic (seeded shear layer, no dataset)",
                "config": {"workload": "2D ideal-gas shear layer 1024^2, periodic, Linear2psLim(BJ)+HLLC, "
                                       f"{steps} RK steps, CFL 0.4", "cells": cells,
                           "l2": "state 84 MB per FP64 copy: below L2 (129 MB); the mixed step also moves "
                                 "the FP32 residual, 2 x 42 MB, so its working set spills"},
                "e2e": e2e,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": profile_traffic("shear2d", top, cells), "kernel": top,
                             "kernel_ms": kernels[top], "algorithmic_bytes": BYTES_PER_CELL_UPDATE * cells,
                             "peak_source": peak_kind},
                "cpu_baseline": cpu,
                "fp64_value": cells * steps / (out["fp64"]["ms"] / 1e3),
                "mixed_over_fp64": out["fp64"]["ms"] / t_ms,
                "mixed_error_vs_fp64": dict(steps=steps, **err),
                "clocks": out["mixed"]["clocks"], "gpu_launches": out["mixed"]["launches"],
                "step_info": {k: out["mixed"]["info"][k] for k in ("iteration", "time", "dt", "health")}}
        if emit:
            print(json.dumps(line), flush=True)
    return line


def run_batch2d(args, rank, ws, lr, dist):
    """Steady-state capacity of the served kernel: a batch of 2D quadrant
    problems (8 each of 1024^2, 512^2, 256^2; Roe and HLLC alternating)
    advanced together; a step is one stage of the whole batch."""
    import torch

    from turbostructred_gb300 import build, capi, workloads
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    quad = [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]
    b = capi.Batch(8 << 30, device=lr)
    cells = 0
    for k in range(24):
        side = (1024, 512, 256)[k % 3]
        c = workloads.quadrant_case(side, capi.RS_ROE if k % 2 else capi.RS_HLLC, 10**6)
        b.add(c, workloads.stream_state(c, quad, k))
        cells += side * side
    choice = b.autotune(args.tune_stages) if args.tune_stages > 0 else None
    b.step(args.warmup)
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_uuid(lr))
    s0 = b.stats()
    t0 = time.perf_counter()
    b.step(args.steps)
    t1 = time.perf_counter()
    s1 = b.stats()
    clocks = sampler.stop()
    b.close()
    cu = s1["cell_updates"] - s0["cell_updates"]
    value = replica_rate(cu, t1 - t0, dist)
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL_UPDATE * cu / (t1 - t0) / 1e9
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * (t1 - t0) / args.steps,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64 state / f32 flux", "data": "synthetic",
                          "config": {"workload": "batch of 24 2D quadrant problems (8 x 1024^2, 8 x 512^2, "
                                                 "8 x 256^2), Linear2psLim(BJ), Roe/HLLC", "cells": cells,
                                     "tile": choice},
                          "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                       "frac": achieved / peak,
                                       "traffic": profile_traffic("batch2d", "k_mix_step", cells),
                                       "kernel": "k_mix_step (batched, one-row 2D tiles)",
                                       "algorithmic_bytes": BYTES_PER_CELL_UPDATE * cells,
                                       "basis": "80 B x the batch's cell-updates over the timed stages' wall "
                                                "time (one launch per (solver, tile) group per stage); traffic: "
                                                "the captured bytes per cell times the batch's cells, per stage",
                                       "peak_source": peak_kind},
                          "clocks": clocks, "gpu_launches": s1["launches"] - s0["launches"]}), flush=True)


def run_rows(args, rank, ws, lr, dist):
    """The paths beyond the explicit step proper, each timed on the GPU with the
    oracle port (the reference's algorithm, all host threads) beside it:
    exact Godunov flux (FP64 path), source terms (mixed path), viscous flow
    (FP64 path), and the solution-file and Tecplot writers."""
    import numpy as np

    from oracle import oracle as O
    from turbostructred_gb300 import build, capi, workloads
    if rank == 0 or dist is None:
        build.build()
    if dist is not None:
        dist.barrier()
    capi.load()
    threads = os.cpu_count() or 1
    nat = (capi.BC_NATURAL, 0.0, (0.0, 0.0, 0.0), 0.0)
    wall = (capi.BC_WALL, 0.0, (0.0, 0.0, 0.0), 0.0)
    movw = (capi.BC_MOVING_WALL, 0.0, (0.3, 0.0, 0.0), 0.0)
    quad = [1.5, 0.0, 0.0, 1.5, 0.53, 1.2, 0.0, 0.3, 0.14, 1.2, 1.2, 0.03, 0.53, 0.0, 1.2, 0.3]
    heavy_top = [2.0, 0.0, 0.0, 2.5, 2.0, 0.0, 0.0, 2.5, 1.0, 0.0, 0.0, 2.5, 1.0, 0.0, 0.0, 2.5]
    n = 512
    rows = {
        "godunov": ("exact Godunov flux, 2D quadrant problem 512^2, Linear2psLim(BJ), FP64 path",
                    dict(ndims=2, nx=n, ny=n, periodic=(0, 0, 1), recon=capi.RECON_LINEAR2_LIM,
                         solver=capi.RS_GODUNOV, cfl=0.4, bc=[nat] * 6), capi.PRECISION_FP64,
                    capi.SCENARIO_QUADRANTS, quad, 20),
        "sources": ("uniform acceleration (Rayleigh-Taylor set-up) 512^2, Linear2psLim(BJ)+Roe, mixed path",
                    dict(ndims=2, nx=n, ny=n, periodic=(1, 0, 1), recon=capi.RECON_LINEAR2_LIM,
                         solver=capi.RS_ROE, cfl=0.4, uniform_acceleration=(0.0, -1.0, 0.0),
                         bc=[nat, nat, wall, wall, nat, nat]), capi.PRECISION_MIXED,
                    capi.SCENARIO_QUADRANTS, heavy_top, 200),
        "viscous": ("viscous channel 512^2 (periodic x, wall and moving wall), mu = 1e-3, Linear2psLim(BJ)+Roe, "
                    "FP64 path", dict(ndims=2, nx=n, ny=n, periodic=(1, 0, 1), recon=capi.RECON_LINEAR2_LIM,
                                      solver=capi.RS_ROE, cfl=0.4, viscous=True, viscosity=1e-3,
                                      bc=[nat, nat, wall, movw, nat, nat]), capi.PRECISION_FP64,
                    capi.SCENARIO_SHEAR_LAYER, [2.0, 1.0, 0.5, 2.5, 0.05], 20),
    }
    out = {}
    for key, (desc, kw, prec, scen, params, steps) in rows.items():
        case = capi.make_case(**dict(kw, max_iter=10**6, max_time=1e30))
        ic = capi.fill_scenario(case, scen, 5, params)
        with capi.Solver(case, prec, device=lr) as s:
            s.set_state(ic)
            s.step(3)
            _, tm = s.step_timed(steps)
        gpu_s = rank_max(tm["total_ms"] / 1e3, dist)
        value = rank_sum(n * n * steps, dist) / gpu_s
        cpu = None
        if rank == 0 and not args.skip_cpu:
            full = O.embed(case, ic)
            t0 = time.perf_counter()
            full, _ = O.advance(case, full, 2, threads=threads)
            # a sample of about 3 s of host work
            k = max(2, min(400, int(3.0 / max((time.perf_counter() - t0) / 2, 1e-6))))
            t0 = time.perf_counter()
            O.advance(case, full, k, threads=threads)
            secs = time.perf_counter() - t0
            cpu = {"value": n * n * k / secs, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                   "sample": f"{k} RK steps of the same {n}^2 case after 2 warm-up steps", "seconds": secs}
        out[key] = {"workload": desc, "value": value, "unit": "cell-updates/s", "steps": steps,
                    "ms_per_step": 1e3 * gpu_s / steps, "precision": "fp64" if prec == capi.PRECISION_FP64 else
                    "mixed", "gpu_launches": tm["launches"], "cpu_baseline": cpu}
    # solution files: Kernel::SaveSolution binary and the Tecplot text of a 128^3 state
    io = {}
    m = 128
    case = workload_case(capi, m)
    ic = capi.fill_scenario(case, capi.SCENARIO_BLAST, 3, BLAST)
    with tempfile.TemporaryDirectory() as d, capi.Solver(case, capi.PRECISION_MIXED, device=lr) as s:
        s.set_state(ic)
        s.step(2)
        s.synchronize()
        for name, fn in (("save_solution", lambda p: s.save_solution(p)),
                         ("save_tecplot", lambda p: (s.save_tecplot(p), s.wait_writes()))):
            path = os.path.join(d, name)
            t0 = time.perf_counter()
            fn(path)
            secs = time.perf_counter() - t0
            io[name] = {"bytes": os.path.getsize(path), "seconds": secs,
                        "MB_per_s": os.path.getsize(path) / secs / 1e6}
    out["solution_files"] = {"workload": f"3D blast state {m}^3 written by ts_save_solution and ts_save_tecplot",
                             **io}
    if rank == 0:
        line = {"metric": METRIC, "value": out["viscous"]["value"], "unit": "cell-updates/s", "n_gpus": ws,
                "steps": out["viscous"]["steps"], "warmup": 3, "ms_per_step": out["viscous"]["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded scenarios, no dataset)",
                "config": {"workload": "the rows beyond the explicit step: exact Godunov flux, source terms, "
                                       "viscous flow (value), solution files", "grid": [n, n]},
                "rows": out,
                "gpu_launches": sum(v["gpu_launches"] for k, v in out.items() if k != "solution_files")}
        print(json.dumps(line), flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default 500 for blast3d, 200 otherwise; tubes: 3, a step being the whole "
                        "batch solved to t_end)")
    p.add_argument("--warmup", type=int, default=None, help="untimed warm-up steps (default 5; tubes: 3)")
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["auto", "mixed", "fp64"], default="auto")
    p.add_argument("--n", type=int, default=N_DEFAULT)
    p.add_argument("--fp64-steps", type=int, default=5)
    p.add_argument("--err-steps", type=int, default=50)
    p.add_argument("--e2e-jobs", type=int, default=2)
    p.add_argument("--cpu-steps", type=int, default=10)
    p.add_argument("--skip-fp64", action="store_true")
    p.add_argument("--skip-e2e", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--workload", choices=["blast3d", "tubes", "served", "shear2d", "batch2d", "rows"],
                   default="blast3d")
    p.add_argument("--shear-steps", type=int, default=1000)
    p.add_argument("--skip-workloads", action="store_true",
                   help="default line: leave out the shear-layer, tubes and served-stream measurements")
    p.add_argument("--served-sample-seconds", type=float, default=10.0)
    p.add_argument("--tubes", type=int, default=4096)
    p.add_argument("--tune-stages", type=int, default=8)
    p.add_argument("--err-tubes", type=int, default=16)
    p.add_argument("--rate", type=float, default=200.0)
    p.add_argument("--seconds", type=float, default=60.0)
    p.add_argument("--served-steps", type=int, default=500)
    p.add_argument("--budget-gb", type=float, default=150.0)
    p.add_argument("--chunk-ms", type=float, default=2.0)
    p.add_argument("--order", choices=["fifo", "shortest"], default="shortest")
    p.add_argument("--max-cells", type=float, default=16e6)
    args = p.parse_args()
    if args.steps is None:
        # the 3D blast's timed region spans ~0.5 s (several clock samples);
        # the reference arm's CPU step of the whole 256^3 box takes ~0.7 s
        if args.impl == "reference":
            args.steps = 1 if args.workload == "tubes" else 20
        else:
            args.steps = 3 if args.workload == "tubes" else (500 if args.workload == "blast3d" else 200)
    if args.warmup is None:
        args.warmup = 3 if args.workload == "tubes" else 5
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        run_reference(args, rank, int(os.environ.get("WORLD_SIZE", "1")))
        return
    rank, ws, lr, dist = dist_init()
    {"blast3d": run_ours, "tubes": run_tubes, "served": run_served, "shear2d": run_shear,
     "batch2d": run_batch2d, "rows": run_rows}[args.workload](
        args, rank, ws, lr, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
