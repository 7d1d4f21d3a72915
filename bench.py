#!/usr/bin/env python
"""Benchmark of the GB300 source-term / diffusion hot path.

Default workload (the configuration the headline metric is quoted on): the
isolated batched source-term step -- 4096 seeded constant-pressure reactor
states of the seeded synthetic 150-species / 1000-reaction mechanism, each
integrated over its own dt (log-uniform 1e-6..1e-4 s) by the QSS integrator
with the reference's default options (interp kinetics), FP64, one launch per
step. Metric: source-term point-integrations per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload qss|bdf|diffusion|split|adjoint]

N > 1 runs under torch.distributed.run: every rank integrates its own batch
of points (no data exchange; the path has none), value = all points / max
time over ranks ("scaling": "weak").

--impl reference times the reference algorithm's CPU implementation on the
host cores: the reference itself (C++ on Cantera/SUNDIALS) cannot be built
here, so this is the CPU oracle port (oracle/), threaded over points like the
reference's TBB loop.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

N_POINTS = 4096
MECH_SEED = 150_1000
STATE_SEED = 4096
METRIC = "source-term point-integrations/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="qss", choices=["qss", "bdf", "diffusion", "split", "adjoint", "transport",
                                                             "convection", "sweep"])
    p.add_argument("--points", type=int, default=N_POINTS)
    p.add_argument("--kinetics", default="interp", choices=["interp", "standard"])
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--mech", default="150", choices=["150", "53"],
                   help="source workloads: the 150-species/1000-reaction mechanism or the GRI-3.0-sized "
                        "53-species/325-reaction one")
    p.add_argument("--no-plain", action="store_true",
                   help="split workload: skip the plain per-flame GPU path measured beside the batched step")
    p.add_argument("--split-dt", type=float, default=0.0,
                   help="split workload: global time step (0: 2e-5 s; the GRI-sized BDF case needs 5e-6 s on the "
                        "seeded profiles)")
    p.add_argument("--convection", action="store_true",
                   help="split workload: the reference's full D C D S D C D step with the convection stage")
    p.add_argument("--source", default="qss", choices=["qss", "bdf"],
                   help="split and adjoint workloads: source-term integrator (the C5 sweep names BDF)")
    p.add_argument("--no-secondary", action="store_true",
                   help="qss workload: skip the secondary figures (BDF, diffusion, split steps, adjoint)")
    p.add_argument("--regrid-interval", type=int, default=20,
                   help="sweep workload: steps between regrids (regridStepInterval)")
    p.add_argument("--bdf-layout", type=int, default=0, choices=[0, 1, 2, 3, 4],
                   help="bdf workload with --threads: matrix placement (codes of ember_mech_get_tuning; 0: first "
                        "that fits)")
    p.add_argument("--threads", type=int, default=0,
                   help="QSS threads per point; 0: ember_source_autotune picks it before the timed region")
    return p.parse_args()


# ---------------------------------------------------------------- clocks --

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ utilities --

def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float, ws: int, device) -> float:
    """The largest value over the ranks (each rank's timed total; replicas
    finish when the slowest does)."""
    if ws <= 1:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def workload_inputs(n_points: int, rank: int, mech_size: str = "150"):
    from ember_gb300.mechanism import synthetic_mechanism, reactor_states
    if mech_size == "53":
        mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)
    else:
        mech = synthetic_mechanism(seed=MECH_SEED)
    state, dt = reactor_states(mech, n_points, seed=STATE_SEED + rank)
    return mech, state, dt


def source_options(kinetics: str, method: str):
    from ember_gb300.source import SourceOptions, KINETICS_INTERP, KINETICS_STANDARD
    return SourceOptions.defaults(kinetics_model=KINETICS_INTERP if kinetics == "interp" else KINETICS_STANDARD)


def cpu_sample_rate(mech, state, dt, opts, method: int, target_s: float, threads: int):
    """Points/s of the CPU oracle on a bounded sample of the workload: the
    first n states, n grown until one pass takes a quarter of target_s.
    Returns (rate, n, seconds, (state_out, status, stats) of those n states)."""
    from oracle import chem
    om = chem.OracleMech(mech)
    n = 16
    t = 0.0
    while True:
        t0 = time.perf_counter()
        om.integrate(method, state[:n], dt[:n], opts, n_threads=threads)
        t = time.perf_counter() - t0
        if t >= 0.25 * target_s or n >= len(state):
            break
        n = min(len(state), int(n * max(2.0, min(8.0, 0.3 * target_s / max(t, 1e-3)))))
    # one more pass at the final sample size for the figure
    t0 = time.perf_counter()
    res = om.integrate(method, state[:n], dt[:n], opts, n_threads=threads)
    t = time.perf_counter() - t0
    return n / t, n, t, res


# How far the oracle itself is pinned to the reference (stated beside every parity figure).
ORACLE_PINS = ("the oracle is pinned to reference-held data only for the tridiagonal integrator (the reference's "
               "golden table) and the QSS integrator (the CHEMEQ2 cesium problem); kinetics, thermo, transport and "
               "the CVODE-method BDF and Adams integrators are unpinned restatements (Cantera and SUNDIALS are "
               "absent)")


def source_parity(out, status, stats, ref_out, ref_status, ref_stats) -> dict:
    """Agreement of a source-term batch with the oracle on the same states:
    points equal bit for bit, the largest relative error of T and of the
    mass fractions above 1e-14, the largest |sum Y - 1| of both results
    (the integrators do not renormalise), and status / counter mismatches."""
    import numpy as np
    g, r = np.asarray(out, dtype=np.float64), np.asarray(ref_out, dtype=np.float64)
    n = min(len(g), len(r))
    g, r = g[:n], r[:n]
    with np.errstate(divide="ignore", invalid="ignore"):
        rel_t = np.abs(g[:, 1] - r[:, 1]) / np.abs(r[:, 1])
        yr, yg = r[:, 2:], g[:, 2:]
        big = np.abs(yr) > 1e-14
        rel_y = np.where(big, np.abs(yg - yr) / np.where(big, np.abs(yr), 1.0), 0.0)
    return {
        "against": "oracle (FP64 CPU restatement of the reference path), same seeded states",
        "oracle_pins": ORACLE_PINS,
        "n_compared": int(n),
        "n_bitwise": int(np.all(g.view(np.int64) == r.view(np.int64), axis=1).sum()),
        "max_rel_err_T": float(np.nanmax(rel_t)) if n else 0.0,
        "max_rel_err_Y_above_1e-14": float(np.nanmax(rel_y)) if n else 0.0,
        "max_abs_sumY_minus_1": float(np.abs(yg.sum(axis=1) - 1.0).max()) if n else 0.0,
        "max_abs_sumY_minus_1_oracle": float(np.abs(yr.sum(axis=1) - 1.0).max()) if n else 0.0,
        "status_mismatches": int((np.asarray(status)[:n] != np.asarray(ref_status)[:n]).sum()),
        "counter_mismatches": int(np.any(np.asarray(stats)[:n] != np.asarray(ref_stats)[:n], axis=1).sum()),
        "failed_points_oracle": int((np.asarray(ref_status)[:n] != 0).sum()),
    }


def field_parity(rows, ref_rows, tol=None) -> dict:
    """Agreement of per-variable rows (list of 1-D arrays, GPU and oracle):
    rows equal bit for bit and the largest error relative to the row's
    largest |value| (the tolerance form of the tridiagonal path). With
    tol = [(rtol, atol) per row], also the largest |error| / (rtol |ref| +
    atol): the error in units of an integrator's own tolerance."""
    import numpy as np
    worst, same, worst_tol = 0.0, 0, 0.0
    for r, (a, b) in enumerate(zip(rows, ref_rows)):
        a, b = np.asarray(a), np.asarray(b)
        same += int(np.array_equal(a, b))
        scale = float(np.abs(b).max())
        err = float(np.abs(a - b).max())
        worst = max(worst, err / scale if scale > 0 else err)
        if tol is not None:
            rt, at = tol[r]
            worst_tol = max(worst_tol, float((np.abs(a - b) / (rt * np.abs(b) + at)).max()))
    out = {"against": "oracle (FP64 CPU restatement of the reference path), same seeded inputs", "oracle_pins": ORACLE_PINS,
           "n_compared": len(rows), "n_bitwise": same, "max_err_rel_to_row_max": worst}
    if tol is not None:
        out["max_err_in_tolerance_units"] = worst_tol
    return out


# ------------------------------------------------------- reference arm --

def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    from oracle import chem
    method = chem.QSS if args.workload == "qss" else chem.BDF
    mech, state, dt = workload_inputs(args.points, 0, args.mech)
    opts = source_options(args.kinetics, args.workload)
    threads = os.cpu_count() or 1
    om = chem.OracleMech(mech)
    # size one step's sample to ~args.cpu_seconds/2 of host work
    rate, n, t, _ = cpu_sample_rate(mech, state, dt, opts, method, args.cpu_seconds / 2, threads)
    for _ in range(args.warmup):
        om.integrate(method, state[:n], dt[:n], opts, n_threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        om.integrate(method, state[:n], dt[:n], opts, n_threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"C2 isolated source-term step, {args.workload.upper()}, {args.kinetics} kinetics, "
                               f"synthetic {mech.n_species}-species/{mech.n_reactions}-reaction mechanism, {args.points} seeded states",
                   "sample_points_per_step": n},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": f"{n} of the {args.points} states per step, all host threads"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# -------------------------------------------------------------- our arm --

def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300 import _lib
    from ember_gb300 import roofline
    from ember_gb300.source import GpuMechanism, integrate_production_terms, autotune, tuning, QSS, BDF, STATS_WIDTH
    import ctypes as C

    lib = _lib.lib()
    method = QSS if args.workload == "qss" else BDF
    mech, state, dt = workload_inputs(args.points, rank, args.mech)
    opts = source_options(args.kinetics, args.workload)
    gm = GpuMechanism(mech)
    dev = torch.device("cuda", local)
    st_d = torch.as_tensor(state, device=dev)
    dt_d = torch.as_tensor(dt, device=dev)
    out_d = torch.empty_like(st_d)
    status_d = torch.zeros(args.points, dtype=torch.int32, device=dev)
    stats_d = torch.zeros((args.points, STATS_WIDTH), dtype=torch.int32, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream()

    peak = C.c_double()
    _lib.check(lib.ember_probe_fp64_rate(0, C.byref(peak)), "probe")
    fp64_peak = peak.value

    # launch width: autotuned on this batch (outside the timed region), or given
    tune_ms = {}
    if args.threads == 0:
        # on the whole batch: a sample's makespan need not rank the candidates as the batch's does
        width, tune_ms = autotune(gm, method, st_d, dt_d, opts, stream=stream)
    else:
        width = args.threads
        opts.threads_per_point = width
        opts.bdf_layout = args.bdf_layout

    def step():
        integrate_production_terms(gm, method, st_d, dt_d, opts, out=out_d, status=status_d, stats=stats_d,
                                   stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    w0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - w0
    kernel_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(kernel_ms)
    total_ms = max_over_ranks(total_ms, ws, dev)

    # end to end through the public API with pinned host buffers (copies inside the call)
    st_h = torch.as_tensor(state).pin_memory()
    dt_h = torch.as_tensor(dt).pin_memory()
    out_h = torch.empty_like(st_h).pin_memory()
    status_h = torch.zeros(args.points, dtype=torch.int32).pin_memory()
    stats_h = torch.zeros((args.points, STATS_WIDTH), dtype=torch.int32).pin_memory()

    def step_host():
        integrate_production_terms(gm, method, st_h.numpy(), dt_h.numpy(), opts, out=out_h.numpy(),
                                   status=status_h.numpy(), stats=stats_h.numpy())

    step_host()
    if ws > 1:
        torch.distributed.barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_host()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_times)
    e2e_s = max_over_ranks(e2e_s, ws, dev)
    clocks = sampler.stop()

    status = status_d.cpu().numpy()
    stats = stats_d.cpu().numpy()
    n_fail = int((status != 0).sum())
    if method == QSS:
        flops = float(roofline.qss_point_flops(mech, opts.kinetics_model, stats[:, 0], stats[:, 1]).sum())
    else:
        flops = float(roofline.bdf_point_flops(mech, opts.kinetics_model, stats[:, 0], stats[:, 1],
                                               stats[:, 3]).sum())
    avg_launch_s = total_ms / args.steps / 1e3
    achieved = flops / avg_launch_s / 1e12
    peak_t = fp64_peak / 1e12

    # DRAM bytes per launch from the ncu captures of the integration kernels
    # (150-species mechanism), scaled to this launch's points.
    per_point = roofline.QSS_DRAM_BYTES_PER_POINT if method == QSS else roofline.BDF_DRAM_BYTES_PER_POINT
    traffic = per_point * args.points if args.mech == "150" else None

    line = {
        "metric": METRIC, "value": ws * args.points * args.steps / (total_ms / 1e3), "unit": "points/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mechanism and reactor states)",
        "config": {"workload": f"C2 isolated source-term step, {args.workload.upper()}, {args.kinetics} kinetics, "
                               f"synthetic {mech.n_species}-species/{mech.n_reactions}-reaction mechanism, {args.points} seeded states "
                               f"per GPU",
                   "points_per_gpu": args.points, "n_vars": mech.n_vars, "n_reactions": mech.n_reactions,
                   "l2": "256 MB buffer written between timed iterations", "parallelism": f"replicas x{ws}",
                   "failed_points": n_fail,
                   "mean_steps_per_point": float(stats[:, 0].mean()),
                   "mean_rhs_calls_per_point": float(stats[:, 1].mean()),
                   "threads_per_point": width or "default for the mechanism size",
                   "autotune_ms": {str(k): round(v, 2) for k, v in tune_ms.items()},
                   "tuning": tuning(gm)},
        "e2e": {"value": ws * args.points * args.steps / e2e_s, "unit": "points/s",
                "h2d_bytes_per_step": int(state.nbytes + dt.nbytes),
                "d2h_bytes_per_step": int(state.nbytes + status_h.numpy().nbytes + stats_h.numpy().nbytes)},
        "gpu_launches": 4 * args.steps,  # per call: 3 work-order kernels + the integrator
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak_t, "unit": "TFLOP/s",
                     "frac": achieved / peak_t, "traffic": traffic,
                     "peak_source": "live DFMA throughput probe (ember_probe_fp64_rate); MEASURED_PEAKS.json "
                                    "has no FP64 figure",
                     "work_model": "algorithmic flops of ember_gb300/roofline.py (exp/log/div = 1 flop)"},
        "clocks": clocks,
        "wall_s_timed_region": wall,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, n, t, ref = cpu_sample_rate(mech, state, dt, opts, method, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "points/s", "cores": threads, "kind": "port",
                                "sample": f"first {n} of the {args.points} states, {t:.1f} s on {threads} threads"}
        if n < args.points:  # the rest of the batch, for the parity figures only (not timed)
            from oracle import chem
            rest = chem.OracleMech(mech).integrate(method, state[n:], dt[n:], opts, n_threads=threads)
            ref = tuple(np.concatenate([a, b]) for a, b in zip(ref, rest))
        line["parity"] = source_parity(out_d.cpu().numpy(), status, stats, *ref)
    return line


# ------------------------------------------------- diffusion workload (C3) --

DIFF_METRIC = "tridiagonal value-updates/s"


def diffusion_inputs(rank: int):
    from ember_gb300.diffusion import synthetic_flames
    return synthetic_flames(seed=6455 + rank)


def run_reference_diffusion(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    import oracle
    grids, B, D, S, Y, h = diffusion_inputs(0)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.diffusion_batch(grids, B, D, S, Y, 0.0, 1e-5, h=h, n_threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.diffusion_batch(grids, B, D, S, Y, 0.0, 1e-5, h=h, n_threads=threads)
    total = time.perf_counter() - t0
    value = Y.size * args.steps / total
    print(json.dumps({
        "impl": "reference", "metric": DIFF_METRIC, "value": value, "unit": "values/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "C3 batched tridiagonal diffusion: 64 flames x 55 variables, N uniform 100-4000, "
                               "one BDF1x8 step of 1e-5 s", "values": int(Y.size)},
        "cpu_baseline": {"value": value, "unit": "values/s", "cores": threads, "kind": "port",
                         "sample": "the whole workload per step, all host threads"},
        "e2e": {"value": value, "unit": "values/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_ours_diffusion(args):
    import numpy as np
    import torch
    import ctypes as C
    ws, rank, local = dist_info()
    from ember_gb300 import _lib, roofline
    from ember_gb300.diffusion import integrate_diffusion_terms
    lib = _lib.lib()
    grids, B, D, S, Y, h = diffusion_inputs(rank)
    dev = torch.device("cuda", local)
    Bd, Dd, Sd = (torch.as_tensor(v, device=dev) for v in (B, D, S))
    Y0 = torch.as_tensor(Y, device=dev)
    Yd = Y0.clone()
    xd = torch.as_tensor(np.concatenate([g.x for g in grids]), device=dev)
    hd = torch.as_tensor(h, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    peak = C.c_double()
    _lib.check(lib.ember_probe_fp64_rate(0, C.byref(peak)), "probe")

    def step():
        Yd.copy_(Y0)
        integrate_diffusion_terms(grids, Bd, Dd, Sd, Yd, 0.0, 1e-5, h=hd, stream=stream, x=xd)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        Yd.copy_(Y0)
        flush.zero_()
        starts[i].record(stream)
        integrate_diffusion_terms(grids, Bd, Dd, Sd, Yd, 0.0, 1e-5, h=hd, stream=stream, x=xd)
        ends[i].record(stream)
    torch.cuda.synchronize()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    total_ms = max_over_ranks(total_ms, ws, dev)
    # end to end with host arrays in pinned memory (copies inside the call)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    Bh, Dh, Sh, Yh = pin(B), pin(D), pin(S), pin(Y)
    e2e = []
    for _ in range(args.steps):
        Yh[:] = Y
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        integrate_diffusion_terms(grids, Bh, Dh, Sh, Yh, 0.0, 1e-5, h=h)
        e2e.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    n_vals = int(Y.size)
    avg_s = total_ms / args.steps / 1e3
    flops = roofline.tridiag_flops_per_point() * n_vals
    achieved = flops / avg_s / 1e12
    line = {
        "metric": DIFF_METRIC, "value": ws * n_vals * args.steps / (total_ms / 1e3), "unit": "values/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded grids, diffusivities and profiles)",
        "config": {"workload": "C3 batched tridiagonal diffusion: 64 flames x 55 variables, N uniform 100-4000, "
                               "one BDF1x8 step of 1e-5 s per system", "values": n_vals,
                   "l2": "256 MB buffer written between timed iterations"},
        "e2e": {"value": ws * n_vals * args.steps / sum(e2e), "unit": "values/s",
                "h2d_bytes_per_step": int(B.nbytes + D.nbytes + S.nbytes + Y.nbytes),
                "d2h_bytes_per_step": int(Y.nbytes)},
        "gpu_launches": 2 * args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (peak.value / 1e12), "traffic": None,
                     "hbm_achieved_gbs": roofline.tridiag_bytes_per_point() * n_vals / avg_s / 1e9,
                     "peak_source": "live DFMA throughput probe (ember_probe_fp64_rate)"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        reps = 0
        ref = None
        while time.perf_counter() - t0 < args.cpu_seconds or reps == 0:
            ref = oracle.diffusion_batch(grids, B, D, S, Y, 0.0, 1e-5, h=h, n_threads=threads)
            reps += 1
        tcpu = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_vals * reps / tcpu, "unit": "values/s", "cores": threads, "kind": "port",
                                "sample": f"the whole workload x{reps}, {tcpu:.1f} s on {threads} threads"}
        gy = Yd.cpu().numpy()
        rows, ref_rows, p = [], [], 0
        nv = Y.size // sum(g.n_points for g in grids)
        for g in grids:
            for _ in range(nv):
                rows.append(gy[p:p + g.n_points])
                ref_rows.append(ref[p:p + g.n_points])
                p += g.n_points
        line["parity"] = field_parity(rows, ref_rows)
        line["parity"]["tolerance"] = "1e-12 of each system's largest |y| (warp-parallel Thomas vs the sequential order)"
    return line


# ------------------------------------------------ split-step workload (C5) --

SPLIT_METRIC = "ms per split step"
SPLIT_DT = 2e-5
SPLIT_WORKLOAD = ("C5 strain-sweep proxy: 32 seeded flame-like profiles (150-700 points), synthetic "
                  "150-species/1000-reaction mechanism, FlameSolver step without convection: thermo and "
                  "Approx transport (seeded kinetic-theory fits), B/D and cross terms from the step-start "
                  "state, balanced D-S-D split step (dt 2e-5 s; diffusion h rule, QSS source, interp kinetics)")
SPLIT_TRANSPORT_SEED = 1523
SPLIT_THRESHOLD = 1e-5


def split_inputs(rank: int, mech_size: str = "150"):
    from ember_gb300.mechanism import synthetic_mechanism
    from ember_gb300.split import flame_batch
    if mech_size == "53":
        mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)
    else:
        mech = synthetic_mechanism(seed=MECH_SEED)
    return (mech,) + flame_batch(mech, n_flames=32, n_min=150, n_max=700, seed=3232 + rank)


def split_workload(args, mech) -> str:
    w = SPLIT_WORKLOAD.replace("150-species/1000-reaction", f"{mech.n_species}-species/{mech.n_reactions}-reaction") \
        .replace("QSS source", f"{args.source.upper()} source").replace("dt 2e-5 s", f"dt {args.split_dt or SPLIT_DT:g} s")
    if args.convection:
        w = w.replace("FlameSolver step without convection", "FlameSolver step with convection") \
            .replace("balanced D-S-D split step", "balanced D-C-D-S-D-C-D split step (three-operator split constants)")
        w += ("; convection: strain rates 100-2000 1/s log-spaced over the flames, U = a sqrt(rho_u/rho), inflow "
              "through the left boundary")
    return w


def split_convection(mech, grids, state, rho_u):
    """Convection parameters for the split workload: U = a sqrt(rho_u / rho)
    (written into ``state``), strain rates log-spaced 100-2000 1/s, the
    continuity integral from the left with inflow rho_u * 0.4 m/s."""
    import numpy as np
    from ember_gb300.convection import BC_CONTROL_VOLUME, ConvectionFlame, mean_molecular_weight
    from ember_gb300.split import mixture_properties
    rho, _ = mixture_properties(mech, state)
    strains = np.geomspace(100.0, 2000.0, len(grids))
    flames, y_left = [], []
    p = 0
    for f, g in enumerate(grids):
        N = g.n_points
        a = float(strains[f])
        state[p:p + N, 0] = a * np.sqrt(rho_u[f] / rho[p:p + N])
        y0 = state[p, 2:].copy()
        flames.append(ConvectionFlame(n_points=N, left_bc=g.left_bc, right_bc=g.right_bc, alpha=g.alpha,
                                      rv_zero=0.4 * float(rho_u[f]), t_left=float(state[p, 1]),
                                      w_left=float(mean_molecular_weight(y0, mech.mol_weight)[0]),
                                      rhou=float(rho_u[f]), strain_initial=a, strain_final=a))
        y_left.append(y0)
        p += N
    return flames, np.array(y_left)


def run_reference_split(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    from oracle.chem import OracleMech
    from oracle import split as osplit
    from ember_gb300.source import QSS, BDF
    mech, grids, state, B, D, rho_u, ju, jb = split_inputs(0, args.mech)
    opts = source_options(args.kinetics, args.source)
    method = QSS if args.source == "qss" else BDF
    split_dt = args.split_dt or SPLIT_DT
    om = OracleMech(mech)
    conv = None
    if args.convection:
        from ember_gb300.convection import ConvectionOptions
        cflames, y_left = split_convection(mech, grids, state, rho_u)
        conv = (cflames[:1], y_left[:1], ConvectionOptions())
    # bounded sample: the first flame, one split step per timed step
    g0 = grids[:1]
    n0 = g0[0].n_points
    nv = mech.n_vars
    st0, B0, D0 = state[:n0], B[:nv * n0], D[:nv * n0]
    from ember_gb300.transport import synthetic_transport
    tr = (synthetic_transport(mech, seed=SPLIT_TRANSPORT_SEED), SPLIT_THRESHOLD, True)
    for _ in range(args.warmup):
        osplit.split_steps(om, g0, st0, 0.0, B0, D0, split_dt, 1, method, opts, transport=tr, convection=conv)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        osplit.split_steps(om, g0, st0, 0.0, B0, D0, split_dt, 1, method, opts, transport=tr, convection=conv)
    per_flame = (time.perf_counter() - t0) / args.steps
    # scaled to the 32-flame batch by points
    ms = 1e3 * per_flame * len(state) / n0
    threads = os.cpu_count() or 1
    print(json.dumps({
        "impl": "reference", "metric": SPLIT_METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": split_workload(args, mech), "points": int(len(state))},
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": threads, "kind": "port",
                         "sample": f"flame 0 ({n0} points) per step, scaled to {len(state)} points"
                                   + ("; flame 0 has the lowest strain rate, so its convection stages take the "
                                      "fewest steps" if args.convection else "")},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def _flame_ranges(sizes):
    """(first, end) point of each flame of a batch with these point counts."""
    import numpy as np
    off = np.cumsum([0] + list(sizes))
    return [(int(off[i]), int(off[i + 1])) for i in range(len(sizes))]


def run_ours_split(args):
    import ctypes as C
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300 import _lib, roofline
    from ember_gb300.source import GpuMechanism, QSS, BDF, autotune, tuning
    from ember_gb300.split import FlameBatchSplitSolver
    mech, grids, state, B, D, rho_u, ju, jb = split_inputs(rank, args.mech)
    opts = source_options(args.kinetics, args.source)
    method = QSS if args.source == "qss" else BDF
    split_dt = args.split_dt or SPLIT_DT
    cflames = y_left = copts = None
    if args.convection:
        from ember_gb300.convection import ConvectionOptions
        cflames, y_left = split_convection(mech, grids, state, rho_u)
        copts = ConvectionOptions()
    gm = GpuMechanism(mech)
    # QSS launch width tuned on the flames' start states over one step (before the solver takes it)
    width, tune_ms = autotune(gm, method, state, np.full(len(state), split_dt), opts)
    solver = FlameBatchSplitSolver(gm, grids, split_dt, method=method, source_options=opts)
    from ember_gb300.transport import GpuTransport, synthetic_transport
    tdata = synthetic_transport(mech, seed=SPLIT_TRANSPORT_SEED)
    gtr = GpuTransport(gm, tdata)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    peak = C.c_double()
    _lib.check(_lib.lib().ember_probe_fp64_rate(0, C.byref(peak)), "probe")
    solver.set_state(0.0, state)
    solver.set_transport(B, D)
    solver.set_transport_model(gtr, SPLIT_THRESHOLD, cross_terms=True)
    if args.convection:
        solver.set_convection(cflames, y_left, copts)
    solver.step(args.warmup, graph=True, stream=stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    src_flops = 0.0
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        solver.step(1, graph=True, stream=stream)
        ends[i].record(stream)
        torch.cuda.synchronize()
        _, stats = solver.source_status()
        if method == QSS:
            src_flops += float(roofline.qss_point_flops(mech, opts.kinetics_model, stats[:, 0], stats[:, 1]).sum())
        else:
            src_flops += float(roofline.bdf_point_flops(mech, opts.kinetics_model, stats[:, 0], stats[:, 1],
                                                        stats[:, 3]).sum())
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    total_ms = max_over_ranks(total_ms, ws, dev)
    n_fail_src, n_fail_diff = solver.failures()
    # end to end: the last step's state in from the host, one step, the state out to the host
    e2e = []
    host, _ = solver.state()
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.load_state(host)
        solver.step(1, graph=True)
        host, _ = solver.state()
        e2e.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    ms = total_ms / args.steps
    # the plain per-flame GPU path beside it: one solver per flame, stream launches, flames one after another
    plain_ms = 0.0
    if not args.no_plain:
        nv = mech.n_vars
        off = np.cumsum([0] + [g.n_points for g in grids])
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for f in range(len(grids)):
            a, b = off[f], off[f + 1]
            one = FlameBatchSplitSolver(gm, grids[f:f + 1], split_dt, method=method, source_options=opts)
            one.set_state(0.0, state[a:b])
            one.set_transport(B[a * nv:b * nv], D[a * nv:b * nv])
            one.set_transport_model(gtr, SPLIT_THRESHOLD, cross_terms=True)
            if args.convection:
                one.set_convection(cflames[f:f + 1], y_left[f:f + 1], copts)
            one.step(args.warmup, graph=False, stream=stream)
            torch.cuda.synchronize()
            e0.record(stream)
            one.step(args.steps, graph=False, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            plain_ms += e0.elapsed_time(e1) / args.steps
            del one
    n_vals = state.size
    flops = (src_flops / args.steps + 4 * roofline.tridiag_flops_per_point() * n_vals
             + float(np.sum(roofline.transport_point_flops(mech.n_species,
                                                           major_counts(mech, state[:, 2:], SPLIT_THRESHOLD)))))
    achieved = flops / (ms / 1e3) / 1e12
    line = {
        "metric": SPLIT_METRIC, "value": ms, "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded flame-like profiles, synthetic transport)",
        "config": {"workload": split_workload(args, mech), "points": int(len(state)), "flames": len(grids),
                   "points_per_s": len(state) / (ms / 1e3), "l2": "256 MB buffer written between timed steps",
                   "graph": True, "failed_source_points": n_fail_src, "failed_diffusion_systems": n_fail_diff,
                   "threads_per_point": width, "autotune_ms": {str(k): round(v, 2) for k, v in tune_ms.items()},
                   "tuning": tuning(gm),
                   "plain_per_flame_ms": plain_ms if not args.no_plain else None,
                   "batched_vs_plain_per_flame": plain_ms / ms if not args.no_plain else None},
        "e2e": {"value": 1e3 * sum(e2e) / len(e2e), "unit": "ms", "h2d_bytes_per_step": int(state.nbytes),
                "d2h_bytes_per_step": int(state.nbytes)},
        # per step: transport, B/D, jCorr (flux, step size, 2 integrator kernels, failure count), 2 cross-term
        # kernels; begin, 2 x (transpose, 2 x (stage, failure count, delta), transpose back), stage dt,
        # 3 work-order kernels + QSS, failure count, end, mass fractions, clock
        # with the convection stage: the density derivative, and per half 3 convection kernels, failure
        # count and delta (the diffusion pairs become single stages around it, same launches)
        "gpu_launches": (46 if args.convection else 35) * args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (peak.value / 1e12), "traffic": None,
                     "peak_source": "live DFMA throughput probe (ember_probe_fp64_rate)",
                     "work_model": "QSS flops of the source stage + 4 diffusion stages x 73 flops/value + transport and "
                                   "cross terms per point (roofline.py)"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        from oracle.chem import OracleMech
        from oracle import split as osplit
        om = OracleMech(mech)
        n0 = grids[0].n_points
        nv = mech.n_vars
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < args.cpu_seconds or reps == 0:
            osplit.split_steps(om, grids[:1], state[:n0], 0.0, B[:nv * n0], D[:nv * n0], split_dt, 1, method, opts,
                               transport=(tdata, SPLIT_THRESHOLD, True),
                               convection=(cflames[:1], y_left[:1], copts) if args.convection else None)
            reps += 1
        tcpu = (time.perf_counter() - t0) / reps
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = {"value": 1e3 * tcpu * len(state) / n0, "unit": "ms", "cores": threads,
                                "kind": "port",
                                "sample": f"flame 0 ({n0} points) x{reps} on {threads} threads, scaled by points"
                                          + ("; flame 0 has the lowest strain rate, so its convection stages take "
                                             "the fewest steps" if args.convection else "")}
        # parity: one step of the batched solver from the start state, against the oracle's step of
        # the first, middle and last flame (flames are independent, so a subset steps as in the batch)
        solver.set_state(0.0, state)
        solver.step(1, graph=True, stream=stream)
        torch.cuda.synchronize()
        gpu_state, _ = solver.state()
        sel = sorted({0, len(grids) // 2, len(grids) - 1})
        off = np.cumsum([0] + [g.n_points for g in grids])
        pick = lambda a, per: np.concatenate([a[off[f] * per:off[f + 1] * per] for f in sel])
        ref_state, _, _, _, _ = osplit.split_steps(
            om, [grids[f] for f in sel], pick(state.reshape(-1), nv).reshape(-1, nv), 0.0, pick(B, nv), pick(D, nv),
            split_dt, 1, method, opts, transport=(tdata, SPLIT_THRESHOLD, True),
            convection=([cflames[f] for f in sel], y_left[sel], copts) if args.convection else None)
        rows, ref_rows, tol, p = [], [], [], 0
        for f in sel:
            a, b = off[f], off[f + 1]
            for v in range(nv):
                rows.append(gpu_state[a:b, v])
                ref_rows.append(ref_state[p:p + (b - a), v])
                if args.convection:   # the loosest integrator on the path: the convection stage's Adams
                    atol = (copts.abstol_u, copts.abstol_t)[v] if v < 2 else copts.abstol_y
                    tol.append((copts.reltol, atol))
                else:
                    atol = (opts.bdf_abstol_momentum, opts.bdf_abstol_energy)[v] if v < 2 else opts.bdf_abstol_species
                    tol.append((opts.bdf_reltol, atol))
            p += b - a
        adaptive = method == BDF or args.convection
        line["parity"] = field_parity(rows, ref_rows, tol if adaptive else None)
        # the same flames through the serial diffusion algorithm (the reference's sequential
        # Thomas order): the rest of the step is then bitwise the oracle's
        ser = FlameBatchSplitSolver(gm, [grids[f] for f in sel], split_dt, method=method, source_options=opts,
                                    diffusion_algorithm=_lib.DIFFUSION_SERIAL)
        ser.set_state(0.0, pick(state.reshape(-1), nv).reshape(-1, nv))
        ser.set_transport(pick(B, nv), pick(D, nv))
        ser.set_transport_model(gtr, SPLIT_THRESHOLD, cross_terms=True)
        if args.convection:
            ser.set_convection([cflames[f] for f in sel], y_left[sel], copts)
        ser.step(1, graph=False, stream=stream)
        torch.cuda.synchronize()
        ser_state, _ = ser.state()
        ranges = _flame_ranges([grids[f].n_points for f in sel])
        line["parity"]["serial_diffusion"] = {
            "n_compared": len(ranges) * nv,
            "n_bitwise": int(sum(np.array_equal(ser_state[a:b, v], ref_state[a:b, v]) for a, b in ranges
                                 for v in range(nv))),
            "max_abs_err": float(np.abs(ser_state - ref_state).max())}
        del ser
        if args.convection:
            line["parity"]["tolerance"] = ("|error| / (reltol |y| + abstol) with the convection stage's tolerances "
                                           "(reltol 1e-6; abstol 1e-7 U, 1e-8 T, 1e-13 Y): rounding-level "
                                           "differences of the parallel diffusion can change its adaptive steps")
        elif method == BDF:
            line["parity"]["tolerance"] = ("BDF: |error| / (reltol |y| + abstol) with the source options' CVODE "
                                           "tolerances (reltol 1e-6; abstol 1e-7 U, 1e-8 T, 1e-13 Y)")
        line["parity"].update({"flames_compared": sel, "steps": 1,
                               "note": "the product path runs warp-parallel diffusion (rounding-level differences "
                                       "from the sequential order, which the adaptive integrators after it can "
                                       "amplify up to their tolerances); serial_diffusion: the same flames and step "
                                       "with the sequential algorithm"})
    return line


# ---------------------------------------------------- adjoint workload (C4) --

ADJ_METRIC = "adjoint/forward cost"
ADJ_DT = 2e-5
ADJ_WORKLOAD = ("C4 proxy: one flame-like profile of 400 points, synthetic 53-species/325-reaction mechanism "
                "(GRI-3.0 sizes), balanced D-S-D split step (dt 2e-5 s, {src}), "
                "gradient of heat release + consumption speed w.r.t. the start state and ln A of every reaction")
ADJ_SOURCES = {"bdf": "BDF source with CVODE default tolerances",
               "qss": "QSS source (the reference's default integrator) with its default options"}


def adjoint_method(args):
    from ember_gb300.source import BDF, QSS
    return BDF if args.source == "bdf" else QSS


def adjoint_inputs(rank: int):
    from ember_gb300.mechanism import synthetic_mechanism
    from ember_gb300.split import flame_batch
    mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53325)
    return (mech,) + flame_batch(mech, n_flames=1, n_min=400, n_max=400, seed=4000 + rank)


def run_reference_adjoint(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    from oracle.chem import OracleMech
    from oracle import split as osplit
    method = adjoint_method(args)
    mech, grids, state, B, D, rho_u, ju, jb = adjoint_inputs(0)
    opts = source_options(args.kinetics, args.source)
    om = OracleMech(mech)
    for _ in range(args.warmup):
        osplit.split_steps(om, grids, state, 0.0, B, D, ADJ_DT, 1, method, opts)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        osplit.split_steps(om, grids, state, 0.0, B, D, ADJ_DT, 1, method, opts)
    fwd = (time.perf_counter() - t0) / args.steps
    # the reference has no adjoint: central differences need 2 forward steps per ln A
    ratio = 2.0 * mech.n_reactions
    threads = os.cpu_count() or 1
    print(json.dumps({
        "impl": "reference", "metric": ADJ_METRIC, "value": ratio, "unit": "x", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * fwd * ratio, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ADJ_WORKLOAD.format(src=ADJ_SOURCES[args.source]), "forward_ms": 1e3 * fwd,
                   "gradient_method": "central differences of the CPU split step (2 steps per ln A)"},
        "cpu_baseline": {"value": ratio, "unit": "x", "cores": threads, "kind": "port",
                         "sample": f"one forward split step of the 400-point flame, {1e3 * fwd:.1f} ms"},
        "e2e": {"value": ratio, "unit": "x", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_ours_adjoint(args):
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300.source import GpuMechanism
    from ember_gb300.split import FlameBatchSplitSolver
    method = adjoint_method(args)
    mech, grids, state, B, D, rho_u, ju, jb = adjoint_inputs(rank)
    opts = source_options(args.kinetics, args.source)
    gm = GpuMechanism(mech)
    solver = FlameBatchSplitSolver(gm, grids, ADJ_DT, method=method, source_options=opts)
    solver.set_transport(B, D)
    stream = torch.cuda.current_stream()
    wq, wsc = np.ones(1), np.ones(1)

    def forward():
        solver.set_state(0.0, state)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.step(1, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def adjoint():
        solver.set_state(0.0, state)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = solver.adjoint(wq, wsc, rho_u, ju, jb, tape_cap=4096)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    for _ in range(args.warmup):
        forward()
        adjoint()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    fw, ad = [], []
    for _ in range(args.steps):
        fw.append(forward())
        t_ad, (hr, cs, sbar, lbar) = adjoint()
        ad.append(t_ad)
    clocks = sampler.stop()
    fwd_ms, adj_ms = sum(fw) / len(fw), sum(ad) / len(ad)
    line = {
        "metric": ADJ_METRIC, "value": adj_ms / fwd_ms, "unit": "x", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": adj_ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded flame-like profile, synthetic transport)",
        "config": {"workload": ADJ_WORKLOAD.format(src=ADJ_SOURCES[args.source]), "forward_ms": fwd_ms,
                   "adjoint_ms": adj_ms,
                   "gradients": int(state.size + mech.n_reactions), "heat_release": float(hr[0]),
                   "consumption_speed": float(cs[0])},
        "e2e": {"value": adj_ms / fwd_ms, "unit": "x", "h2d_bytes_per_step": int(state.nbytes),
                "d2h_bytes_per_step": int(state.nbytes + 8 * mech.n_reactions)},
        "gpu_launches": None,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        from oracle.chem import OracleMech
        from oracle import split as osplit
        om = OracleMech(mech)
        t0 = time.perf_counter()
        osplit.split_steps(om, grids, state, 0.0, B, D, ADJ_DT, 1, method, opts)
        tcpu = time.perf_counter() - t0
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = {"value": 2.0 * mech.n_reactions, "unit": "x", "cores": threads, "kind": "port",
                                "sample": f"central differences on the CPU split step: 2 x {mech.n_reactions} "
                                          f"forward steps of {1e3 * tcpu:.0f} ms each ({threads} threads)"}
        ref_state, _, _, _, _ = osplit.split_steps(om, grids, state, 0.0, B, D, ADJ_DT, 1, method, opts)
        _, rhr, rcs = osplit.objectives(om, grids, ref_state, opts.pressure, opts.kinetics_model, rho_u, ju, jb)
        line["parity"] = {"against": "oracle split step and objectives (FP64 CPU restatement), same start state",
                          "oracle_pins": ORACLE_PINS,
                          "heat_release_rel_err": float(abs(hr[0] - rhr[0]) / abs(rhr[0])),
                          "consumption_speed_rel_err": float(abs(cs[0] - rcs[0]) / abs(rcs[0])),
                          "note": "forward objectives of the taped step; the gradients are checked against "
                                  "central differences of the oracle in tests/test_adjoint.py"}
    return line


# ------------------------------------------------------ transport workload --

TRANSPORT_METRIC = "transport property evaluations/s"
TRANSPORT_POINTS = 16384
TRANSPORT_WORKLOAD = ("updateChemicalProperties of 16384 seeded states (the C2 state distribution): thermo and "
                      "Approx mixture-averaged transport (threshold 1e-5), synthetic 150-species mechanism with "
                      "seeded kinetic-theory fits")


def major_counts(mech, Y, threshold):
    """Species per state whose mole fraction is at least the threshold."""
    import numpy as np
    y = np.maximum(np.asarray(Y, dtype=float), 0.0)
    xw = y / mech.mol_weight[None, :]
    X = xw / xw.sum(axis=1, keepdims=True)
    return (np.maximum(X, 1e-20) >= threshold).sum(axis=1)


def transport_inputs(rank: int):
    from ember_gb300.mechanism import reactor_states, synthetic_mechanism
    from ember_gb300.transport import synthetic_transport
    mech = synthetic_mechanism(seed=MECH_SEED)
    state, _ = reactor_states(mech, TRANSPORT_POINTS, seed=4096 + rank)
    return mech, synthetic_transport(mech, seed=SPLIT_TRANSPORT_SEED), state


def _transport_cpu_rate(mech, td, state, target_s: float, threads: int = 1):
    """States/s of the threaded oracle: a growing prefix of the states, then
    repeats of all of them, until the sample takes a quarter of target_s."""
    from oracle import chem
    om = chem.OracleMech(mech)
    n = 8 * threads
    while True:
        reps, t0 = 0, time.perf_counter()
        while True:
            chem.transport_eval(om, td, state[:n, 1], state[:n, 2:], 101325.0, SPLIT_THRESHOLD, n_threads=threads)
            reps += 1
            t = time.perf_counter() - t0
            if n < len(state) or t > target_s / 4:
                break
        if t > target_s / 4 or n >= len(state):
            return n * reps / t, n * reps, t
        n = min(len(state), n * 4)


def run_reference_transport(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    mech, td, state = transport_inputs(0)
    threads = os.cpu_count() or 1
    rates = [_transport_cpu_rate(mech, td, state, args.cpu_seconds / max(args.steps, 1), threads)
             for _ in range(args.steps)]
    rate = statistics.median(r[0] for r in rates)
    print(json.dumps({
        "impl": "reference", "metric": TRANSPORT_METRIC, "value": rate, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * TRANSPORT_POINTS / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": TRANSPORT_WORKLOAD, "points": TRANSPORT_POINTS},
        "cpu_baseline": {"value": rate, "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": f"{rates[0][1]} state evaluations per step, {threads} threads"},
        "e2e": {"value": rate, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_ours_transport(args):
    import ctypes as C
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300 import _lib, roofline
    from ember_gb300.source import GpuMechanism
    from ember_gb300.transport import GpuTransport
    mech, td, state = transport_inputs(rank)
    gm = GpuMechanism(mech)
    gt = GpuTransport(gm, td)
    dev = torch.device("cuda", local)
    T_d = torch.as_tensor(np.ascontiguousarray(state[:, 1]), device=dev)
    Y_d = torch.as_tensor(np.ascontiguousarray(state[:, 2:]), device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    peak = C.c_double()
    _lib.check(_lib.lib().ember_probe_fp64_rate(0, C.byref(peak)), "probe")
    for _ in range(args.warmup):
        gt.eval(T_d, Y_d, threshold=SPLIT_THRESHOLD, stream=stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        gt.eval(T_d, Y_d, threshold=SPLIT_THRESHOLD, stream=stream)
        ends[i].record(stream)
    torch.cuda.synchronize()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    total_ms = max_over_ranks(total_ms, ws, dev)
    # end to end: host states in, properties out, both in page-locked host memory
    n_pts_t = len(state)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    T_h, Y_h = pin(state[:, 1]), pin(state[:, 2:])
    S_ = mech.n_species
    out = {k: torch.empty(shp, dtype=torch.float64).pin_memory().numpy()
           for k, shp in (("density", (n_pts_t,)), ("mean_mol_weight", (n_pts_t,)), ("cp_mass", (n_pts_t,)),
                          ("cp_species", (n_pts_t, S_)), ("h_species", (n_pts_t, S_)),
                          ("conductivity", (n_pts_t,)), ("viscosity", (n_pts_t,)), ("rho_d", (n_pts_t, S_)))}
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gt.eval(T_h, Y_h, threshold=SPLIT_THRESHOLD, out=out)
        e2e.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    ms = total_ms / args.steps
    n = TRANSPORT_POINTS
    flops = float(np.sum(roofline.transport_point_flops(mech.n_species, major_counts(mech, state[:, 2:],
                                                                                     SPLIT_THRESHOLD),
                                                         cross_terms=False)))
    achieved = flops / (ms / 1e3) / 1e12
    S = mech.n_species
    line = {
        "metric": TRANSPORT_METRIC, "value": ws * n / (ms / 1e3), "unit": "points/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded states and transport fits)",
        "config": {"workload": TRANSPORT_WORKLOAD, "points": n, "n_species": S,
                   "l2": "256 MB buffer written between timed iterations"},
        "e2e": {"value": ws * n * len(e2e) / sum(e2e), "unit": "points/s",
                "h2d_bytes_per_step": int(T_h.nbytes + Y_h.nbytes),
                "d2h_bytes_per_step": int(sum(v.nbytes for v in out.values()))},
        "gpu_launches": args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (peak.value / 1e12), "traffic": None,
                     "peak_source": "live DFMA throughput probe (ember_probe_fp64_rate)",
                     "work_model": "roofline.transport_point_flops with each state's major-species count"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, ns, t = _transport_cpu_rate(mech, td, state, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "points/s", "cores": threads, "kind": "port",
                                "sample": f"{ns} state evaluations, {t:.1f} s on {threads} threads"}
    return line

# ------------------------------------------------------------ convection --

CONV_METRIC = "convection-stage points/s"
CONV_DT = 1e-5
CONV_WORKLOAD = ("convection stage (ConvectionSystemSplit::integrateToTime) of 32 seeded strained-flame profiles "
                 "(150-700 points, strain rates 100-2000 1/s), synthetic 53-species mechanism: per flame the UTW "
                 "system and 53 species systems, Adams integrators, one stage of 1e-5 s (half the 2e-5 s global "
                 "step)")


def convection_inputs(rank: int):
    from ember_gb300.convection import convection_batch
    from ember_gb300.mechanism import synthetic_mechanism
    mech = synthetic_mechanism(n_species=53, n_reactions=325, seed=53_325)
    return mech, convection_batch(mech, n_flames=32, n_min=150, n_max=700, seed=3232 + rank, split_scale=0.1,
                                  drhodt_scale=0.1)


def _convection_cpu_rate(mech, b, target_s: float, threads: int):
    """Points/s of the oracle over whole flames, one flame per thread (ctypes
    releases the interpreter lock), on a growing prefix of the flames."""
    from concurrent.futures import ThreadPoolExecutor
    from ember_gb300.convection import ConvectionOptions
    from oracle import convection as oc
    S = mech.n_species
    opts = ConvectionOptions()
    offs, voffs = [0], [0]
    for fl in b.flames:
        offs.append(offs[-1] + fl.n_points)
        voffs.append(voffs[-1] + (S + 2) * fl.n_points)

    def one(f):
        fl = b.flames[f]
        p0, p1, v0, v1 = offs[f], offs[f + 1], voffs[f], voffs[f + 1]
        oc.convection_flame(fl, mech.mol_weight, b.x[p0:p1], b.y_left[f], b.drhodt[p0:p1], b.split_const[v0:v1],
                            b.state[v0:v1], 0.0, CONV_DT, opts)
        return fl.n_points

    n = min(len(b.flames), threads)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        while True:
            t0 = time.perf_counter()
            pts = sum(ex.map(one, range(n)))
            t = time.perf_counter() - t0
            if t > target_s / 4 or n >= len(b.flames):
                return pts / t, n, t
            n = min(len(b.flames), n * 2)


def run_reference_convection(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    mech, b = convection_inputs(0)
    threads = os.cpu_count() or 1
    rates = [_convection_cpu_rate(mech, b, args.cpu_seconds / max(args.steps, 1), threads)
             for _ in range(args.steps)]
    rate = statistics.median(r[0] for r in rates)
    total = sum(fl.n_points for fl in b.flames)
    print(json.dumps({
        "impl": "reference", "metric": CONV_METRIC, "value": rate, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": CONV_WORKLOAD, "flames": len(b.flames), "points": total},
        "cpu_baseline": {"value": rate, "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": f"first {rates[0][1]} flames per step, one flame per thread, {threads} threads"},
        "e2e": {"value": rate, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_ours_convection(args):
    import ctypes as C
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300 import _lib, roofline
    from ember_gb300.convection import ConvectionOptions, integrate_convection_terms
    mech, b = convection_inputs(rank)
    S = mech.n_species
    dev = torch.device("cuda", local)
    opts = ConvectionOptions()
    x_d, yl_d, dr_d, sc_d = (torch.as_tensor(np.ascontiguousarray(a), device=dev)
                             for a in (b.x, b.y_left, b.drhodt, b.split_const))
    W_d = torch.as_tensor(mech.mol_weight, device=dev)
    init_d = torch.as_tensor(b.state, device=dev)
    work = init_d.clone()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    peak = C.c_double()
    _lib.check(_lib.lib().ember_probe_fp64_rate(0, C.byref(peak)), "probe")

    def stage():
        return integrate_convection_terms(b.flames, W_d, x_d, yl_d, dr_d, sc_d, work, 0.0, CONV_DT, opts,
                                          stream=stream)


    for _ in range(args.warmup):
        work.copy_(init_d)
        stage()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        work.copy_(init_d)
        flush.zero_()
        starts[i].record(stream)
        _, status, stats = stage()
        ends[i].record(stream)
    torch.cuda.synchronize()
    total_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    total_ms = max_over_ranks(total_ms, ws, dev)
    status = status.cpu().numpy()
    stats = stats.cpu().numpy()
    # end to end: host arrays in, the state back on the host
    e2e = []
    for _ in range(args.steps):
        st_h = b.state.copy()
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        integrate_convection_terms(b.flames, mech.mol_weight, b.x, b.y_left, b.drhodt, b.split_const, st_h, 0.0,
                                   CONV_DT, opts)
        e2e.append(time.perf_counter() - t0)
    clocks = sampler.stop()
    ms = total_ms / args.steps
    npts = int(sum(fl.n_points for fl in b.flames))
    Ns = np.array([fl.n_points for fl in b.flames], dtype=float)
    flops = float(np.sum(roofline.convection_flame_flops(Ns, stats)))
    achieved = flops / (ms / 1e3) / 1e12
    h2d = b.state.nbytes + b.split_const.nbytes + b.x.nbytes + b.drhodt.nbytes + b.y_left.nbytes
    line = {
        "metric": CONV_METRIC, "value": ws * npts / (ms / 1e3), "unit": "points/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded strained-flame profiles)",
        "config": {"workload": CONV_WORKLOAD, "flames": len(b.flames), "points": npts, "n_species": S,
                   "failed_systems": int((status != 0).sum()),
                   "mean_utw_steps": float(stats[:, 0].mean()),
                   "mean_species_steps": float(stats[:, 2].sum() / (S * len(b.flames))),
                   "l2": "256 MB buffer written between timed iterations"},
        "e2e": {"value": ws * npts * len(e2e) / sum(e2e), "unit": "points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(b.state.nbytes)},
        "gpu_launches": 3 * args.steps,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (peak.value / 1e12), "traffic": None,
                     "peak_source": "live DFMA throughput probe (ember_probe_fp64_rate)",
                     "work_model": "roofline.convection_flame_flops over the measured step and RHS counts"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, nf, t = _convection_cpu_rate(mech, b, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "points/s", "cores": threads, "kind": "port",
                                "sample": f"first {nf} flames, one flame per thread, {t:.1f} s on {threads} threads"}
    return line


# ------------------------------------------------------ secondary figures --

# The other parts of the headline metric ("ms per split step; adjoint/forward
# cost") and the other configurations, measured in the same default run beside
# the headline: (workload overrides, timed steps, CPU-sample seconds).
SECONDARY = (
    ("bdf", {"workload": "bdf", "mech": "150"}, 5, 4.0),
    ("diffusion", {"workload": "diffusion"}, 10, 2.0),
    ("split_bdf53", {"workload": "split", "mech": "53", "source": "bdf", "split_dt": 5e-6}, 3, 4.0),
    ("split_qss150", {"workload": "split", "mech": "150", "source": "qss", "split_dt": 0.0}, 5, 4.0),
    # the reference's full D C D S D C D step at 5e-6 s: at the 2e-5 s of the other split lines these
    # seeded, non-converged profiles diverge within five steps once convection is on (the oracle shows
    # failed points from step 4 and 30-280 times the integrator steps by step 10), at 5e-6 s they do not
    ("split_conv53", {"workload": "split", "mech": "53", "source": "qss", "split_dt": 5e-6, "convection": True},
     3, 4.0),
    ("adjoint", {"workload": "adjoint", "source": "bdf"}, 3, 1.0),
    ("adjoint_qss", {"workload": "adjoint", "source": "qss"}, 3, 1.0),
)

RUNNERS = {}


# ------------------------------------------- strain sweep run (C5 loop) --

SWEEP_METRIC = "ms per split step with regrids and termination tests"


def run_ours_sweep(args):
    """The C5 proxy through FlameBatchRun: split steps of the 32-flame batch
    with FlameSolver's loop around them (heat release and consumption speed
    recorded every step, termination tests every 10 steps, a regrid of every
    flame every --regrid-interval steps with the batch rebuilt on the new
    grids and its graph captured again). The timed region is the whole loop,
    host work included."""
    import numpy as np
    import torch
    ws, rank, local = dist_info()
    from ember_gb300.source import GpuMechanism, QSS, BDF, autotune, tuning
    from ember_gb300.sweep import FlameBatchRun, TerminationOptions
    from ember_gb300.transport import GpuTransport, synthetic_transport
    mech, grids, state, B, D, rho_u, ju, jb = split_inputs(rank, args.mech)
    opts = source_options(args.kinetics, args.source)
    method = QSS if args.source == "qss" else BDF
    split_dt = args.split_dt or SPLIT_DT
    conv = None
    if args.convection:
        from ember_gb300.convection import ConvectionOptions
        flames, y_left = split_convection(mech, grids, state, rho_u)
        conv = (flames, y_left, ConvectionOptions())
    gm = GpuMechanism(mech)
    width, tune_ms = autotune(gm, method, state, np.full(len(state), split_dt), opts)
    gtr = GpuTransport(gm, synthetic_transport(mech, seed=SPLIT_TRANSPORT_SEED))
    term = TerminationOptions(regrid_step_interval=args.regrid_interval)
    strains = list(np.geomspace(100.0, 2000.0, len(grids)))
    run = FlameBatchRun(gm, gtr, grids, state, split_dt, rho_u, method=method, source_options=opts,
                        threshold=SPLIT_THRESHOLD, convection=conv, strain_rates=strains, termination=term)
    run.run(args.warmup)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    rebuilds0, steps0 = run.n_rebuilds, run.n_steps
    t0 = time.perf_counter()
    run.run(args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    steps = run.n_steps - steps0
    ms = 1e3 * wall / max(steps, 1)
    recs = run.records
    sc_last = [r.Sc[-1] for r in recs]
    n_pts = [r.n_points[-1] for r in recs]
    line = {
        "metric": SWEEP_METRIC, "value": ms, "unit": "ms", "n_gpus": ws, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded flame-like profiles, synthetic transport)",
        "config": {"workload": split_workload(args, mech) + f"; FlameSolver loop: regrid every {args.regrid_interval} "
                               "steps, termination test every 10", "flames": len(grids),
                   "threads_per_point": width, "tuning": tuning(gm),
                   "rebuilds_in_timed_region": run.n_rebuilds - rebuilds0,
                   "points_at_end": int(sum(n_pts)), "points_per_flame_at_end": [int(n) for n in n_pts],
                   "consumption_speed_at_end": sc_last,
                   "terminated": [r.terminated for r in recs],
                   "heat_release_rms_variation": [r.rms_rel for r in recs],
                   "timing": "wall clock around the whole loop (host regrid and rebuilds included), after "
                             f"{args.warmup} untimed steps"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "note": "the loop is driven from the host API; the state stays on the device between regrids"},
        "gpu_launches": None,
        "clocks": clocks,
    }
    return line


def run_secondary(args) -> dict:
    """Each secondary workload at its own configuration, with W >= 3 warm-up
    steps and a few timed steps; every entry carries its own roofline,
    cpu_baseline, parity and clocks."""
    out = {}
    for name, over, steps, cpu_s in SECONDARY:
        a = argparse.Namespace(**vars(args))
        for k, v in over.items():
            setattr(a, k, v)
        a.steps = min(args.steps, steps)
        a.warmup = max(3, min(args.warmup, 3))
        a.cpu_seconds = min(args.cpu_seconds, cpu_s)
        a.threads = 0
        a.convection = over.get("convection", False)
        a.no_plain = False
        t0 = time.perf_counter()
        line = RUNNERS[a.workload](a)
        line["wall_s"] = round(time.perf_counter() - t0, 2)
        out[name] = line
    return out


def main():
    args = parse_args()
    if args.impl == "reference":
        ref = {"transport": run_reference_transport, "convection": run_reference_convection,
               "diffusion": run_reference_diffusion, "split": run_reference_split, "sweep": run_reference_split,
               "adjoint": run_reference_adjoint}
        return ref.get(args.workload, run_reference)(args)
    import torch
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl")
    RUNNERS.update({"qss": run_ours, "bdf": run_ours, "transport": run_ours_transport,
                    "convection": run_ours_convection, "diffusion": run_ours_diffusion, "split": run_ours_split,
                    "adjoint": run_ours_adjoint, "sweep": run_ours_sweep})
    try:
        line = RUNNERS[args.workload](args)
        if args.workload == "qss" and not args.no_secondary:
            line["secondary"] = run_secondary(args)
        if rank == 0:
            print(json.dumps(line))
    finally:
        if ws > 1:
            torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
