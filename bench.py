#!/usr/bin/env python
"""Benchmark: cell-updates/s of the explicit first-order FV step on one GB300.

Workload (default): single-phase Rusanov step on 2^24 cells, 64 seeded
piecewise-constant segments (rho/rho0 log-uniform in [0.9, 1.1], |u| <= 0.5 b0
in a uniform direction, A = R (I + 0.05 G)), CFL 0.5, frozen end cells, default
Barton2009. One "step" = one time step over all cells. Inputs are larger than
L2 (state 1.88 GB in FP64), so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's step (the
oracle, the same per-cell algorithm main.jl runs) on all host cores, each step
a bounded window of the same workload. Prints one JSON line (rank 0).
"""
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
sys.path.insert(0, ROOT)

LOCAL_RANK = int(os.environ.get("LOCAL_RANK", "0"))
RANK = int(os.environ.get("RANK", "0"))
WORLD = int(os.environ.get("WORLD_SIZE", "1"))
if WORLD > 1:  # one process per GPU: each rank sees only its own device
    os.environ["CUDA_VISIBLE_DEVICES"] = str(LOCAL_RANK)

import numpy as np  # noqa: E402

METRIC = "cell-updates/s"
BYTES_PER_CELL_UPDATE = {"single": 224, "multi": 480}  # state read + write per cell-update (14 or 30 values x 8 B x 2)
# floating-point operations of the formulation per cell-update (tests/flop_count.cpp: the product's
# FP64 physics run with an operation-counting scalar type; Rusanov single phase, HLL two-phase)
FLOPS_PER_CELL_UPDATE = {"single": 674, "multi": 15087}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel):
    """dram bytes per cell for `kernel` from the committed ncu summary (profiles/ncu_traffic.txt)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 2 and not line.startswith("#") and parts[0] == kernel:
                return float(parts[1])
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc, self.path = None, None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.25)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    if WORLD == 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")  # only timing scalars cross ranks; the problems are independent
    return dist


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(n_cells, seed=None):
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = h.Barton2009()
    seg_p = segment_states(eos, 64) if seed is None else segment_states(eos, 64, seed)
    seg_q = H.prim2cons(eos, seg_p)  # conservative segment states on the GPU
    return eos, seg_q, segment_fill


PRECISION_NOTE = {"fp64": "FP64 throughout",
                  "mixed": "FP32 fluxes and wave speeds, compensated hi/lo FP32 state, float-float cons2prim islands"}


def config_block(args):
    return {"workload": f"single-phase Rusanov FV step, {args.n_cells} cells, 64 seeded segments, CFL 0.5",
            "n_cells": args.n_cells, "model": "single-phase (Barton2009 default)", "flux": "rusanov",
            "bc": "frozen", "cfl": 0.5,
            "l2": "inputs larger than L2 (state %.2f GB)" % (args.n_cells * 14 * 8 / 1e9)}


def cpu_sample(Q0, target_s, nthreads):
    """Time the oracle (the reference's per-cell algorithm, literal face evaluation)
    on a window of the workload; returns (cell-updates/s, description)."""
    import oracle
    pb = oracle.problem(cfl=0.5)
    nx = Q0.shape[1]
    start = (nx * 37) // 64 - 2048
    W = np.ascontiguousarray(Q0[:, start:start + 4096])
    t0 = time.perf_counter()
    oracle.run(pb, W, max_steps=1, nthreads=nthreads, literal=True)
    per = (time.perf_counter() - t0) / W.shape[1]
    cells = int(min(nx, max(4096, 2 ** round(math.log2(max(4096, 0.5 / per))))))
    steps = max(1, int(target_s / (per * cells)))
    start = max(0, (nx * 37) // 64 - cells // 2)
    W = np.ascontiguousarray(Q0[:, start:start + cells])
    t0 = time.perf_counter()
    oracle.run(pb, W, max_steps=steps, nthreads=nthreads, literal=True)
    el = time.perf_counter() - t0
    return W.shape[1] * steps / el, f"{steps} steps of a {W.shape[1]}-cell window of the workload ({el:.1f} s)"


def run_reference(args):
    if RANK != 0:
        return 0
    import oracle
    oracle.build()
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = h.Barton2009()
    pb = oracle.problem(cfl=0.5)
    seg_q = oracle.prim2cons(pb, segment_states(eos, 64))
    nthreads = os.cpu_count()
    # window size so that one step of the window takes about 0.25 s on all host cores
    probe = segment_fill(seg_q, 4096)
    t0 = time.perf_counter()
    oracle.run(pb, probe, max_steps=1, nthreads=nthreads, literal=True)
    per = (time.perf_counter() - t0) / 4096
    cells = int(2 ** round(math.log2(max(4096, 0.25 / per))))
    full = args.n_cells
    start = (full * 37) // 64 - cells // 2
    idx = np.arange(start, start + cells)
    Q0 = np.ascontiguousarray(seg_q[(idx * 64) // full].T)
    Q, _, _, _ = oracle.run(pb, Q0, max_steps=args.warmup, nthreads=nthreads, literal=True)
    t0 = time.perf_counter()
    oracle.run(pb, Q, max_steps=args.steps, nthreads=nthreads, literal=True)
    el = time.perf_counter() - t0
    v = cells * args.steps / el
    sample = f"each step: a {cells}-cell window (around a segment boundary) of the {full}-cell workload"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(args), "precision": "FP64 (CPU restatement of the reference's step)",
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


KERNEL_NAMES = {("fp64", "cell"): "cell1_f64_kernel", ("fp64", "update"): "update1_f64_kernel",
                ("mixed", "cell"): "step1_mixed_kernel"}


def density(Q, rho0=8.93):
    """rho_true = sqrt(det(rho A)/rho0) of SoA single-phase states (cons2prim's density)."""
    m = Q[5:14]
    det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
           + m[6] * (m[1] * m[5] - m[4] * m[2]))
    return np.sqrt(det / rho0)


def device_run(h, eos, Q0, prec, K, W, dist, clocks=True):
    """W untimed steps, then K steps timed with CUDA events (per-kernel events on)."""
    s = h.Solver(eos, Q0.shape[1], precision=prec, cfl=0.5)
    s.upload(Q0)
    s.step(max_steps=W)
    s.set_profiling(True)
    if dist:
        dist.barrier()
    clk = ClockSampler() if clocks else None
    if clk:
        clk.start()
    s.step(max_steps=K)
    ck = clk.stop() if clk else None
    tm = s.timing()
    s.set_profiling(False)
    Q = s.download()
    s.close()
    return tm, ck, Q


def roofline(tm, prec, n, peak, peak_kind):
    kern = "cell" if tm["ms_cell"] >= tm["ms_update"] else "update"
    ms_k = tm["ms_" + kern] / max(1, tm["n_" + kern])
    alg = BYTES_PER_CELL_UPDATE["single"] * n
    achieved = alg / (ms_k / 1e3) / 1e9
    name = KERNEL_NAMES[(prec, kern)]
    tr = ncu_traffic(name)
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": (tr * n if tr is not None else None),
            "algorithmic_bytes_per_launch": alg, "ms_per_launch": ms_k}


def run_ours(args):
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._lib import PinnedArray
    dist = dist_setup()
    h.build_library()
    eos, seg_q, segment_fill = workload(args.n_cells)
    n, K, W = args.n_cells, args.steps, args.warmup
    Q0 = segment_fill(seg_q, n)
    state_bytes = Q0.nbytes
    prec = args.precision
    peak, peak_kind = measured_peaks()
    # ---- device-resident throughput of the headline precision -------------
    tm, clocks, Qh = device_run(h, eos, Q0, prec, K, W, dist)
    ms_total = dist_max(dist, tm["ms_total"])
    value = WORLD * n * K / (ms_total / 1e3)
    # ---- end to end through the C ABI from pinned host memory -------------
    s = h.Solver(eos, n, precision=prec, cfl=0.5)
    pin_in, pin_out = PinnedArray(Q0.shape), PinnedArray(Q0.shape)
    pin_in.array[...] = Q0
    s.upload(pin_in.array)
    s.step(max_steps=W)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    s.upload(pin_in.array)
    t1 = time.perf_counter()
    # the K steps with the time after each one read back (the reference logs Step / t / dt
    # every step, main.jl:229-237), then the final state
    s.step_times(max_steps=K)
    t2 = time.perf_counter()
    s.download(pin_out.array)
    t3 = time.perf_counter()
    e2e_s = dist_max(dist, t3 - t0)
    e2e = WORLD * n * K / e2e_s
    e2e_parts = {"upload_ms": 1e3 * (t1 - t0), "steps_ms": 1e3 * (t2 - t1), "download_ms": 1e3 * (t3 - t2)}
    s.close()
    pin_in.close()
    pin_out.close()
    # ---- the plain FP64 step on the same workload, and the accuracy -------
    fp64 = None
    if prec == "mixed" and not args.no_fp64:
        tm64, _, Q64 = device_run(h, eos, Q0, "fp64", K, W, dist, clocks=False)
        ms64 = dist_max(dist, tm64["ms_total"])
        a, b = density(Qh), density(Q64)
        fp64 = {"value": WORLD * n * K / (ms64 / 1e3), "ms_per_step": ms64 / K,
                "mixed_over_fp64": (WORLD * n * K / (ms_total / 1e3)) / (WORLD * n * K / (ms64 / 1e3)),
                "roofline": roofline(tm64, "fp64", n, peak, peak_kind),
                "density_error_vs_fp64": {"l1": float(np.sum(np.abs(a - b)) / np.sum(np.abs(b))),
                                          "linf": float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
                                          "after_steps": W + K}}
    if RANK != 0:
        return 0
    rf = roofline(tm, prec, n, peak, peak_kind)
    rf["step_hbm_frac"] = (BYTES_PER_CELL_UPDATE["single"] * n / (ms_total / K / 1e3) / 1e9) / peak
    rf["formulation_flops_per_cell_update"] = FLOPS_PER_CELL_UPDATE["single"]
    rf["formulation_tflops"] = FLOPS_PER_CELL_UPDATE["single"] * n / (ms_total / K / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": WORLD, "steps": K, "warmup": W,
        "ms_per_step": ms_total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == "fp64" else "f32", "data": "synthetic",
        "config": config_block(args), "precision": PRECISION_NOTE[prec],
        "clocks": clocks,
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": state_bytes / K,
                "d2h_bytes_per_step": state_bytes / K + 8, **e2e_parts},
        "gpu_launches": tm["n_cell"] + tm["n_update"],
        "roofline": rf,
    }
    if fp64:
        line["fp64"] = fp64
    if not args.no_cpu:
        v, sample = cpu_sample(Q0, args.cpu_seconds, os.cpu_count())
        line["cpu_baseline"] = {"value": v, "unit": METRIC, "cores": os.cpu_count(), "kind": "port", "sample": sample}
    if WORLD == 1 and not args.no_workloads:
        line["measured_rates"] = measure_rates()
        line["workloads"] = workload_summaries(args)
    print(json.dumps(line))
    return 0


def emit(line, args):
    """Print a workload's line (standalone run), or hand it back to the default run."""
    if getattr(args, "nested", False):
        return line
    print(json.dumps(line))
    return 0


def nested_args(args, workload):
    """The arguments of one of the other workloads at its own default size and steps,
    for its summary inside the default line."""
    a = argparse.Namespace(**vars(args))
    a.nested = True
    a.workload = workload
    a.steps = DEFAULT_STEPS[workload]
    a.n_cells = DEFAULT_CELLS[workload]
    a.warmup = max(3, args.warmup if workload != "adjoint" else 1)
    a.flux = "hll"
    return a


def workload_summaries(args):
    """Compact results of the batch (4096 problems x 500 steps), two-phase (2^22 cells x
    300 HLL steps) and adjoint (65,536 cells x 1000 steps) workloads."""
    out = {}
    b = run_batch(nested_args(args, "batch"))
    out["batch"] = {"workload": b["config"]["workload"], "value": b["value"], "unit": b["unit"],
                    "ms_per_step": b["ms_per_step"], "hbm_frac": b["roofline"]["frac"],
                    "fp64_value": b["fp64_batch"]["value"], "mixed_over_fp64": b["value"] / b["fp64_batch"]["value"],
                    "density_l1_max_vs_fp64": b["density_error_vs_fp64_per_problem"]["l1_max"],
                    "clocks": b["clocks"]}
    m = run_mph(nested_args(args, "mph"))
    out["mph"] = {"workload": m["config"]["workload"], "value": m["value"], "unit": m["unit"],
                  "ms_per_step": m["ms_per_step"], "hbm_frac": m["roofline"]["frac"], "fp64_value": m["fp64"]["value"],
                  "mixed_over_fp64": m["fp64"]["mixed_over_fp64"],
                  "density_l1_vs_fp64_per_phase": [e["l1"] for e in m["density_error_vs_fp64_per_phase"]],
                  "clocks": m["clocks"]}
    a = run_adjoint(nested_args(args, "adjoint"))
    out["adjoint"] = {"workload": a["config"]["workload"], "adjoint_over_forward": a["adjoint_over_forward"],
                      "adjoint_over_forward_dense_seed": a["dense_seed"]["adjoint_over_forward"],
                      "ms_forward": a["ms"]["forward"], "ms_reverse": a["ms"]["recompute"] + a["ms"]["adjoint"],
                      "fd_max_rel": a["fd_check"]["max_rel"], "clocks": a["clocks"]}
    return out


def measure_rates(reps=3, nbytes=1 << 30, layout_cells=1 << 24):
    """FP64 / FP32 / packed-f32x2 FMA throughput and the host link's copy rates of this GPU
    (hyp_measure_peaks): the denominators the driver's copy and GEMM peaks do not give;
    and the step's memory traffic without the physics in the row-major and the
    tile-major state layout (hyp_measure_layouts)."""
    import ctypes
    import hyperelasticsolver_gb300 as h
    L = h._lib.load()
    out = np.zeros(6)
    h._lib.check(L.hyp_measure_peaks(int(reps), int(nbytes), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                 what="hyp_measure_peaks")
    lay = np.zeros(2)
    h._lib.check(L.hyp_measure_layouts(int(reps), int(layout_cells), lay.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                 what="hyp_measure_layouts")
    return {"fp64_fma_tflops": out[0], "fp32_fma_tflops": out[1], "fp32x2_fma_tflops": out[2],
            "h2d_gbs": out[3], "d2h_gbs": out[4], "bidirectional_gbs_each_way": out[5],
            "copy_bytes": nbytes, "step_traffic_rowmajor_gbs": lay[0], "step_traffic_tilemajor_gbs": lay[1],
            "layout_cells": layout_cells,
            "note": "best of %d; FMA: 8 independent chains per thread, 8 x 256-thread blocks per SM; "
                    "step traffic: 256 B per cell, 32 FP32 rows read and written, no physics" % reps}


def run_peaks(args):
    import hyperelasticsolver_gb300 as h
    h.build_library()
    clk = ClockSampler()
    clk.start()
    r = measure_rates()
    clocks = clk.stop()
    line = {"metric": "measured rates", "value": r["fp64_fma_tflops"], "unit": "FP64 TFLOP/s", "n_gpus": 1,
            "steps": 1, "warmup": 0, "higher_is_better": True, "data": "synthetic", "rates": r, "clocks": clocks,
            "config": {"workload": "FMA chains and page-locked host copies"}}
    print(json.dumps(line))
    return 0


def run_batch(args):
    """Batched workload: 4096 independent single-phase Riemann problems, cell counts
    log-uniform in [256, 65536] (seeded), 500 steps each with per-problem CFL dt, mixed
    precision with the autotuned kernel variant, the whole run one CUDA-graph launch;
    per-problem L1 density error against the FP64 batch."""
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    from hyperelasticsolver_gb300._cases import batch_sizes, batch_prims, batch_fill
    h.build_library()
    eos = h.Barton2009()
    sizes = batch_sizes(args.problems)
    Pl, Pr = batch_prims(eos, len(sizes))
    Q0 = batch_fill(H.prim2cons(eos, Pl), H.prim2cons(eos, Pr), sizes)
    K, W = args.steps, args.warmup
    total = int(sizes.sum())
    with h.Batch(eos, sizes, precision="mixed") as b:
        b.upload(Q0)
        chosen, tune_ms = b.autotune(trial_steps=5)
        b.upload(Q0)
        b.step(W)
        clk = ClockSampler()
        clk.start()
        b.step(K)
        clocks = clk.stop()
        ms = b.last_ms()
        Qm = b.download()
    with h.Batch(eos, sizes, precision="fp64") as b:
        b.upload(Q0)
        b.step(W)
        b.step(K)
        ms64 = b.last_ms()
        Q64 = b.download()
    a, r = density(Qm), density(Q64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    l1 = np.array([np.sum(np.abs(a[o:e] - r[o:e])) / np.sum(np.abs(r[o:e])) for o, e in zip(offs[:-1], offs[1:])])
    linf = np.array([np.max(np.abs(a[o:e] - r[o:e])) / np.max(np.abs(r[o:e])) for o, e in zip(offs[:-1], offs[1:])])
    peak, peak_kind = measured_peaks()
    v = total * K / (ms / 1e3)
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": 1, "steps": K, "warmup": W,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"batched: {len(sizes)} single-phase Riemann problems, cell counts log-uniform in "
                                   f"[256, 65536] (total {total}), per-problem CFL dt, {K} steps in one CUDA graph",
                       "l2": "inputs larger than L2"},
            "precision": PRECISION_NOTE["mixed"], "clocks": clocks,
            "autotune": {"chosen_variant": chosen, "variants": ["256x4 persistent", "256x3 persistent", "256x4 block per tile"],
                         "ms_per_step": [float(x) for x in tune_ms]},
            "roofline": {"bound": "hbm", "achieved": BYTES_PER_CELL_UPDATE["single"] * total / (ms / K / 1e3) / 1e9,
                         "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                         "frac": BYTES_PER_CELL_UPDATE["single"] * total / (ms / K / 1e3) / 1e9 / peak},
            "fp64_batch": {"value": total * K / (ms64 / 1e3), "ms_per_step": ms64 / K},
            "density_error_vs_fp64_per_problem": {"l1_max": float(l1.max()), "l1_median": float(np.median(l1)),
                                                  "linf_max": float(linf.max())}}
    return emit(line, args)


def phase_densities(Q, rho0=8.93):
    """rho_true of both phases of SoA two-phase states (30, n) (HyperelasticityMPh.jl:113-114)."""
    out = []
    for p in range(2):
        m = Q[15 * p + 6:15 * p + 15] / Q[15 * p]
        det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
               + m[6] * (m[1] * m[5] - m[4] * m[2]))
        out.append(np.sqrt(det / rho0))
    return out


def run_mph(args):
    """Two-phase workload: 2^22 cells, alpha1 a smoothed step from 1 - 1e-6 to 1e-6 over
    8 cells at x = 0.5, both phases carrying the single-phase Riemann states, phase 2 with
    the shear modulus scaled by 0.1 (c0 held), path-conservative HLL, frozen ends; the
    mixed-precision step timed, then the FP64 step on the same input for the ratio and
    each phase's density error."""
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    h.build_library()
    eos = (h.Barton2009(), h.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    n, K, W = args.n_cells, args.steps, args.warmup
    Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos, mph_interface_prims(eos[0], n)).T)
    res = {}
    clocks = None
    for prec in ("mixed", "fp64"):
        with h.Solver(eos, n, model="multi", flux=args.flux, precision=prec, cfl=0.5) as s:
            s.upload(Q0)
            s.step(max_steps=W)
            s.set_profiling(True)
            clk = ClockSampler()
            clk.start()
            s.step(max_steps=K)
            c = clk.stop()
            clocks = clocks or c
            res[prec] = (s.timing(), s.download())
    tm, Qm = res["mixed"]
    tm64, Q64 = res["fp64"]
    errs = []
    for a, b in zip(phase_densities(Qm), phase_densities(Q64)):
        errs.append({"l1": float(np.sum(np.abs(a - b)) / np.sum(np.abs(b))),
                     "linf": float(np.max(np.abs(a - b)) / np.max(np.abs(b)))})
    peak, peak_kind = measured_peaks()
    ms = tm["ms_total"] / K
    ach = BYTES_PER_CELL_UPDATE["multi"] * n / (ms / 1e3) / 1e9
    line = {"metric": METRIC, "value": n * K / (tm["ms_total"] / 1e3), "unit": METRIC, "n_gpus": 1, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"two-phase {args.flux.upper()} path-conservative step, {n} cells, alpha1 1-1e-6 -> 1e-6 over "
                                   "8 cells, phase 2 shear modulus x0.1", "l2": "inputs larger than L2"},
            "precision": "FP32 two-phase physics and fluxes, compensated hi/lo FP32 state, float-float cons2prim "
                         "islands per phase", "clocks": clocks,
            # the mixed step runs its faces and update in one kernel, after the cell kernel
            "kernels_ms_per_step": {"cell": tm["ms_cell"] / max(1, tm["n_cell"]),
                                    "face+update": tm["ms_update"] / max(1, tm["n_update"])},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "peak_source": peak_kind,
                         "frac": ach / peak,
                         "formulation_flops_per_cell_update": FLOPS_PER_CELL_UPDATE["multi"],
                         "formulation_tflops": FLOPS_PER_CELL_UPDATE["multi"] * n / (ms / 1e3) / 1e12,
                         "note": "the face kernel (HLL: 18 evaluations of B per face, LxF: 6; the update "
                                 "fused in) is bound by FP32 issue, not HBM"},
            "fp64": {"value": n * K / (tm64["ms_total"] / 1e3), "ms_per_step": tm64["ms_total"] / K,
                     "kernels_ms_per_step": {"cell+face": tm64["ms_cell"] / max(1, tm64["n_cell"]),
                                             "update": tm64["ms_update"] / max(1, tm64["n_update"])},
                     "mixed_over_fp64": tm64["ms_total"] / tm["ms_total"]},
            "density_error_vs_fp64_per_phase": errs}
    return emit(line, args)


def run_adjoint(args):
    """Adjoint workload: 1000 FP64 Rusanov steps of a single-phase two-state problem on
    65536 cells, gradient of L = 1/2 |rho_T - target|^2 with respect to the 13 left-state
    parameters and the moduli (b0sq, k0), checkpoints every 50 steps with recompute in
    between; target = the forward run at parameters perturbed by a seeded 2% Gaussian.
    Reports the reverse pass (recompute + adjoint steps) against the plain forward run,
    and the central-difference check (step 1e-6 relative) of all 15 components."""
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300.adjoint import RiemannMisfit, PARAM_NAMES
    from hyperelasticsolver_gb300._cases import adjoint_states, adjoint_target_theta
    h.build_library()
    eos = h.Barton2009()
    n, K = args.n_cells, args.steps
    pl, pr = adjoint_states(eos)
    pb = RiemannMisfit(eos, pl, pr, n, K, ckpt_every=args.ckpt_every)
    th0 = pb.theta0()
    target = pb.final_density(adjoint_target_theta(th0))
    e, _, _, Q0 = pb.setup(th0)
    with h.Solver(e, n, flux="rusanov", precision="fp64") as s:  # the plain forward run, for the ratio
        for _ in range(max(1, args.warmup)):
            s.upload(Q0)
            s.step(max_steps=K)
        s.upload(Q0)
        clk = ClockSampler()
        clk.start()
        s.step(max_steps=K)
        ms_fwd = s.timing()["ms_total"]
        for _ in range(max(1, args.warmup) - 1):
            pb.loss_and_grad(th0, target)
        L, g, tm = pb.loss_and_grad(th0, target)
        # the same reverse pass seeded with a dense random dL/dQ: no cell's adjoint vanishes
        s.upload(Q0)
        s.record(K, args.ckpt_every)
        s.adjoint(np.random.default_rng(7).standard_normal((14, n)))
        tm_dense = s.adjoint_timing()
        clocks = clk.stop()
    fd = pb.fd_grad(th0, target)
    scale = np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    rel = np.abs(g - fd) / scale
    ms_rev = tm["ms_recompute"] + tm["ms_adjoint"]
    line = {"metric": "adjoint cell-updates/s", "value": n * K / (ms_rev / 1e3), "unit": "cell-updates/s",
            "n_gpus": 1, "steps": K, "warmup": args.warmup, "ms_per_step": ms_rev / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"adjoint of {K} FP64 Rusanov steps, {n} cells, gradient w.r.t. 13 left-state "
                                   f"parameters + (b0sq, k0), checkpoint every {args.ckpt_every} steps",
                       "l2": "state (7.3 MB) resident in L2"},
            "clocks": clocks,
            "adjoint_over_forward": ms_rev / ms_fwd,
            "dense_seed": {"adjoint_over_forward": (tm_dense["ms_recompute"] + tm_dense["ms_adjoint"]) / ms_fwd,
                           "ms_adjoint": tm_dense["ms_adjoint"],
                           "note": "dL/dQ_final standard normal in every cell, so no cell's VJP is skipped"},
            "adjoint_steps_over_forward": tm["ms_adjoint"] / ms_fwd,
            "ms": {"forward": ms_fwd, "record": tm["ms_record"], "recompute": tm["ms_recompute"],
                   "adjoint": tm["ms_adjoint"]},
            "loss": L,
            "fd_check": {"max_rel": float(rel.max()), "per_param": {PARAM_NAMES[k]: float(rel[k]) for k in range(15)},
                         "step_rel": 1e-6}}
    return emit(line, args)


def run_evaluators(args):
    """Function-level API workload: each evaluator that a per-cell function of the
    reference maps to (Strains, EquationsOfState, Hyperelasticity, HyperelasticityMPh,
    NumFluxes; Barton2009 and Hank2016), called on n seeded cells with host arrays in and
    out, so the timed call holds the device allocation, both copies and the kernel.
    Per evaluator: cells/s of the whole call (median of --steps calls after --warmup
    untimed ones)."""
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300 import Strains as St, EquationsOfState as E, Hyperelasticity as H
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM, NumFluxes as NF
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    h.build_library()
    n = args.n_cells
    rng = np.random.default_rng(20261204)
    eos, hank = h.Barton2009(), E.Hank2016()
    eos2 = (h.Barton2009(), h.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    A = np.tile(np.eye(3).reshape(1, 9, order="F"), (n, 1)) + 0.03 * rng.standard_normal((n, 9))
    S = rng.uniform(0.0, 1e-3, n)
    P = np.empty((n, 14))
    P[:, 0] = 8.93 * rng.uniform(0.95, 1.05, n)
    P[:, 1:4] = rng.uniform(-0.5, 0.5, (n, 3))
    P[:, 4] = S
    P[:, 5:] = A
    Q = H.prim2cons(eos, P)
    P2 = mph_interface_prims(eos2[0], n)
    Q2 = HM.prim2cons_mph(eos2, P2)
    G = St.finger(A)
    inv = St.invariants(G)
    e_int = E.energy(eos, S, G)
    den = 2.7 * rng.uniform(0.95, 1.05, n)
    pres = rng.uniform(0.0, 1e9, n)
    lam = np.max(np.abs(H.get_eigvals(eos, Q)), axis=1)
    calls = {
        "Strains.finger": lambda: St.finger(A),
        "Strains.invariants": lambda: St.invariants(G),
        "EquationsOfState.energy": lambda: E.energy(eos, S, G),
        "EquationsOfState.entropy": lambda: E.entropy(eos, e_int, G),
        "EquationsOfState.stress": lambda: E.stress(eos, S, A),
        "EquationsOfState.acoustic": lambda: E.acoustic(eos, S, A),
        "Hyperelasticity.prim2cons": lambda: H.prim2cons(eos, P),
        "Hyperelasticity.cons2prim": lambda: H.cons2prim(eos, Q),
        "Hyperelasticity.flux": lambda: H.flux(eos, Q),
        "Hyperelasticity.get_eigvals": lambda: H.get_eigvals(eos, Q),
        "NumFluxes.lxf (one phase)": lambda: NF.lxf(eos, Q[:-1], Q[1:], lam[1:]),
        "HyperelasticityMPh.prim2cons_mph": lambda: HM.prim2cons_mph(eos2, P2),
        "HyperelasticityMPh.cons2prim_mph": lambda: HM.cons2prim_mph(eos2, Q2),
        "HyperelasticityMPh.flux_mph": lambda: HM.flux_mph(eos2, Q2),
        "HyperelasticityMPh.get_eigvals": lambda: HM.get_eigvals(eos2, Q2),
        "HyperelasticityMPh.noncons_flux": lambda: HM.noncons_flux(eos2, Q2),
        "NumFluxes.hll (two phases)": lambda: NF.hll(eos2, Q2[:-1], Q2[1:]),
        "NumFluxes.lxf (two phases)": lambda: NF.lxf(eos2, Q2[:-1], Q2[1:], 10.0),
        "Hank2016 energy": lambda: E.energy(hank, den, pres, G),
        "Hank2016 pressure": lambda: E.pressure(hank, den, e_int, inv),
        "Hank2016 stress": lambda: E.stress(hank, den, pres, A),
    }
    rates, total_s = {}, 0.0
    for name, f in calls.items():
        for _ in range(args.warmup):
            f()
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        t = sorted(ts)[len(ts) // 2]
        total_s += t
        rates[name] = n / t
    unit = "cell evaluations/s"
    line = {"metric": "function-level evaluations/s (host arrays in and out)", "value": len(calls) * n / total_s,
            "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / len(calls),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"every function-level evaluator on {n} seeded cells, one call each, host arrays "
                                   "(allocation, copies and kernel timed)", "n_cells": n},
            "per_evaluator": rates}
    print(json.dumps(line))
    return 0


DEFAULT_STEPS = {"single": 200, "batch": 500, "mph": 300, "adjoint": 1000, "evaluators": 3, "peaks": 1}
DEFAULT_CELLS = {"single": 1 << 24, "batch": None, "mph": 1 << 22, "adjoint": 65536, "evaluators": 1 << 20,
                 "peaks": None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 single, 500 batch, 300 mph, 1000 adjoint)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n-cells", type=int, default=None,
                    help="cells (default: 2^24 single, 2^22 mph, 65536 adjoint)")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-workloads", action="store_true",
                    help="single workload: skip the batch / two-phase / adjoint summaries in its line")
    ap.add_argument("--workload", choices=["single", "batch", "mph", "adjoint", "evaluators", "peaks"], default="single",
                    help="single: the headline single-phase step; batch: 4096 ragged problems; mph: two-phase HLL; "
                         "adjoint: gradient of a 1000-step run; evaluators: the function-level API")
    ap.add_argument("--flux", choices=["hll", "lxf"], default="hll", help="two-phase workload's face flux")
    ap.add_argument("--ckpt-every", type=int, default=50)
    ap.add_argument("--problems", type=int, default=4096)
    args = ap.parse_args()
    if args.warmup < 1:
        ap.error("--warmup must be >= 1")
    wl = "single" if args.impl == "reference" else args.workload
    if args.steps is None:
        args.steps = DEFAULT_STEPS[wl]
    if args.n_cells is None:
        args.n_cells = DEFAULT_CELLS[wl]
    if args.impl == "reference":
        return run_reference(args)
    runner = {"batch": run_batch, "adjoint": run_adjoint, "mph": run_mph,
              "evaluators": run_evaluators, "peaks": run_peaks}.get(args.workload, run_ours)
    return runner(args)


if __name__ == "__main__":
    sys.exit(main())
