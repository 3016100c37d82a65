#!/usr/bin/env python
"""Benchmark of HyPar's explicit WENO5 RHS + Runge-Kutta step on GB300.

Default workload (the configuration the headline metric is quoted on): 2-D
Euler isentropic vortex, 1024 x 1024 periodic grid on [0,10)^2, b = 5,
characteristic WENO5 (Jiang-Shu) + Roe, SSPRK3, dt at CFL 0.5, FP64.  A
"step" is one SSPRK3 step of that grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload vortex|tgv|sod|rtb|rtb64|dns|dns64cr|ensemble|adjoint|
                              convergence|parity|kernel-vjp|kernel-jvp|kernel-step]

The default line also carries the metric's other two parts, measured after the
timed region on reduced step counts: an "ensemble" block (batched vs one at a
time) and an "adjoint" block (gradient and backward cost over the forward solve,
central-difference and dot-product checks).  --workload parity prints where the
per-right-hand-side distance from the oracle comes from; kernel-* only launch one
entry point for profilers.

--impl ours       the fused CUDA path through libgbhypar's C ABI (value: device
                  time of the resident solution; e2e: host buffers copied in and
                  out every step through gb_solver_set_state/step/get_state).
--impl reference  the reference algorithm on the host cores (the CPU oracle,
                  a restatement of the reference's C; the reference's own build
                  needs its source tree, which only the build container has).
N > 1 runs N independent replicas (one per GPU, weak scaling); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 cell-updates/s & HBM%; ensemble vs serial speedup; adjoint/forward cost"
UNIT = "cell-component updates/s"

# FP64 work of one whole step per grid cell, summed over every kernel of the step:
# floating-point operations (DFMA = 2, DMUL / DADD = 1) and FP64-pipe thread
# instructions, from ncu's instruction counters (smsp__sass_thread_inst_executed_op_
# {dfma,dmul,dadd}_pred_on.sum, sm__thread_inst_executed_pipe_fp64_pred_on.sum) over
# the launches of one step, captured on the grid given (2-D / 3-D: a smaller grid
# with the launch shapes the autotuner picks at full size, whose per-cell work is
# that of the full grid to within the segment-boundary share).
FP64_PER_CELL_STEP = {
    "vortex": {"tile": {"flops": 8454.6, "instr": 5494.4, "captured": "512^2, tiles of 128 interfaces"},
               "walker": {"flops": 8585.4, "instr": 5575.5, "captured": "512^2, segments 54/27"}},
    "sod": {"lanes": {"flops": 3654.7, "instr": 2455.2, "captured": "1024 (the full grid), lane groups of 16"}},
    "tgv": {"walker": {"flops": 18445.5, "instr": 12291.2,
                       "captured": "128^3, segments 48/32/32 (the earlier 256^3 shape)"},
            "tile": {"flops": 16107.9, "instr": 10815.0, "captured": "128^3, tiles of 64 (the 256^3 shape)"}},
    "rtb": {"walker": {"flops": 16583.3, "instr": 11627.6, "captured": "128^3, segments 32/32/32 (the 201^3 shape)"}},
    "rtb64": {"walker": {"flops": 25265.3, "instr": 17712.2, "captured": "64^3 (the full grid), segments 7/7/7"}},
    "dns": {"walker": {"flops": 20731.2, "instr": 14874.6, "captured": "128^3, segments 48/48/48 (the 256^3 shape)"}},
    "dns64cr": {"walker": {"flops": 34332.9, "instr": 23470.2, "captured": "64^3 (the full grid), segments 5/5/4"}},
}
# DRAM bytes (read + write) per cell of one launch (x launch / y launch with the RK
# update), per kernel form: the segment walker from a 2048^2 capture of the
# centre-relative kernels (traffic proportional to cells at these sizes), the tile form
# from a capture of the default 1024^2 run (the 34 MB state partly stays in L2 there).
DRAM_BYTES_PER_CELL = {"vortex": {("hyp_x", "walker"): 57.32, ("hyp_y", "walker"): 153.39,
                                  ("hyp_x", "tile"): 32.35, ("hyp_y", "tile"): 110.18}}
TRAFFIC_SOURCE = {"walker": "a 2048^2 capture of the segment-walker form, scaled by cells",
                  "tile": "a 1024^2 capture of the tile form"}


# The reference's published GPU numbers for the same decks (cell-component updates/s):
# RisingThermalBubble_Config1_CUDA/out.log:53-150, 64^3, RK4: 0.021 s/step on one V100;
# DNS_IsotropicTurbulenceDecay_CUDA/out.log:53-84, 256^3, SSPRK3: 82.42 s / 1000 steps on
# 64 V100s (4x4x4 ranks), the whole job; DNS_IsotropicTurbulenceDecay/output.log, 64^3
# CRWENO5, RK4: 1495.8 s / 200 steps on 4 CPU ranks.
PUBLISHED = {
    "rtb64": (64 ** 3 * 5 / 0.021, "1x V100 (IBM Power9), RisingThermalBubble_Config1_CUDA/out.log"),
    "dns": (256 ** 3 * 5 * 1000 / 82.42, "64x V100 aggregate (16 nodes x 4), DNS_IsotropicTurbulenceDecay_CUDA/out.log"),
    "dns64cr": (64 ** 3 * 5 * 200 / 1495.8, "CPU, 4 MPI ranks (2x2x1), DNS_IsotropicTurbulenceDecay/output.log"),
}


def workload(name: str, size: int = 0):
    from hypar_gb300 import cases as C
    if name == "vortex":
        n = size or 1024
        case = C.vortex(n, n_iter=200)
        desc = (f"Euler2D isentropic vortex {n}x{n} periodic [0,10)^2, b=5, char-WENO5(JS)+Roe, "
                "SSPRK3, CFL 0.5")
    elif name == "tgv":
        n = size or 256
        case = C.tgv(n, n_iter=100)
        desc = (f"NavierStokes3D Taylor-Green vortex {n}^3 periodic [0,2pi)^3, Mach 0.1, Re 1600, Pr 0.72, "
                "comp-WENO5(JS)+Roe + 4th-order viscous, RK4, dt 2e-3")
    elif name == "rtb":
        n = size or 201
        case = C.rising_thermal_bubble(n, n_iter=100)
        desc = (f"NavierStokes3D rising thermal bubble {n}^3 on [0,1000 m]^3, gravity 9.8 along y (HB 2, "
                "well-balanced), slip walls, comp-WENO5(YC)+Rusanov, SSPRK3, dt 0.01")
    elif name == "rtb64":
        n = size or 64
        case = C.rising_thermal_bubble(n, n_iter=100, dt=0.025, scheme="44")
        desc = (f"NavierStokes3D rising thermal bubble {n}^3 (the reference's RisingThermalBubble_Config1_CUDA "
                "deck), gravity 9.8 along y (HB 2), slip walls, comp-WENO5(YC)+Rusanov, RK4, dt 0.025")
    elif name == "dns":
        n = size or 256
        case = C.isotropic_turbulence(n, n_iter=100)
        desc = (f"NavierStokes3D decaying isotropic turbulence {n}^3 periodic [0,2pi)^3 (the reference's "
                "DNS_IsotropicTurbulenceDecay_CUDA deck: kp 4, u_rms = Minf 0.3, Re 333.3), "
                "comp-WENO5(mapped)+Roe + 4th-order viscous, SSPRK3, dt 0.005")
    elif name == "dns64cr":
        n = size or 64
        case = C.isotropic_turbulence(n, n_iter=200, dt=0.025, scheme="44")
        case.hyp_scheme = "crweno5"
        desc = (f"NavierStokes3D decaying isotropic turbulence {n}^3 periodic [0,2pi)^3 (the reference's "
                "DNS_IsotropicTurbulenceDecay deck: kp 4, u_rms = Minf 0.3, Re 333.3), "
                "comp-CRWENO5(mapped)+Roe + 4th-order viscous, RK4, dt 0.025")
    elif name == "sod":
        n = size or 1024
        case = C.sod(n, n_iter=1000)
        desc = f"Euler1D Sod shock tube {n} cells, comp-WENO5(JS)+Roe, RK4, dt 1e-4, extrapolate BCs"
    else:
        raise SystemExit(f"unknown workload {name}")
    return case, desc


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def stage_bytes(cfg, s) -> float:
    """Algorithmic HBM bytes per cell of the last-direction kernel of stage s
    (stencil input, accumulated hyperbolic term, viscous term, RK arrays)."""
    nv, ns = cfg.nvars, cfg.rk_nstages
    reads = 1 + (1 if cfg.ndims > 1 else 0)
    writes = 1
    need_u = s == 0
    for t in range(s + 1, ns):
        a = cfg.rk_A[4 * t + s]
        if a != 0.0:
            writes += 1
            touched = any(cfg.rk_A[4 * t + i] != 0.0 for i in range(s))
            reads += 1 if touched else 0
            need_u = need_u or not touched
    if s > 0:
        reads += 1 + (1 if need_u else 0)
    return 8.0 * nv * (reads + writes)


def common_config(case, desc, args, ws) -> dict:
    """The config object both arms print (the same keys and values for the same
    workload, so that the two lines can be matched)."""
    import numpy as np
    return {"workload": desc, "cells": int(np.prod(case.size)), "nvars": case.nvars, "dt": case.dt,
            "steps": args.steps, "parallelism": f"replicas x{ws}" if ws > 1 else "one device",
            "l2": ("GPU arm: a 256 MB buffer written between timed steps (L2 flush); CPU arm: state "
                   "arrays larger than the host caches at the full sizes")}


def run_ours(args, case, desc, ws, rank, local):
    import ctypes
    import numpy as np
    import torch
    from hypar_gb300 import _lib
    from hypar_gb300 import replicas as R
    from hypar_gb300.solver import Solver

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp(prefix="gbh_bench_")
    case.write(tmp)
    s = Solver.from_dir(tmp, device=local)
    stream = torch.cuda.Stream()  # a real stream: handle 0 would mean "the solver's own"
    torch.cuda.set_stream(stream)
    s.set_stream(stream.cuda_stream)
    if args.launch:
        # a fixed launch shape per direction (profiling: the autotuner's choice under a
        # profiler's serialised replays can differ from its choice in a plain run)
        for d, item in enumerate(args.launch.split(",")):
            sg, _, bl = item.partition(":")
            s.set_launch(d, int(sg), int(bl or 0))
        tuned = [s.get_launch(d) for d in range(case.ndims)]
    else:
        tuned = s.autotune(2)  # launch shape per direction (state restored), outside the timed region
    cells = int(np.prod(case.size))
    nv = case.nvars
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    for _ in range(args.warmup):
        s.step(1)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")  # ncu --nvtx --nvtx-include timed/ selects these launches
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            s.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1e3
    # per-kernel-class launch times from a second, untimed pass with the launch
    # profiler on (its events around every launch group add latency that the
    # timed steps above do not carry)
    s.profile(True)
    for k in range(args.steps):
        flush.fill_(float(k))
        s.step(1)
    torch.cuda.synchronize()
    prof = s.profile_read()
    s.profile(False)
    t_dev = R.max_over_ranks(t_dev, dist, "cuda")
    finite = s.check_finite()

    # e2e: the user call with host buffers, copies in and out every step
    host = torch.from_numpy(s.get_state()).pin_memory()
    hp = host.data_ptr()
    L = _lib.lib()
    torch.cuda.synchronize()
    n_e2e = max(1, min(args.steps, 10))
    te = time.perf_counter()
    for _ in range(n_e2e):
        _lib.check(L.gb_solver_set_state(s._h, hp, _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
        _lib.check(L.gb_solver_step(s._h, 1))
        _lib.check(L.gb_solver_get_state(s._h, hp, _lib.LAYOUT_INTERIOR, _lib.MEM_HOST))
    t_e2e = (time.perf_counter() - te) / n_e2e
    t_e2e = R.max_over_ranks(t_e2e, dist, "cuda")

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None

    pk = ctypes.c_double()
    _lib.check(L.gb_probe_fp64_peak(ctypes.byref(pk)))
    fp64_peak = pk.value

    value = R.aggregate_rate(cells * nv * args.steps, ws, t_dev)
    e2e_value = R.aggregate_rate(cells * nv, ws, t_e2e)
    # dominant kernel: largest accumulated time among the launch classes
    cls, (ms_tot, nl) = max(prof.items(), key=lambda kv: kv[1][0])
    avg_launch_s = ms_tot / 1e3 / max(nl, 1)
    cfg = s.config
    hbm_peak, hbm_src = measured_peaks()
    last_dir = f"hyp_{'xyz'[cfg.ndims - 1]}"
    if cls == last_dir:
        bytes_per_launch = cells * sum(stage_bytes(cfg, st) for st in range(cfg.rk_nstages)) / cfg.rk_nstages
    else:
        bytes_per_launch = cells * 8.0 * nv * 2  # read U, write the partial hyperbolic term
    achieved_gbs = bytes_per_launch / avg_launch_s / 1e9
    cls_dir = "xyz".index(cls[-1]) if cls.startswith("hyp_") else 0
    seg0 = tuned[cls_dir][0] if tuned else 0
    form = "lanes" if seg0 in (-8, -16) else ("tile" if seg0 < 0 else "walker")
    traffic = DRAM_BYTES_PER_CELL.get(args.workload, {}).get((cls, form))
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "traffic": traffic * cells if traffic else None,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of "
                                   + TRAFFIC_SOURCE[form]) if traffic else None, "kernel": cls,
                "kernel_form": form,
                "avg_launch_ms": avg_launch_s * 1e3, "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": bytes_per_launch}
    step_bytes = cells * sum(stage_bytes(cfg, st) + (8.0 * nv * 2) * (cfg.ndims - 1)
                             for st in range(cfg.rk_nstages))
    forms = ["lanes" if sg in (-8, -16) else ("tile" if sg < 0 else "walker") for sg, _ in tuned]
    known = FP64_PER_CELL_STEP.get(args.workload, {}) if not args.size else {}
    fw = None
    if known and all(f in known for f in forms):
        # per direction the form's share of the step (directions of one form each do half
        # of a 2-D step's work, a third of a 3-D step's)
        fw = {"flops": sum(known[f]["flops"] for f in forms) / len(forms),
              "instr": sum(known[f]["instr"] for f in forms) / len(forms),
              "captured": "; ".join(sorted({known[f]["captured"] for f in forms}))}
    roofline_fp64 = {"bound": "fp64", "peak": fp64_peak, "unit": "TFLOP/s",
                     "peak_source": "measured DFMA loop (gb_probe_fp64_peak) on this GPU"}
    if fw:
        ach = fw["flops"] * cells * args.steps / t_dev / 1e12
        ins = fw["instr"] * cells * args.steps
        pipe = ins / t_dev / (fp64_peak * 1e12 / 2.0)  # the pipe retires one FP64 instruction per FMA slot
        roofline_fp64.update({"achieved": ach, "frac": ach / fp64_peak, "flops_per_cell_step": fw["flops"],
                              "fp64_instr_per_cell_step": fw["instr"], "fp64_pipe_busy_frac": pipe,
                              "scope": "every kernel of the step, over the step's device time",
                              "flops_source": "ncu instruction counters of one step, " + fw["captured"]})
    launches_per_step = 0
    for k, (ms_k, n_k) in prof.items():
        # the viscous group is 5 kernels; a CRWENO5 direction is a solve and a flux kernel
        per = 5 if k == "viscous" else (2 if k.startswith("hyp") and cfg.hyp_scheme == 1 else 1)
        launches_per_step += per * n_k
    gpu_launches = launches_per_step  # counted over a pass of as many steps as the timed region
    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": common_config(case, desc, args, ws), "launch_seg_block_per_dir": tuned,
        "hbm_pct_step": 100.0 * (step_bytes / (t_dev / args.steps)) / 1e9 / hbm_peak,
        "roofline": roofline, "roofline_fp64": roofline_fp64,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": cells * nv * 8,
                "d2h_bytes_per_step": cells * nv * 8,
                "path": "gb_solver_set_state(host) + gb_solver_step(1) + gb_solver_get_state(host)"},
        "gpu_launches": gpu_launches, "clocks": clocks, "wall_s": wall, "finite": finite,
        "kernel_ms": {k: v[0] for k, v in prof.items() if v[1]},
    }
    pub = PUBLISHED.get(args.workload)
    if pub and not args.size:
        out["vs_baseline"] = value / pub[0]
        out["baseline_published"] = {"value": pub[0], "unit": UNIT, "hardware": pub[1]}
    if args.workload == "vortex" and ws == 1 and not args.size and not args.no_extras:
        # the metric's other two parts, measured after the timed region on reduced step
        # counts (stated in each block) so that the default run stays within minutes
        from hypar_gb300 import cases as C
        members = C.ensemble_vortex(64, n_iter=100)
        m = ensemble_measure(members, steps=3, warmup=1, local=local)
        out["ensemble"] = ensemble_summary(m, len(members), 3)
        out["ensemble"]["workload"] = ENSEMBLE_DESC
        out["ensemble"]["reduced"] = "3 timed steps (1 warm-up) per arm instead of 100"
        # many small members: where per-member launches, not FP64 work, set the pace
        small = C.ensemble_vortex(256, sizes=C.ensemble_sizes(256, 20261203, 32, 128, 16), n_iter=100)
        ms = ensemble_measure(small, steps=5, warmup=2, local=local)
        out["ensemble"]["small_members"] = ensemble_summary(ms, len(small), 5)
        out["ensemble"]["small_members"]["workload"] = SMALL_ENSEMBLE_DESC
        torch.cuda.set_stream(stream)
        block, _ = adjoint_measure(256, 400, 1, local, policies=("sqrt",), fd_directions=4,
                                   fd_kinds=("smooth", "noise"))
        block["workload"] = ADJOINT_DESC.format(n=256, nsteps=400)
        block["reduced"] = ("1 timed gradient (2 warm-up), sqrt checkpointing only, 4 central-difference "
                            "directions per kind instead of 16")
        out["adjoint"] = block
        torch.cuda.set_stream(stream)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(case, budget_s=args.cpu_budget)
    if dist:
        dist.destroy_process_group()
    return out


def ensemble_measure(members, steps: int, warmup: int, local: int, dist=None):
    """One batched ensemble (one launch per direction per stage, CUDA graph, autotuned)
    against the same members advanced one at a time by single-grid solvers, each with
    the default launch shape and with its size's autotuned shape.  Returns the times
    per step (seconds, max over ranks) and the batched launch shape."""
    import torch
    from hypar_gb300 import cases as C
    from hypar_gb300 import replicas as R
    from hypar_gb300.solver import Ensemble, Solver

    tmp = tempfile.mkdtemp(prefix="gbh_ens_")
    C.write_ensemble(members, tmp)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    e = Ensemble.from_dir(tmp, device=local)
    e.set_stream(stream.cuda_stream)
    tuned = e.autotune(1)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        e.step(1)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            e.step(1)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_b = R.max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / 1e3 / steps, dist, "cuda")
    e.close()
    tune_cache = {}
    t_s = 0.0   # one at a time, launch shape tuned per size (strongest single-grid baseline)
    t_d = 0.0   # one at a time, default launch shape (what gb_run_case does per deck)
    for k, c in enumerate(members):
        d = os.path.join(tmp, f"single_{k}")
        c.write(d)
        s = Solver.from_dir(d, device=local)
        s.set_stream(stream.cuda_stream)
        for tuned_run in (False, True):
            if tuned_run:
                key = tuple(c.size)
                if key not in tune_cache:
                    tune_cache[key] = s.autotune(1)
                for dd, (sg, bl) in enumerate(tune_cache[key]):
                    s.set_launch(dd, sg, bl)
            s.step(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush.fill_(1.0)
            a.record(stream)
            s.step(steps)
            b.record(stream)
            torch.cuda.synchronize()
            dt_ = a.elapsed_time(b) / 1e3 / steps
            if tuned_run:
                t_s += dt_
            else:
                t_d += dt_
        s.close()
    t_s = R.max_over_ranks(t_s, dist, "cuda")
    t_d = R.max_over_ranks(t_d, dist, "cuda")
    return {"t_batched": t_b, "t_tuned": t_s, "t_default": t_d, "tuned": tuned, "clocks": clk.summary()}


def ensemble_summary(m, nmembers: int, steps: int) -> dict:
    return {"batched_ms_per_step": m["t_batched"] * 1e3,
            "one_at_a_time_default_shape_ms_per_step": m["t_default"] * 1e3,
            "batched_vs_one_at_a_time_default_shape_speedup": m["t_default"] / m["t_batched"],
            "one_at_a_time_tuned_ms_per_step": m["t_tuned"] * 1e3,
            "batched_vs_one_at_a_time_tuned_speedup": m["t_tuned"] / m["t_batched"],
            "launches_per_step_batched": 2 * 3, "launches_per_step_one_at_a_time": 2 * 3 * nmembers,
            "timed_steps": steps, "batched_launch_seg_block_per_dir": m["tuned"]}


def run_ensemble(args, ws, rank, local):
    """64 isentropic vortices of seeded sizes {128..1024}: one batched ensemble
    (one launch per direction per stage, CUDA graph) against the same members
    advanced one at a time by single-grid solvers (each autotuned).  Over N GPUs
    the members are partitioned by cell count (every rank builds the whole
    seeded ensemble, so dt is the full ensemble's, and keeps its share); the
    job's time is the slowest rank's."""
    import numpy as np
    import torch
    from hypar_gb300 import cases as C
    from hypar_gb300 import replicas as R

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    everyone = C.ensemble_vortex(args.members, n_iter=100)
    total_cells = sum(int(np.prod(c.size)) for c in everyone)
    mine = R.shard_members([int(np.prod(c.size)) for c in everyone], ws)[rank]
    if not mine:
        raise SystemExit(f"rank {rank}: no ensemble member for this rank ({len(everyone)} members, {ws} ranks)")
    members = [everyone[k] for k in mine]
    m = ensemble_measure(members, args.steps, args.warmup, local, dist)
    if dist:
        dist.destroy_process_group()
    if rank != 0:
        return None
    t_b = m["t_batched"]
    value = total_cells * 4 / t_b
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_b * 1e3, "higher_is_better": True,
        "scaling": "strong" if ws > 1 else "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ENSEMBLE_DESC, "members": len(everyone), "cells": total_cells,
                   "sizes": [c.size[0] for c in everyone], "dt": everyone[0].dt,
                   "parallelism": (f"members partitioned over {ws} GPUs by cell count (rank 0: {len(mine)} "
                                   "members), no data exchanged" if ws > 1 else "single GPU"),
                   "launch_seg_block_per_dir": m["tuned"], "l2": "256 MB buffer written between timed steps"},
        "ensemble": ensemble_summary(m, len(everyone), args.steps),
        "gpu_launches": 6 * args.steps, "clocks": m["clocks"],
    }
    return out


ENSEMBLE_DESC = ("ensemble of 64 Euler2D isentropic vortices, sizes seeded from {128,192,...,1024}^2, b~U[1,5], "
                 "centre~U[3,7]^2, char-WENO5(JS)+Roe, SSPRK3, common dt at CFL 0.5")
SMALL_ENSEMBLE_DESC = ("ensemble of 256 Euler2D isentropic vortices, sizes seeded from {32,48,...,128}^2, "
                       "b~U[1,5], centre~U[3,7]^2, char-WENO5(JS)+Roe, SSPRK3, common dt at CFL 0.5")
ADJOINT_DESC = ("adjoint: d/d rho0 of 0.5||rho(T)-rho_target||^2, Euler2D {n}x{n} periodic [0,10)^2, target "
                "from the b=5 vortex, guess b=4 shifted by U[-0.5,0.5]^2, comp-WENO5(JS)+Roe, RK4, {nsteps} "
                "steps, sqrt checkpointing")


def adjoint_measure(n: int, nsteps: int, K: int, local: int, policies=("sqrt", "store_all"),
                    fd_directions: int = 16, fd_kinds=("smooth", "smooth_unit", "noise", "noise_unit")):
    """Gradient of 0.5 ||rho(T) - rho_target||^2 with respect to the initial density
    (2D Euler n^2 periodic, comp-WENO5 + Roe, RK4, nsteps steps) under each
    checkpoint policy (sqrt: ceil(sqrt(nsteps)) checkpoints; store_all: every state),
    timed as forward sweep + backward sweep over K gradients, against the plain fused
    forward solve of the same steps; then the sqrt gradient against central
    differences (h = 1e-6) on fd_directions random density directions per kind, and
    the adjoint against the tangent-linear model (dot-product test)."""
    import numpy as np
    import torch
    from hypar_gb300 import cases as C
    from hypar_gb300 import _lib
    from hypar_gb300.adjoint import Adjoint
    from hypar_gb300.solver import Inputs, Solver

    case, u_true = C.adjoint_problem(n, nsteps)
    tmp = tempfile.mkdtemp(prefix="gbh_adj_")
    case.write(tmp)
    inp = Inputs(tmp)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    s = Solver(inp.config, inp.dxinv, device=local)
    s.set_stream(stream.cuda_stream)
    s.set_state(case.u)
    fwd_shape = s.autotune(1)
    L = _lib.lib()
    results = {}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for tag in policies:
        ncheck = {"sqrt": 0, "store_all": 1}[tag]
        adj = Adjoint(inp.config, inp.dxinv, nsteps, ncheck=ncheck, device=local)
        adj.set_stream(stream.cuda_stream)
        for d, (sg, bl) in enumerate(fwd_shape):
            adj.set_launch(d, sg, bl)
        u_t = adj.ghosted(torch.from_numpy(u_true.reshape(n, n, 4).copy()).cuda()).contiguous()
        u0_int = torch.from_numpy(case.u.reshape(n, n, 4).copy()).cuda()
        u0 = adj.ghosted(u0_int).contiguous()
        vjp_shape = adj.autotune(u0)
        uT = adj.empty()
        adj.forward(u_t, uT)
        rho_tgt = adj.interior(uT)[..., 0].clone()
        adj.forward(u0, uT)
        ubarT = adj.empty()
        adj.interior(ubarT)[..., 0] = adj.interior(uT)[..., 0] - rho_tgt
        ub0 = adj.empty()
        for _ in range(2):
            adj.forward(u0, uT)
            adj.backward(ubarT, ub0)
        torch.cuda.synchronize()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
        with ClockSampler(local) as clk:
            for k in range(K):
                flush.fill_(float(k))
                ev[k][0].record(stream)
                _lib.check(L.gb_adjoint_forward(adj._h, u0.data_ptr(), uT.data_ptr()))
                ev[k][1].record(stream)
                _lib.check(L.gb_adjoint_backward(adj._h, ubarT.data_ptr(), ub0.data_ptr()))
                ev[k][2].record(stream)
            torch.cuda.synchronize()
        t_fs = sum(e[0].elapsed_time(e[1]) for e in ev) / K
        t_bs = sum(e[1].elapsed_time(e[2]) for e in ev) / K
        info = adj.info()
        results[tag] = {"ncheck": ncheck, "adj": adj, "t_fs": t_fs, "t_bs": t_bs, "info": info,
                        "vjp_seg": vjp_shape, "clocks": clk.summary(), "u0": u0, "u0_int": u0_int,
                        "rho_tgt": rho_tgt, "ub0": ub0.clone()}
        if tag != policies[0]:
            adj.close()  # only the first policy's adjoint is kept for the checks below
    # the plain forward solve: the solver's fused steps over the same steps
    s.set_state(case.u)
    s.step(nsteps)
    tf = []
    for k in range(K):
        s.set_state(case.u)
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _lib.check(L.gb_solver_step(s.handle, nsteps))
        b.record(stream)
        torch.cuda.synchronize()
        tf.append(a.elapsed_time(b))
    t_f = sum(tf) / K
    s.close()
    # accuracy: central differences and the dot-product test, with the first policy's adjoint
    R = results[policies[0]]
    adj, u0_int, rho_tgt = R["adj"], R["u0_int"], R["rho_tgt"]
    grad = adj.interior(R["ub0"])[..., 0]

    def misfit(u_int):
        out = adj.empty()
        adj.forward(adj.ghosted(u_int).contiguous(), out)
        r = adj.interior(out)[..., 0] - rho_tgt
        return 0.5 * float((r * r).sum())

    h = 1e-6
    gen = torch.Generator(device="cpu").manual_seed(20261203)
    rng = np.random.default_rng(20261203)
    xg = np.arange(n) / n
    X, Y = np.meshgrid(xg, xg, indexing="xy")

    def smooth_field():
        f = np.zeros((n, n))
        for _ in range(6):
            kx, ky = rng.integers(-4, 5, size=2)
            f += rng.normal() * np.sin(2 * np.pi * (kx * X + ky * Y) + rng.uniform(0, 2 * np.pi))
        return torch.from_numpy(f).cuda()

    fd = {k: [] for k in fd_kinds}
    for kind in fd:
        for _ in range(fd_directions):
            v = smooth_field() if kind.startswith("smooth") else torch.randn((n, n), generator=gen,
                                                                                dtype=torch.float64).cuda()
            if kind.endswith("unit"):
                v /= float(v.norm())
            up, um = u0_int.clone(), u0_int.clone()
            up[..., 0] += h * v
            um[..., 0] -= h * v
            d = (misfit(up) - misfit(um)) / (2 * h)
            g = float((grad * v).sum())
            fd[kind].append(abs(d - g) / max(abs(d), abs(g)))
    v = adj.ghosted(torch.randn((n, n, 4), generator=gen, dtype=torch.float64).cuda()).contiguous()
    w = adj.ghosted(torch.randn((n, n, 4), generator=gen, dtype=torch.float64).cuda()).contiguous()
    uT2, Mv, MTw, uT = adj.empty(), adj.empty(), adj.empty(), adj.empty()
    adj.tlm(R["u0"], v, uT2, Mv)
    adj.forward(R["u0"], uT)
    adj.backward(w, MTw)
    lhs = float((adj.interior(Mv) * adj.interior(w)).sum())
    rhs_ = float((adj.interior(v) * adj.interior(MTw)).sum())
    dot_err = abs(lhs - rhs_) / max(abs(lhs), abs(rhs_))
    ns = inp.config.rk_nstages
    launches_fs = nsteps * ns * 2
    launches_bs = R["info"]["recomputed_steps"] * ns * 2 + nsteps * (ns + 1)
    adj.close()
    block = {"forward_solve_ms": t_f, "timed_gradients": K, "nsteps": nsteps, "cells": n * n}
    for tag in policies:
        P = results[tag]
        g_ms = P["t_fs"] + P["t_bs"]
        block[tag] = {"forward_sweep_ms": P["t_fs"], "backward_sweep_ms": P["t_bs"], "gradient_ms": g_ms,
                      "gradient_over_forward": g_ms / t_f, "backward_over_forward": P["t_bs"] / t_f,
                      "checkpoints": P["info"]["segments"], "recomputed_steps": P["info"]["recomputed_steps"],
                      "device_bytes": P["info"]["bytes"], "vjp_seg": P["vjp_seg"]}
    block["fd_check"] = {kind: {"directions": fd_directions, "h": h, "max_rel_err": max(e),
                                "median_rel_err": statistics.median(e)} for kind, e in fd.items()}
    block["fd_directions"] = ("smooth: 6 random Fourier modes |k| <= 4 of the initial density (amplitude "
                              "O(1) per cell); noise: N(0,1) in every cell; *_unit: the same scaled to unit "
                              "2-norm (a per-cell step near 1e-6/n, where rounding in the misfit dominates "
                              "the difference); central differences of the misfit through the fused forward "
                              "solve")
    block["dot_product_rel_err"] = dot_err
    block["forward_launch_seg_block"] = fwd_shape
    return block, {"grad_ms": R["t_fs"] + R["t_bs"], "t_f": t_f, "clocks": R["clocks"], "dt": case.dt,
                   "info": R["info"], "launches": K * (launches_fs + launches_bs)}


def run_adjoint(args, ws, rank, local):
    """The adjoint configuration (256^2, RK4, 400 steps, sqrt checkpointing) as its own
    line: a "step" is one gradient evaluation (forward sweep with checkpoints +
    backward sweep); value = gradient time / plain forward solve time."""
    import torch

    torch.cuda.set_device(local)
    n = args.size or 256
    nsteps = 400
    K = max(1, min(args.steps, 5))
    block, extra = adjoint_measure(n, nsteps, K, local)
    return {
        "metric": METRIC, "value": extra["grad_ms"] / extra["t_f"], "unit": "x (gradient time / forward solve time)",
        "n_gpus": 1, "steps": K, "warmup": 2, "ms_per_step": extra["grad_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ADJOINT_DESC.format(n=n, nsteps=nsteps), "cells": n * n, "dt": extra["dt"],
                   "nsteps": nsteps, "checkpoints": extra["info"]["segments"],
                   "segment_len": extra["info"]["segment_len"],
                   "l2": "256 MB buffer written between timed gradients"},
        "adjoint": block,
        "gpu_launches": extra["launches"], "clocks": extra["clocks"],
    }


def run_parity(args, ws, rank, local):
    """Where the per-right-hand-side distance from the oracle comes from, on the
    benchmark's vortex (char-WENO5 + Roe) at 128^2 .. 1024^2.  Three evaluations of
    the same right-hand side: the GPU, the oracle (the reference's operation order,
    no contraction) and the oracle compiled with FMA contraction (the same formulas
    and order, rounded differently).  Their pairwise relative L2 distances d give,
    if their rounding errors are independent, each one's own error against the
    exact right-hand side: e_a^2 = (d_ab^2 + d_ac^2 - d_bc^2) / 2.  Then the 100-step
    state distance at 1024^2 (the benchmark configuration)."""
    import numpy as np
    import torch
    import oracle as O
    from hypar_gb300 import cases as C
    from hypar_gb300.solver import Solver

    torch.cuda.set_device(local)
    O.build()
    O.set_threads(os.cpu_count() or 1)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    rows = []
    sizes = [int(v) for v in args.parity_sizes.split(",")]
    for n in sizes:
        case = C.vortex(n, n_iter=1)
        d = tempfile.mkdtemp(prefix=f"gbh_par{n}_")
        case.write(d)
        s = Solver.from_dir(d, device=local)
        P, PF = O.Problem(case), O.Problem(case, fma=True)
        u0 = P.u0()
        out = torch.zeros(u0.size, dtype=torch.float64, device="cuda")
        s.rhs(out, torch.from_numpy(u0).cuda())
        g = O.interior(out.cpu().numpy(), case.size, 4, 3)
        o = O.interior(P.rhs(u0.copy()), case.size, 4, 3)
        f = O.interior(PF.rhs(u0.copy()), case.size, 4, 3)
        d_go, d_gf, d_of = rel(g, o), rel(g, f), rel(f, o)
        e2 = lambda a, b, c: max((a * a + b * b - c * c) / 2.0, 0.0) ** 0.5  # noqa: E731
        rows.append({"n": n, "gpu_vs_oracle": d_go, "gpu_vs_oracle_fma": d_gf, "oracle_vs_oracle_fma": d_of,
                     "own_error_gpu": e2(d_go, d_gf, d_of), "own_error_oracle": e2(d_go, d_of, d_gf),
                     "own_error_oracle_fma": e2(d_gf, d_of, d_go),
                     "per_variable_gpu_vs_oracle": [rel(g[:, k], o[:, k]) for k in range(4)]})
        s.close()
    state = None
    if args.steps > 0:
        n = sizes[-1]
        case = C.vortex(n, n_iter=args.steps)
        d = tempfile.mkdtemp(prefix="gbh_parsteps_")
        case.write(d)
        s = Solver.from_dir(d, device=local)
        s.step(args.steps)
        got = s.get_state()
        s.close()
        P = O.Problem(case)
        ref = O.interior(P.rk(P.u0(), args.steps), case.size, 4, 3).reshape(-1)
        state = {"n": n, "steps": args.steps, "gpu_vs_oracle_state": rel(got, ref)}
    return {"metric": "relative L2 distance of one right-hand side, GPU vs oracle", "value": rows[-1]["gpu_vs_oracle"],
            "unit": "relative L2", "n_gpus": 1, "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "Euler2D isentropic vortex b=5, char-WENO5(JS)+Roe, t=0 state",
                       "sizes": sizes},
            "rhs": rows, "state": state}


def run_kernel_probe(args, ws, rank, local):
    """Single-entry-point launches for profilers (nothing timed, no JSON metric): the
    adjoint test problem (Euler2D n^2, comp-WENO5 + Roe, RK4) and --steps calls of one
    entry point: the right-hand side's VJP (gb_adjoint_rhs_vjp, --launch sx,sy sets the
    reverse kernel's segment lengths), its dual-number JVP (gb_adjoint_rhs_jvp), or
    one fused Runge-Kutta step (gb_solver_step).  Nothing else is launched besides
    the set-up copies, so a profiler can select the launches by kernel name."""
    import torch
    from hypar_gb300 import cases as C
    from hypar_gb300.adjoint import Adjoint
    from hypar_gb300.solver import Inputs, Solver

    torch.cuda.set_device(local)
    what = args.workload.split("-", 1)[1]
    n = args.size or 256
    case, _ = C.adjoint_problem(n, 4)
    d = tempfile.mkdtemp(prefix="gbh_kprobe_")
    case.write(d)
    inp = Inputs(d)
    if what == "step":
        s = Solver(inp.config, inp.dxinv, device=local)
        s.set_state(case.u)
        s.step(args.steps)
        s.sync()
        return {"probe": what, "size": n, "calls": args.steps, "ok": True}
    adj = Adjoint(inp.config, inp.dxinv, 4, 0, local)
    if args.launch and what == "vjp":
        sx, sy = (int(v) for v in args.launch.split(","))
        adj.set_launch(2, sx)
        adj.set_launch(3, sy)
    u = adj.ghosted(torch.from_numpy(case.u.reshape(n, n, 4).copy()).cuda()).contiguous()
    a, b = adj.empty(), adj.empty()
    a.normal_()
    for _ in range(args.steps):
        if what == "vjp":
            adj.rhs_vjp(u, a, b)
        else:
            adj.rhs_jvp(u, a, b, adj.empty())
    torch.cuda.synchronize()
    return {"probe": what, "size": n, "calls": args.steps, "ok": True}


def run_convergence(args, ws, rank, local):
    """Grid convergence on the smooth isentropic vortex (b = 5, periodic [0,10)^2,
    characteristic WENO5 + Roe): grids 64^2..512^2, one small dt for all (RK4,
    dt = 1e-3, so the time error is ~1e-13 and the spatial error dominates),
    T = 0.5; errors against the translated exact vortex through the library's
    CalculateError (gb_solver_error, the whole domain, relative), and the L2 error
    over the centre [2,8]^2 (away from the periodic seam, where the vortex's
    exp(-12) tail leaves a 5e-5 jump in v that no grid resolves)."""
    import numpy as np
    import torch
    from hypar_gb300 import cases as C
    from hypar_gb300.solver import Solver

    torch.cuda.set_device(local)
    dt, T = 1e-3, 0.5
    nsteps = int(round(T / dt))
    rows = []
    t0 = time.perf_counter()
    for n in (64, 128, 256, 512):
        case = C.vortex(n, n_iter=nsteps, dt=dt, interp="characteristic", upwinding="roe", scheme="44")
        d = tempfile.mkdtemp(prefix=f"gbh_conv{n}_")
        case.write(d)
        s = Solver.from_dir(d, device=local)
        s.step(nsteps)
        x, uex = C.vortex_state(n, 5.0, 5.0 + 0.5 * T, 5.0)
        err = s.error(uex)
        u = s.get_state().reshape(n, n, 4)
        ue = uex.reshape(n, n, 4)
        m = (x >= 2.0) & (x <= 8.0)
        e = (u - ue)[m][:, m]
        centre_l2 = float(np.sqrt(np.mean(e * e)) / np.sqrt(np.mean(ue[m][:, m] ** 2)))
        rows.append({"n": n, "L1": err[0], "L2": err[1], "Linf": err[2], "centre_L2": centre_l2})
        s.close()
    wall = time.perf_counter() - t0
    for a, b in zip(rows, rows[1:]):
        for k in ("L1", "L2", "Linf", "centre_L2"):
            b["order_" + k] = float(np.log2(a[k] / b[k]))
    last = rows[-1]
    return {
        "metric": "spatial convergence order (L2, 256^2 -> 512^2)", "value": last["order_L2"], "unit": "order",
        "n_gpus": 1, "steps": nsteps, "warmup": 0, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": ("Euler2D isentropic vortex b=5 on [0,10)^2 periodic, char-WENO5(JS)+Roe, RK4, "
                                f"dt={dt}, T={T}, grids 64..512"),
                   "exact": "translated vortex (centre + 0.5 T, 0)"},
        "convergence": rows, "wall_s": wall,
    }


def cpu_baseline(case, budget_s: float = 15.0, threads: int = 0):
    """The oracle (the reference algorithm restated in C) on the host cores,
    timed on whole steps of the same workload until budget_s has elapsed."""
    import numpy as np
    import oracle as O
    O.build()
    n = threads or os.cpu_count() or 1
    O.set_threads(n)
    P = O.Problem(case)
    u = P.u0()
    cells = int(np.prod(case.size))
    t0 = time.perf_counter()
    steps = 0
    while True:
        u = P.rk(u, 1)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    return {"value": cells * case.nvars * steps / el, "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"{steps} full step(s) of the same workload in {el:.1f} s, {n} OpenMP threads",
            "seconds_per_step": el / steps}


def run_ref_vs_port(args, case, desc):
    """The reference's own CPU build (oracle/_ref/HyPar, compiled from the reference's
    sources by oracle/Makefile.ref where they are present) against the oracle port on
    the same deck, single-threaded and with every host thread: seconds per step of
    each.  A step of the reference is timed as the difference of two runs of the same
    deck (n_iter = 1 and 1 + steps), which cancels start-up, input and output.  The
    reference's OpenMP build races in characteristic WENO5 (L and uavg shared in
    WENOFifthOrderCalculateWeightsCharJS); its timing is still its own."""
    import numpy as np
    import oracle as O
    exe = os.path.join(ROOT, "oracle", "_ref", "HyPar")
    if not os.path.exists(exe):
        return {"impl": "ref-vs-port", "unavailable": "oracle/_ref/HyPar is not built here (needs the reference's "
                                                      "source tree, HYPAR_REF)"}
    O.build()
    steps = max(1, args.steps)
    nthr = os.cpu_count() or 1
    cells = int(np.prod(case.size))

    def ref_time(n_iter, threads):
        d = tempfile.mkdtemp(prefix="gbh_refrun_")
        case.n_iter = n_iter
        case.file_op_iter = 10 ** 6
        case.write(d)
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        t0 = time.perf_counter()
        subprocess.run([exe], cwd=d, env=env, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        return time.perf_counter() - t0

    def port_time(threads):
        O.set_threads(threads)
        P = O.Problem(case)
        u = P.rk(P.u0(), 1)
        t0 = time.perf_counter()
        P.rk(u, steps)
        return (time.perf_counter() - t0) / steps

    rows = {}
    for threads in (1, nthr):
        tr = (ref_time(1 + steps, threads) - ref_time(1, threads)) / steps
        tp = port_time(threads)
        rows[str(threads)] = {"reference_s_per_step": tr, "port_s_per_step": tp, "port_speedup": tr / tp}
    return {"impl": "ref-vs-port", "config": {"workload": desc, "cells": cells, "timed_steps": steps},
            "threads": rows,
            "note": "reference = the reference's own serial+OpenMP build of its sources; port = oracle/gbh_oracle.c"}


def run_reference(args, case, desc, ws, rank):
    if rank != 0:
        return None
    import numpy as np
    import oracle as O
    O.build()
    n = os.cpu_count() or 1
    O.set_threads(n)
    P = O.Problem(case)
    u = P.u0()
    cells = int(np.prod(case.size))
    sub = case
    # keep the whole run within a few minutes: time one step first
    t0 = time.perf_counter()
    u = P.rk(u, 1)
    t1 = time.perf_counter() - t0
    total = t1 * (args.steps + args.warmup)
    sample = "full grid"
    if total > 180.0 and case.model == "euler2d":
        from hypar_gb300 import cases as C
        sub = C.vortex(512, n_iter=1, dt=case.dt, interp=case.interp, upwinding=case.upwinding,
                       scheme=case.time_scheme_type)
        P = O.Problem(sub)
        u = P.u0()
        cells = int(np.prod(sub.size))
        sample = "512x512 sub-grid of the same vortex (same dt, scheme)"
    elif total > 180.0 and case.model == "navierstokes3d":
        sub, _ = workload(args.workload, 64)
        P = O.Problem(sub)
        u = P.u0()
        cells = int(np.prod(sub.size))
        sample = "64^3 grid of the same problem (same dt, scheme)"
    for _ in range(max(args.warmup - 1, 0)):
        u = P.rk(u, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u = P.rk(u, 1)
    el = time.perf_counter() - t0
    value = cells * sub.nvars * args.steps / el
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": common_config(case, desc, args, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": n, "kind": "port",
                         "sample": f"{args.steps} timed steps ({sample}, {cells} cells), {n} OpenMP threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference", "ref-vs-port"],
                    help="ref-vs-port: the reference's own CPU build against the oracle port (CPU only, where "
                         "the reference's sources were built into oracle/_ref)")
    ap.add_argument("--workload", default="vortex", choices=["vortex", "tgv", "sod", "rtb", "rtb64", "dns", "dns64cr", "ensemble", "adjoint",
                                                          "convergence", "parity", "kernel-vjp", "kernel-jvp",
                                                          "kernel-step"])
    ap.add_argument("--parity-sizes", default="128,256,512,1024", help="grid sizes of --workload parity")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload only: leave out the ensemble and adjoint blocks")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--size", type=int, default=0, help="override the grid size (profiling of small cases)")
    ap.add_argument("--launch", default="", help="fixed launch shape per direction instead of the autotuner's, "
                                                 "seg[:block] per direction, e.g. -128,-128 (tiles of 128 "
                                                 "interfaces) or 64:128,43:128,43:128")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_env()
    if args.workload in ("ensemble", "adjoint", "convergence", "parity", "kernel-vjp", "kernel-jvp", "kernel-step"):
        from hypar_gb300 import build as B
        B.build()
        fn = {"ensemble": run_ensemble, "adjoint": run_adjoint, "convergence": run_convergence,
              "parity": run_parity, "kernel-vjp": run_kernel_probe, "kernel-jvp": run_kernel_probe,
              "kernel-step": run_kernel_probe}[args.workload]
        out = fn(args, ws, rank, local) if args.impl == "ours" else None
        if out is not None and rank == 0:
            print(json.dumps(out))
        return
    case, desc = workload(args.workload, args.size)
    if args.impl == "ref-vs-port":
        print(json.dumps(run_ref_vs_port(args, case, desc)))
        return
    if args.impl == "reference":
        out = run_reference(args, case, desc, ws, rank)
    else:
        from hypar_gb300 import build as B
        B.build()
        out = run_ours(args, case, desc, ws, rank, local)
    if out is not None and rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
