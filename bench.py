#!/usr/bin/env python3
"""Benchmark: LMM path-steps/s of the LIBOR Market Model Monte Carlo path on one GB300.

Workload (one "step" = one full valuation pass): the lmm40 configuration -- 40
semi-annual forwards (0-20y), 80 Euler-log steps of 0.25y, 10 factors, 2^20 paths,
MT19937 seed 7 -- generating the Brownian increments, simulating the paths with the
spot-measure drift and numeraire, and valuing the 1y-19.5y payer Bermudan swaption by
regression ({1,S,S^2,N,N^2,S*N}) and the 10y-into-10y payer swaption.  Metric = paths *
time steps / seconds.  Synthetic inputs as the workload defines them; the Brownian
increments (6.7 GB) are larger than L2, so no separate flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --case valuation|greeks|portfolio --precision fp64|mixed --paths P --repeat R
      (one named valuation case, for profiling single kernels under ncu)

--impl reference times the CPU restatement of the reference's algorithm (the oracle,
C, all host threads) on a bounded sample of the same workload; under torchrun only
rank 0 runs it.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
for _p in (HERE, os.path.join(HERE, "finmath-lib_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "LMM path-steps/s"
UNIT = "path-steps/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(paths: int, threads: int):
    """The oracle (C restatement of the reference's path) on a bounded sample of the workload."""
    from oracle import pyoracle as po
    from finmath_gb300 import workloads as W
    cfg = W.LMM40
    m = po.build_model(**{k: cfg[k] for k in ("dt", "T_end", "period", "tenor_end", "F", "corr_decay", "abcd",
                                              "curve_nodes", "curve_values")})
    obs = np.zeros(m.T + 1, np.uint8)
    obs[W.tenor_time_indices(cfg)] = 1
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    ex, sfix, spay, sK = W.swaption_schedule(cfg)
    t0 = time.perf_counter()
    dW = po.brownian_increments(m.times, m.F, paths, cfg["seed"])
    sim = po.Simulation(m, dW, observe=obs, threads=threads)
    berm = sim.bermudan(fix, plen, pay, K, basis_id=1)
    swpt = sim.swaption(ex, sfix, spay, sK)
    dt = time.perf_counter() - t0
    return paths * m.T / dt, dt, berm, swpt


def headline_parity(F, W, cfg, sim, berm, swpt, paths, threads):
    """The oracle's valuation of the same workload, timed as the CPU baseline and, when it
    runs at the bench's own path count, compared with the GPU's FP64 valuation of the same
    paths (outside the timed region): Bermudan and swaption value and standard error,
    every per-path Bermudan value, and forward rates and numeraires at a few times."""
    from oracle import pyoracle as po
    m = po.build_model(**{k: cfg[k] for k in ("dt", "T_end", "period", "tenor_end", "F", "corr_decay", "abcd",
                                              "curve_nodes", "curve_values")})
    obs = np.zeros(m.T + 1, np.uint8)
    tenor_tidx = W.tenor_time_indices(cfg)
    obs[tenor_tidx] = 1
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    ex, sfix, spay, sK = W.swaption_schedule(cfg)
    t0 = time.perf_counter()
    dW = po.brownian_increments(m.times, m.F, paths, cfg["seed"])
    osim = po.Simulation(m, dW, observe=obs, threads=threads)
    ob = osim.bermudan(fix, plen, pay, K, basis_id=1, per_path=True)
    os_ = osim.swaption(ex, sfix, spay, sK)
    dt = time.perf_counter() - t0
    del dW
    rate = paths * m.T / dt
    if sim is None or paths != sim.getNumberOfPaths() or sim.process.brownianMotion.precision != F.PRECISION_FP64:
        return rate, dt, None
    gb = berm.getValues(sim, per_path=True)
    gs = swpt.getValues(sim)

    def rel(a, b):
        return abs(a - b) / abs(b)

    vg, vo = gb["values"], ob[2]
    scale = float(np.max(np.abs(vo)))
    dpath = np.abs(vg - vo)
    states = []
    for t, j in ((tenor_tidx[20], 39), (tenor_tidx[-1], 39), (tenor_tidx[2], 10)):
        g, o = sim.process.getProcessValue(int(t), j), osim.process_value(int(t), j)
        states.append({"time_index": int(t), "component": j, "max_rel": float(np.max(np.abs(g - o) / np.abs(o)))})
    nums = []
    for T_ in (1.0, 10.0, 20.0):
        g, o = sim.process.getNumeraire(T_), osim.numeraire(T_)
        nums.append({"time": T_, "max_rel": float(np.max(np.abs(g - o) / np.abs(o)))})
    parity = {
        "paths": paths, "oracle": "oracle/lmm_oracle.c (C restatement of the reference, OpenMP)",
        "bermudan": {"gpu": gb["value"], "oracle": ob[0], "rel": rel(gb["value"], ob[0]),
                     "error_gpu": gb["error"], "error_oracle": ob[1], "error_rel": rel(gb["error"], ob[1])},
        "swaption": {"gpu": gs["value"], "oracle": os_[0], "rel": rel(gs["value"], os_[0]),
                     "error_gpu": gs["error"], "error_oracle": os_[1], "error_rel": rel(gs["error"], os_[1])},
        "bermudan_per_path": {"paths_compared": int(vg.size), "max_abs_over_max_value": float(np.max(dpath) / scale),
                              "paths_beyond_1e-12": int(np.count_nonzero(dpath > 1e-12 * scale))},
        "forward_rates": states, "numeraires": nums,
    }
    parity["within_1e-12"] = bool(parity["bermudan"]["rel"] <= 1e-12 and parity["swaption"]["rel"] <= 1e-12)
    return rate, dt, parity


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    paths = args.cpu_paths
    for _ in range(args.warmup):
        cpu_baseline(paths, threads)
    times = []
    for _ in range(args.steps):
        v, dt, _, _ = cpu_baseline(paths, threads)
        times.append(dt)
    value = paths * 80 * args.steps / sum(times)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "lmm40 (40 forwards, 80 steps, 10 factors, seed 7)", "paths_per_step": paths,
                       "note": "finmath-lib is Java and no JDK exists on this box; the timed CPU path is the "
                               "oracle, a C restatement of the reference's algorithm (sequential MT19937 + ICDF, "
                               "OpenMP Euler over paths, Bermudan regression)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{paths} paths of lmm40 per step (full workload: 1,048,576)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _ncu_counters(kernel, paths):
    """DRAM bytes per launch of a path kernel from the committed ncu counters
    (profiles/ncu_counters.json: one capture on a smaller case), scaled to `paths` by the
    path count (the kernel streams increments in and states out per path, so its traffic
    grows in proportion), with the pipe activity of the same capture; None if absent."""
    try:
        with open(os.path.join(HERE, "profiles", "ncu_counters.json")) as f:
            rec = json.load(f)[kernel]
    except (OSError, ValueError, KeyError):
        return None
    scale = paths / rec["paths"]
    return {"traffic": (rec["dram_bytes_read"] + rec["dram_bytes_write"]) * scale,
            "inst_executed": rec["inst_executed"] * scale if rec.get("inst_executed") else None,
            "pipe_active": rec.get("pipe_active"), "captured_paths": rec["paths"], "scale": scale}


def _measured_hbm_gbs():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"


def kernel_rooflines(stats, steps, P, T, N, Fk, comp_steps, ne, fp64, fp64_peak_tflops):
    """Per kernel family: algorithmic bytes and flops per step over its measured time per step,
    against the measured HBM copy bandwidth and the live FP64 FMA peak; frac = the larger."""
    hbm, hbm_src = _measured_hbm_gbs()
    esz = 8 if fp64 else 4
    nobs = N + 1
    work = {
        # name: (bytes per step, flops per step, flops peak in TFLOP/s or None)
        "mt19937_jump_generate": (T * Fk * P * esz, 0.0, None),
        "lmm_paths_fp64" if fp64 else "lmm_paths_fp32": (
            T * Fk * P * esz + nobs * N * P * esz + (N + 1) * P * 8, P * comp_steps * (6 * Fk + 11),
            fp64_peak_tflops if fp64 else None),
        # Gram pass + backward induction: per exercise date and path ~64 bytes
        "bermudan_regress_step": (64.0 * P * ne, 0.0, None),
        "swaption_value": (P * (10 * esz + 8 + 8), 0.0, None),
    }
    out = {}
    for name, (nbytes, flops, fpeak) in work.items():
        if name not in stats or stats[name][0] == 0:
            continue
        sec = stats[name][1] / max(steps, 1) * 1e-3
        gbs = nbytes / sec / 1e9
        e = {"ms_per_step": sec * 1e3, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "hbm_frac": gbs / hbm}
        if flops and fpeak:
            # FP64-equivalent flops of the reference algorithm; the kernel runs them as
            # double-float pairs on the FP32 pipe (its issue roofline is the headline's)
            e["fp64_equivalent_tflops"] = flops / sec / 1e12
            e["fp64_equivalent_vs_fp64_peak"] = e["fp64_equivalent_tflops"] / fpeak
        e["frac"] = e["hbm_frac"]
        out[name] = e
    out["peaks"] = {"hbm_gbs": hbm, "hbm_source": hbm_src, "fp64_tflops": fp64_peak_tflops,
                    "fp64_source": "live DFMA probe x2"}
    return out


def run_ours(args):
    import torch
    import finmath_gb300 as F
    from finmath_gb300 import workloads as W

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    L = F.load()
    cfg = W.LMM40
    P = args.paths
    prec = F.PRECISION_MIXED if args.precision == "mixed" else F.PRECISION_FP64
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    ex, sfix, spay, sK = W.swaption_schedule(cfg)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    swpt = F.Swaption(ex, sfix, spay, sK)
    T = int(round(cfg["T_end"] / cfg["dt"]))

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # ---------------- device-resident throughput: model tables uploaded once, increments,
    # paths and products recomputed every step (the seed is re-set to force regeneration)
    sim = W.build(cfg, paths=P, precision=prec)
    stream = ctypes.c_void_p()
    L.lmm_process_stream(sim.process._h, ctypes.byref(stream))
    ts = torch.cuda.ExternalStream(stream.value)
    bm = sim.process.brownianMotion

    def step():
        bm.setSeed(cfg["seed"])
        b = berm.getValues(sim)
        s = swpt.getValues(sim)
        return b, s

    for _ in range(args.warmup):
        res = step()
    barrier()
    L.lmm_stats_reset()
    L.lmm_stats_enable_timing(1)
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(ts)
    for _ in range(args.steps):
        res = step()
    e1.record(ts)
    barrier()
    clk = clocks.stop()
    L.lmm_stats_enable_timing(0)
    ms = e0.elapsed_time(e1) / args.steps
    stats = F.kernel_stats()
    launches = sum(v[0] for v in stats.values())
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * P * T / (ms * 1e-3)

    # ---------------- roofline of the dominant kernel (the path kernel)
    kname = "lmm_paths_fp32" if prec == F.PRECISION_MIXED else "lmm_paths_fp64"
    k_launch, k_ms = stats[kname]
    k_avg_s = k_ms / max(k_launch, 1) * 1e-3
    td = F.TimeDiscretizationFromArray(0.0, T, cfg["dt"]).getAsDoubleArray()
    tenor = np.arange(0.0, cfg["tenor_end"] + 1e-9, cfg["period"])
    N, Fk = len(tenor) - 1, cfg["F"]
    comp_steps = sum(N - (int(np.searchsorted(tenor, t, side="right"))) for t in td[:-1])
    flops = P * comp_steps * (6 * Fk + 8 + 3)   # add/mul of drift+diffusion, plus div, exp, log
    fma = ctypes.c_double()
    L.lmm_probe_fp64_fma_rate(ctypes.byref(fma))
    peak = 2.0 * fma.value / 1e12
    algorithmic = flops / k_avg_s / 1e12
    counters = _ncu_counters(kname, P)
    traffic = counters["traffic"] if counters else None
    if prec == F.PRECISION_FP64:
        # The FP64 form runs the drift and diffusion sums, the exponential's polynomial and the
        # splits on the FP32 pipe in double-float arithmetic and keeps three FP64 instructions
        # per component-step, so neither DRAM (under 1 TB/s) nor the FP64 pipe binds it:
        # instruction issue does.  achieved = the kernel's warp instructions per launch (ncu's
        # count at a smaller path count, scaled by the paths: the instructions per path do not
        # depend on the path count) over the launch time; peak = one warp instruction per cycle
        # per SM sub-partition (4 per SM) at the SM clock sampled during the timed region.
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        sm_mhz = float(clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0)
        issue_peak = 4.0 * sms * sm_mhz * 1e6 / 1e9
        inst = counters["inst_executed"] if counters else None
        achieved = inst / k_avg_s / 1e9 if inst else None
        roofline = {"bound": "issue", "kernel": kname, "achieved": achieved, "peak": issue_peak,
                    "unit": "G warp-instructions/s", "frac": achieved / issue_peak if achieved else None,
                    "traffic": traffic, "inst_per_launch": inst,
                    "peak_source": f"4 issue slots per SM x {sms} SMs x {sm_mhz:.0f} MHz (SM clock median during the "
                                   "timed region)",
                    "avg_launch_ms": k_avg_s * 1e3, "component_steps_per_path": comp_steps,
                    "algorithmic_flops_per_launch": flops,
                    "fp64_equivalent_tflops": algorithmic, "fp64_peak_tflops": peak,
                    "fp64_equivalent_vs_fp64_peak": algorithmic / peak,
                    "ncu_fma_pipe_active": counters["pipe_active"] if counters else None,
                    "traffic_source": (f"ncu DRAM read+write of one launch at {counters['captured_paths']} paths, "
                                       f"scaled x{counters['scale']:g} by the path count") if counters else None,
                    "note": "FP64-equivalent flops count the reference algorithm's add/mul per component-step (its "
                            "log, exp and division as one each); the kernel carries them as double-float pairs on "
                            "the FP32 pipe, so that rate exceeds the chip's FP64 peak (live DFMA probe x2)"}
    else:
        hbm, hbm_src = _measured_hbm_gbs()
        nbytes = T * Fk * P * 4 + (N + 1) * N * P * 4 + 2 * (N + 1) * P * 8
        achieved_gbs = nbytes / k_avg_s / 1e9
        roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                    "frac": achieved_gbs / hbm, "traffic": traffic, "algorithmic_bytes_per_launch": nbytes,
                    "algorithmic_flops_per_launch": flops, "algorithmic_tflops": algorithmic,
                    "avg_launch_ms": k_avg_s * 1e3, "peak_source": hbm_src,
                    "ncu_pipe_active": counters["pipe_active"] if counters else None}

    # ---------------- end to end through the C ABI with host buffers (tables in, prices out)
    e2e_times = []
    h2d = d2h = 0
    for i in range(args.steps + 1):
        torch.cuda.synchronize()
        h2d0 = ctypes.c_int64()
        L.lmm_stats_h2d_bytes(ctypes.byref(h2d0))
        t0 = time.perf_counter()
        s2 = W.build(cfg, paths=P, precision=prec)
        b2 = berm.getValues(s2)
        w2 = swpt.getValues(s2)
        s2.process.close()
        s2.process.brownianMotion.close()
        torch.cuda.synchronize()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
        if i == 0:
            # every host-to-device copy the library made during the valuation (tables, the
            # seeded state, the generator's jump lists, product schedules), as it counts them
            h2d1 = ctypes.c_int64()
            L.lmm_stats_h2d_bytes(ctypes.byref(h2d1))
            h2d = int(h2d1.value - h2d0.value)
            d2h = 4 * 16
    e2e_ms = 1e3 * statistics.mean(e2e_times)
    if dist is not None:
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = {"value": ws * P * T / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
           "note": "C-ABI valuation from host tables: Brownian motion + process creation, lazy "
                   "generation/simulation, Bermudan + swaption values read back, handles destroyed"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == F.PRECISION_FP64 else "f32/f64 mixed", "data": "synthetic",
            "config": {"workload": "lmm40: 40 forwards (0-20y), 80 Euler-log steps, 10 factors, seed 7",
                       "paths": P, "products": "payer Bermudan 1y-19.5y K=4% (basis {1,S,S^2,N,N^2,SN}) + 10y10y payer swaption",
                       "parallelism": f"replicas x{ws}", "l2": "inputs larger than L2 (Brownian increments 6.7 GB)"},
            "prices": {"bermudan": res[0], "swaption": res[1]},
            "e2e": e2e, "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
            "kernel_rooflines": kernel_rooflines(stats, args.steps, P, T, N, Fk, comp_steps, len(fix),
                                                 prec == F.PRECISION_FP64, peak),
            "kernels_ms": {k: v[1] / max(args.steps, 1) for k, v in stats.items() if v[0]}}

    if rank == 0 and args.precision == "fp64" and not args.no_forms:
        line["forms"] = {"mixed": mixed_form(args, F, W, cfg, P, T, berm, swpt, res),
                         "mixed_2e22_paths": mixed_form_large(args, F, W, cfg, T, berm, swpt),
                         "greeks": greeks_form(args, F, W, cfg, P, T, berm,
                                               ms - stats["mt19937_jump_generate"][1] / max(args.steps, 1))}
        if not args.no_portfolio:
            line["forms"]["portfolio"] = portfolio_form(args, F, W, cfg, P)
        line["forms"]["random_variable"] = random_variable_form(args, F, W, cfg, P)
        line["forms"]["calibration"] = calibration_form(args, F, W)
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, parity = headline_parity(F, W, cfg, sim, berm, swpt, args.cpu_paths, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{args.cpu_paths} paths of lmm40, one pass ({dt:.1f} s)"}
        if parity is not None:
            line["parity"] = parity
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def mixed_form(args, F, W, cfg, P, T, berm, swpt, res64):
    """The mixed-precision form on the same workload: throughput and price error vs FP64."""
    import torch
    L = F.load()
    sim = W.build(cfg, paths=P, precision=F.PRECISION_MIXED)
    bm = sim.process.brownianMotion
    for _ in range(2):
        bm.setSeed(cfg["seed"])
        b = berm.getValues(sim)
        s = swpt.getValues(sim)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bm.setSeed(cfg["seed"])
        b = berm.getValues(sim)
        s = swpt.getValues(sim)
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / args.steps
    out = {"value": P * T / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
           "bermudan": b, "swaption": s,
           "bermudan_error_bp": 1e4 * (b["value"] - res64[0]["value"]),
           "bermudan_error_in_se": (b["value"] - res64[0]["value"]) / res64[0]["error"],
           "swaption_error_bp": 1e4 * (s["value"] - res64[1]["value"])}
    sim.process.close()
    bm.close()
    return out


def mixed_form_large(args, F, W, cfg, T, berm, swpt, P=1 << 22):
    """The mixed-precision form at 2^22 paths (the second size of the precision form), with
    its price error against an FP64 valuation of the same 2^22 paths."""
    import torch
    sim64 = W.build(cfg, paths=P)
    b64, s64 = berm.getValues(sim64), swpt.getValues(sim64)
    sim64.process.close()
    sim64.process.brownianMotion.close()
    sim = W.build(cfg, paths=P, precision=F.PRECISION_MIXED)
    bm = sim.process.brownianMotion
    bm.setSeed(cfg["seed"])
    b, s = berm.getValues(sim), swpt.getValues(sim)
    reps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        bm.setSeed(cfg["seed"])
        b = berm.getValues(sim)
        s = swpt.getValues(sim)
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / reps
    sim.process.close()
    bm.close()
    return {"paths": P, "value": P * T / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "bermudan": b, "swaption": s,
            "fp64": {"bermudan": b64, "swaption": s64},
            "bermudan_error_bp": 1e4 * (b["value"] - b64["value"]),
            "bermudan_error_in_se": (b["value"] - b64["value"]) / b64["error"],
            "swaption_error_bp": 1e4 * (s["value"] - s64["value"])}


def fd_check(F, W, cfg, P, berm, grads, h=1e-4):
    """Central finite differences (bump 1e-4, common random numbers, the regression re-run in
    every bumped FP64 valuation) of all 40 deltas and 20 vegas spread over the volatility grid
    at the full path count, against the mixed-precision adjoint with frozen exercise decisions
    and against the FP64 adjoint with the reference AAD's DISCRETE_DELTA boundary term: per
    Greek |adjoint - FD| within 2 % of FD or 3 standard errors of the FD (the per-path
    differences' standard error).  The re-run regression moves exercise decisions: the FD
    carries the exercise boundary's response, which frozen decisions leave out and the
    DISCRETE_DELTA sweep approximates (mixed and FP64 forms)."""
    base = W.build(cfg, paths=P)
    bm = base.process.brownianMotion
    model = base.process.model
    cov = model.covarianceModel
    obs = W.tenor_time_indices(cfg)

    def value(bump_fwd=None, bump_vol=None, d=0.0):
        f0, lam0, var0, vol0 = (model.initialForwards.copy(), cov.factorLoadings.copy(), cov.variance.copy(),
                                cov.volatility.copy())
        if bump_fwd is not None:
            model.initialForwards[bump_fwd] += d
        if bump_vol is not None:
            i, j = bump_vol
            sg = cov.volatility[i, j]
            cov.volatility[i, j] = sg + d
            cov.factorLoadings[i, j] *= (sg + d) / sg
            cov.variance[i, j] = (sg + d) * (sg + d)
        proc = F.EulerSchemeFromProcessModel(model, bm, observedTimeIndices=obs)
        r = berm.getValues(F.LIBORMonteCarloSimulationFromLIBORModel(proc), per_path=True)
        proc.close()
        model.initialForwards[:], cov.factorLoadings[:], cov.variance[:], cov.volatility[:] = f0, lam0, var0, vol0
        return r["values"]

    g = grads["mixed"]
    T, N = g["vegas"].shape
    times = base.process._keep["times"]
    tenor = base.process._keep["tenor"]
    vegas = []
    for i in range(0, T, 8):  # ten times, two forwards each: the first alive one and one further out
        alive = [j for j in range(N) if tenor[j] > times[i]]
        if alive:
            vegas += [(i, alive[0]), (i, alive[min(len(alive) - 1, len(alive) // 2 + 3)])]
    rows = []
    for kind, arg in [("delta", j) for j in range(N)] + [("vega", v) for v in vegas[:20]]:
        kw = {"bump_fwd": arg} if kind == "delta" else {"bump_vol": arg}
        diff = (value(d=h, **kw) - value(d=-h, **kw)) / (2 * h)
        rows.append((kind, arg, float(diff.mean()), float(diff.std() / np.sqrt(P))))
    base.process.close()
    bm.close()

    def compare(gr):
        scale = {"delta": float(np.max(np.abs(gr["deltas"]))), "vega": float(np.max(np.abs(gr["vegas"])))}
        out, rel = [], []
        for kind, arg, fd, se in rows:
            ad = float(gr["deltas"][arg]) if kind == "delta" else float(gr["vegas"][arg])
            tol2 = max(0.02 * abs(fd), 1e-6 * scale[kind])  # 2 %, floored for Greeks that vanish
            out.append({"greek": kind, "index": arg if kind == "delta" else list(arg), "adjoint": ad, "fd_fp64": fd,
                        "fd_se": se, "within_2pct": abs(ad - fd) <= tol2,
                        "within_2pct_or_3se": abs(ad - fd) <= max(tol2, 3 * se)})
            if abs(fd) > 1e-3 * scale[kind]:
                rel.append(abs(ad - fd) / abs(fd))
        return {"within_2pct_or_3se": sum(r["within_2pct_or_3se"] for r in out), "within_2pct": sum(r["within_2pct"] for r in out),
                "median_rel_diff": float(np.median(rel)) if rel else None, "greeks": out}

    relse = [se / abs(fd) for kind, arg, fd, se in rows if fd != 0.0]
    res = {"bump": h, "greeks_checked": len(rows), "median_rel_fd_se": float(np.median(relse)) if relse else None,
           "mixed_adjoint_frozen_exercise": compare(grads["mixed"])}
    if "mixed_dd" in grads:
        res["mixed_adjoint_discrete_delta"] = compare(grads["mixed_dd"])
    if "fp64_dd" in grads:
        res["fp64_adjoint_discrete_delta"] = compare(grads["fp64_dd"])
    return res


def greeks_form(args, F, W, cfg, P, T, berm, fp64_valuation_ms):
    """Differentiation form: Bermudan value + 40 deltas + every vega by the checkpointed adjoint,
    from scratch (increments regenerated), mixed precision and FP64, against FP64 bump-and-revalue.
    The headline uses the configured checkpoint stride of 8 steps (intermediate states replayed);
    stride 1 (every state kept in HBM) is reported beside it."""
    import torch
    out = {}
    grads = {}
    for name, prec in (("mixed", F.PRECISION_MIXED), ("fp64", F.PRECISION_FP64)):
        sim = W.build(cfg, paths=P, precision=prec)
        bm = sim.process.brownianMotion
        res = {}
        for stride in (8, 1):
            g = berm.getGradient(sim, checkpointStride=stride)
            reps = max(1, min(args.steps, 3))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                bm.setSeed(cfg["seed"])
                g = berm.getGradient(sim, checkpointStride=stride)
            torch.cuda.synchronize()
            res[stride] = (1e3 * (time.perf_counter() - t0) / reps, g)
        ms, g = res[8]
        grads[name] = g
        if name == "mixed":
            # the reference AAD's default boundary treatment on the mixed form, timed as above
            g_dd = berm.getGradient(sim, checkpointStride=8, diracDeltaApproximationMethod="DISCRETE_DELTA")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                bm.setSeed(cfg["seed"])
                g_dd = berm.getGradient(sim, checkpointStride=8, diracDeltaApproximationMethod="DISCRETE_DELTA")
            torch.cuda.synchronize()
            out["mixed_discrete_delta_ms"] = 1e3 * (time.perf_counter() - t0) / reps
            grads["mixed_dd"] = g_dd
        if name == "fp64":
            # the reference AAD's default treatment of the exercise boundary (DISCRETE_DELTA,
            # width 0.05 standard deviations): the FP64 form's sweep over the backward induction
            t0 = time.perf_counter()
            grads["fp64_dd"] = berm.getGradient(sim, checkpointStride=1, diracDeltaApproximationMethod="DISCRETE_DELTA")
            torch.cuda.synchronize()
            out["fp64_discrete_delta_ms"] = 1e3 * (time.perf_counter() - t0)
        out[name] = {"ms_price_and_greeks": ms, "checkpoint_stride": 8, "ms_price_and_greeks_stride1": res[1][0],
                     "value": g["value"], "error": g["error"],
                     "num_deltas": int(g["deltas"].size), "num_vegas": int(np.count_nonzero(g["vegas"]))}
        sim.process.close()
        bm.close()
    g32, g64 = grads["mixed"], grads["fp64"]
    nv = int(np.count_nonzero(g64["vegas"]))
    # central differences of every delta and vega with common random numbers: 2 revaluations each,
    # the Brownian increments reused (the measured FP64 valuation minus increment generation)
    reval_ms = fp64_valuation_ms
    bump_ms = (2 * (g64["deltas"].size + nv) + 1) * reval_ms
    out["fp64_bump_and_revalue_ms_estimate"] = bump_ms
    out["speedup_mixed_adjoint_vs_fp64_bump_and_revalue"] = bump_ms / out["mixed"]["ms_price_and_greeks"]
    out["mixed_vs_fp64"] = {
        "value_bp": 1e4 * (g32["value"] - g64["value"]),
        "max_abs_delta_diff_bp_per_bp": float(np.max(np.abs(g32["deltas"] - g64["deltas"]))),
        "max_abs_vega_diff_bp_per_vol_pt": float(1e4 * 1e-2 * np.max(np.abs(g32["vegas"] - g64["vegas"]))),
        "max_rel_delta_diff": float(np.max(np.abs(g32["deltas"] - g64["deltas"])) / np.max(np.abs(g64["deltas"]))),
        "max_rel_vega_diff": float(np.max(np.abs(g32["vegas"] - g64["vegas"])) / np.max(np.abs(g64["vegas"]))),
    }
    d32, d64 = grads["mixed_dd"], grads["fp64_dd"]
    out["mixed_vs_fp64_discrete_delta"] = {
        "value_bp": 1e4 * (d32["value"] - d64["value"]),
        "max_abs_delta_diff_bp_per_bp": float(np.max(np.abs(d32["deltas"] - d64["deltas"]))),
        "max_abs_vega_diff_bp_per_vol_pt": float(1e4 * 1e-2 * np.max(np.abs(d32["vegas"] - d64["vegas"]))),
        "max_rel_delta_diff": float(np.max(np.abs(d32["deltas"] - d64["deltas"])) / np.max(np.abs(d64["deltas"]))),
        "max_rel_vega_diff": float(np.max(np.abs(d32["vegas"] - d64["vegas"])) / np.max(np.abs(d64["vegas"]))),
    }
    out["fd_check"] = fd_check(F, W, cfg, P, berm, grads)
    out["note"] = ("bump-and-revalue estimate = (2 x (deltas + nonzero vegas) + 1) x the measured FP64 valuation; "
                   "delta differences are price bp per 1 bp of forward, vega differences price bp per 1 vol point")
    return out


def random_variable_form(args, F, W, cfg, P, n=1 << 26):
    """The device RandomVariable layer (include/lmm_rv.h): streaming elementwise operations
    and a reduction at n = 2^26 realizations (512 MB per operand, above L2), against the
    measured HBM copy bandwidth; and a strip of 40 caplets written against the
    RandomVariable API on the FP64 lmm40 simulation (Caplet.getValue's operations)."""
    from finmath_gb300.randomvariable import RandomVariableGPU as RV
    rng = np.random.default_rng(7)
    x, y, z = (RV.from_array(0.0, rng.random(n)) for _ in range(3))
    hbm, _ = _measured_hbm_gbs()

    import torch
    h = ctypes.c_void_p()
    F.load().lmm_rv_stream(ctypes.byref(h))
    stream = torch.cuda.ExternalStream(h.value)

    def timed(fn, nbytes, reps=10):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3 / reps
        return {"ms": sec * 1e3, "gbs": nbytes / sec / 1e9, "hbm_frac": nbytes / sec / 1e9 / hbm}

    out = {"n": n, "unit": "GB/s of algorithmic bytes (8 B per operand read and per value written)",
           "mult": timed(lambda: x.mult(y).close(), 24 * n),
           "add_product": timed(lambda: x.addProduct(y, z).close(), 32 * n),
           "discount": timed(lambda: x.discount(y, 0.5).close(), 24 * n),
           "exp": timed(lambda: x.exp().close(), 16 * n),
           "average": timed(lambda: x.getAverage(), 8 * n),
           "note": "CUDA events on the library stream over 10 operations (each allocates its result from "
                   "the stream-ordered pool and frees it); discount's correctly rounded division, exp and "
                   "the compensated average are bound by the GPU's FP64 pipe, not HBM"}
    for r in (x, y, z):
        r.close()
    sim = W.build(cfg, paths=P)
    period, w = cfg["period"], 1.0 / P
    N0 = sim.getNumeraireRandomVariable(0.0)  # simulates the paths (lazily, as the reference)
    N0.getAverage()
    t0 = time.perf_counter()
    total = 0.0
    for j in range(1, 40):
        t = int(round(j * period / cfg["dt"]))
        v = sim.getLIBORRandomVariable(t, j).sub(0.04).floor(0.0).mult(period)
        v = v.div(sim.getNumeraireRandomVariable((j + 1) * period)).mult(w).mult(N0).div(w)
        total += v.getAverage()
    out["caplet_strip"] = {"caplets": 39, "paths": P, "ms": 1e3 * (time.perf_counter() - t0), "value_sum": total,
                           "note": "39 caplets 1y-20y K=4% through getLIBOR/getNumeraire random variables: "
                                   "7 elementwise operations and one compensated average each, on the simulated paths"}
    N0.close()
    sim.process.close()
    sim.process.brownianMotion.close()
    return out


def calibration_form(args, F, W, paths=20000, iterations=20):
    """Monte Carlo calibration form: the abcd volatility of the lmm20 model fitted by
    Levenberg-Marquardt to seven swaption prices of another surface (moved by up to 3 %, so no
    exact fit exists), every objective evaluation a new Euler process on one resident
    Brownian motion of `paths` paths and the fused swaption kernel; objective evaluations per
    second (one evaluation prices every calibration product)."""
    import torch
    cfg = W.LMM20
    td = F.TimeDiscretizationFromArray(0.0, int(round(cfg["T_end"] / cfg["dt"])), cfg["dt"])
    tenor = F.TimeDiscretizationFromArray(0.0, int(round(cfg["tenor_end"] / cfg["period"])), cfg["period"])
    curve = F.ForwardCurveInterpolation.createForwardCurveFromForwards("forwardCurve", cfg["curve_nodes"],
                                                                       cfg["curve_values"], cfg["period"])

    def covariance(abcd):
        vol = F.LIBORVolatilityModelFourParameterExponentialForm(td, tenor, *abcd, True)
        corr = F.LIBORCorrelationModelExponentialDecay(td, tenor, cfg["F"], cfg["corr_decay"], False)
        return F.LIBORCovarianceModelFromVolatilityAndCorrelation(td, tenor, vol, corr)

    model = F.LIBORMarketModelFromCovarianceModel.of(tenor, None, curve, F.DiscountCurveFromForwardCurve(curve), None,
                                                     covariance(cfg["abcd"]), None, {})
    bm = F.BrownianMotionFromMersenneRandomNumbers(td, cfg["F"], paths, 31415)
    specs = []
    for ex, n in ((1.0, 4), (2.0, 6), (3.0, 4), (5.0, 8), (7.0, 4), (2.0, 12), (4.0, 10)):
        fix = [ex + 0.5 * i for i in range(n)]
        specs.append((ex, fix, [x + 0.5 for x in fix], 0.05))
    proc = F.EulerSchemeFromProcessModel(model, bm)
    targets = [F.Swaption(*sp).getValue(F.LIBORMonteCarloSimulationFromLIBORModel(proc)) * (1.0 + 0.03 * np.sin(3.0 * i))
               for i, sp in enumerate(specs)]
    proc.close()
    items = [F.CalibrationProduct(f"s{i}", F.Swaption(*sp), t) for i, (sp, t) in enumerate(zip(specs, targets))]
    params = {"brownianMotion": bm, "maxIterations": iterations, "accuracy": 0.0}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    calibrated = covariance((0.25, 0.15, 0.2, 0.12)).getCloneCalibrated(model, items, params)
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    opt = params["optimizer"]
    bm.close()
    count = [opt.evaluations]
    return {"paths": paths, "products": len(specs), "parameters": 4, "objective_evaluations": count[0],
            "seconds": sec, "evaluations_per_second": count[0] / sec, "iterations": opt.getIterations(),
            "rms_error": opt.getRootMeanSquaredError(), "parameters_calibrated": list(calibrated.getParameter()),
            "note": "each evaluation builds the trial covariance model and Euler process on the host; the "
                    "Jacobian's four columns and every product are simulated and priced in one batch "
                    "(lmm_swaption_values_batch: no host round trip between them, one copy back per process)"}


def portfolio_form(args, F, W, cfg, P):
    """Batching form: 256 Bermudan swaptions (seeded schedules, strikes, payer/receiver) with
    values, deltas and vegas on the shared 2^20-path mixed-precision simulation, one graph
    launch; knobs from the autotuner (cached per GPU and problem shape)."""
    import torch
    prods = W.portfolio_products(cfg, n=256, seed=20261203)
    sim = W.build(cfg, paths=P, precision=F.PRECISION_MIXED)
    name = torch.cuda.get_device_name()
    T = int(round(cfg["T_end"] / cfg["dt"]))
    key = F.autotune.key(name, P, T, 40, cfg["F"], F.PRECISION_MIXED)
    t0 = time.perf_counter()
    knobs = F.autotune.tune(sim, prods, key, subset=16)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    pf = F.Portfolio(sim, prods, True, knobs["checkpointStride"], knobs["concurrency"], knobs["adjointThreads"],
                     knobs["gramBlocks"])
    create_s = time.perf_counter() - t0
    pf.run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = pf.run()
    wall_ms = 1e3 * (time.perf_counter() - t0)
    lat = np.sort(out["latency_ms"])
    res = {"products": len(prods), "paths": P, "precision": "mixed", "knobs": knobs,
           "device_ms": out["total_ms"], "wall_ms": wall_ms, "latency_p50_ms": float(np.percentile(lat, 50)),
           "latency_p99_ms": float(np.percentile(lat, 99)), "per_product_ms": out["total_ms"] / len(prods),
           "greeks_per_product": 40 + 1560, "graph_record_s": create_s, "autotune_s": tune_s,
           "value_sum": float(np.sum(out["values"]))}
    pf.close()
    sim.process.close()
    sim.process.brownianMotion.close()
    return res


def run_case(args):
    """A named valuation case for profiling single kernels under ncu (no JSON bench line):
    each repetition regenerates the increments (seed + repetition) and values the
    workload's Bermudan swaption; 'greeks' adds its adjoint deltas and vegas; 'portfolio'
    runs a 16-product portfolio with Greeks through one graph launch.  Kernel counts and
    (with --timing) CUDA-event times exclude the first repetition."""
    import finmath_gb300 as F
    from finmath_gb300 import workloads as W
    L = F.load()
    if args.timing:
        L.lmm_stats_enable_timing(1)
    cfg = W.WORKLOADS[args.workload]
    prec = F.PRECISION_MIXED if args.precision == "mixed" else F.PRECISION_FP64
    sim = W.build(cfg, paths=args.paths, precision=prec)
    fix, plen, pay, K = W.bermudan_schedule(cfg)
    berm = F.BermudanSwaption(np.ones(len(fix)), fix, plen, pay, 1.0, K, True, "swaprate")
    out = None
    if args.case == "portfolio":
        pf = F.Portfolio(sim, W.portfolio_products(cfg, n=16, seed=20261203), True, args.stride, 4, 128, 0)
        for r in range(args.repeat):
            out = pf.run()["total_ms"]
            if r == 0:
                L.lmm_stats_reset()
        pf.close()
    else:
        for r in range(args.repeat):
            sim.process.brownianMotion.setSeed(cfg["seed"] + r)
            if args.case == "greeks":
                out = berm.getGradient(sim, checkpointStride=args.stride)["value"]
            else:
                out = berm.getValue(sim)
            if r == 0:
                L.lmm_stats_reset()
    print(json.dumps({"case": args.case, "precision": args.precision, "paths": args.paths, "last": out,
                      "kernels": F.kernel_stats()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--paths", type=int, default=1 << 20)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--cpu-paths", type=int, default=0,
                    help="CPU sample paths (default: the bench's own path count for the baseline and parity leg, "
                         "2^18 per reference step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--no-portfolio", action="store_true")
    ap.add_argument("--case", choices=["valuation", "greeks", "portfolio"], default=None,
                    help="run one named valuation case for profiling instead of the bench")
    ap.add_argument("--repeat", type=int, default=3, help="--case: repetitions")
    ap.add_argument("--workload", default="lmm40", help="--case: workload name")
    ap.add_argument("--stride", type=int, default=1, help="--case: checkpoint stride")
    ap.add_argument("--timing", action="store_true", help="--case: CUDA-event time per kernel family")
    args = ap.parse_args()
    if args.case:
        if args.paths == (1 << 20) and "--paths" not in sys.argv:
            args.paths = 65536
        run_case(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.cpu_paths <= 0:
        args.cpu_paths = (1 << 18) if args.impl == "reference" else args.paths
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
