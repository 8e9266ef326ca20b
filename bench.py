#!/usr/bin/env python3
"""Benchmark of the GB300 FUNWAVE-TVD SSP-RK3 step on the 2048 x 2048
elliptic-shoal / directional-JONSWAP workload.

Metric: cell-steps/s (interior cells x whole SSP-RK3 steps per second) on
one GB300, mixed-FP32 (float fields, FP64 tridiagonal u/v recovery and
total-depth tests) as ``value``, with the all-FP64 path and the eta error of
the mixed path against it beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One process per GPU (torchrun for N > 1): every rank advances its own
replica of the workload (runs are independent; no collective on the data
path), the step time is the maximum over ranks and value sums all ranks'
cell-steps.  The reference arm times the CPU restatement of the reference's
algorithm (the Fortran reference has no compiler here or on the GPU host)
on all host cores.
"""
import argparse
import json
import os

# more hardware queues for the ensemble's concurrent streams (read at the
# first CUDA call of the process)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

METRIC = "cell-steps/s (1 GB300) mixed-FP32 vs FP64 at stated eta error; ensemble runs/hr"
UNIT = "cell-steps/s"
WORKLOAD = ("2048x2048 1:50 slope + elliptic shoal, JON_2D Hs=1 m Tp=10 s 50x30 cos^2s, "
            "dx=2 m, walls, west sponge (synthetic)")

# Algorithmic bytes per launch unit of each kernel: every distinct array the
# kernel must read once plus every array it must write once (T = bytes of a
# bulk field element, masks 1 byte, tridiagonal right-hand sides 8 bytes).
# Unit: one cell (one face for flux_x / flux_y).
KERNEL_BYTES = {
    "disp_a": lambda T: 13 * T + 1,       # U V Eta Depth P Q + MASK9 -> A B C E ETAx ETAy ETAT
    "disp_b": lambda T: 19 * T + 1,       # A B C E U V U0 V0 Eta Depth ETAx ETAy ETAT + MASK9 -> U4 V4 U1p V1p Udisp Vdisp
    "flux_x": lambda T: 11 * T + 2,       # U V HU HV Eta U4 V4 Depthx + MASK MASK9 -> P Fx Gx
    "flux_y": lambda T: 11 * T + 2,
    "update": lambda T: 32 * T + 2 + 16,  # 28 fields + MASK MASK9 -> Eta Ubar Vbar H + rhs_x rhs_y
    # mixed: rhs_x + the ten float factor arrays of the constant factorised
    # matrix (1/diag, sweep A, L*r, c', the two spike columns, a and c as
    # float pairs for the compensated residual) -> U; FP64: Depth MASK9
    # MASK rhs_x -> U
    "tri_x": lambda T: 2 * T + (40 if T == 4 else 10),
    "tri_y": lambda T: 2 * T + (40 if T == 4 else 10),
    "post": lambda T: 7 * T + 1 + 6 * T,  # U V H Ubar Vbar HU HV + MASK -> U V HU HV Ubar Vbar
    # the fused GET_Eta_U_V_HU_HV tail + UPDATE_MASK + BREAKING (parallel part):
    # U V H ETAT AGE Depth Eta + MASK MASK_STRUC MASK9 -> U V HU HV AGEn nu + MASKn MASK9
    "post_mask_break": lambda T: 13 * T + 5,
    "mask": lambda T: 4 * T + 4 + 2 * T,  # Eta Depth Depthx Depthy + MASK MASK_STRUC -> MASKn MASK9 Depthx Depthy
    "break_a": lambda T: 8 * T + 2 * T,   # H ETAx ETAy ETAT Depth Eta AGE nu -> AGEn nu
    "maskmul": lambda T: 6 * T + 1 + 5 * T,
    "begin": lambda T: 8 * T + 1 + 9 * T,
}
# DRAM bytes per unit (dram__bytes_read.sum + dram__bytes_write.sum of one
# ncu capture of the 2048 x 2048 mixed step, per launch / units; the tri_y
# figure sums the partitioned y-solve kernels of one stage), taken with
# the launch shapes pinned to the autotuner's choice
TRAFFIC_PER_UNIT_MIXED = {
    "tri_x": 49.4, "update": 137.4, "flux_x": 41.0, "flux_y": 41.6, "disp_b": 72.6, "disp_a": 42.7,
    "maskmul": 30.8, "tri_y": 95.2, "post_mask_break": 42.5,
}
# kernel launches per stage (tri_* count the partitioned solve as one)
PER_STAGE = ["disp_a", "disp_b", "flux_x", "flux_y", "update", "tri_x", "tri_y", "post_mask_break", "post",
             "mask", "break_a", "maskmul"]
# whole-step algorithmic bytes per cell-step: the cross-stage state each of
# the three stages must read and write once (61 reals + 6 mask bytes)
STEP_BYTES = {"fp64": 61 * 8 + 6, "mixed": 61 * 4 + 6}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                out = self.p.communicate(timeout=5)[0]
            except subprocess.TimeoutExpired:
                self.p.kill()
                out = self.p.communicate()[0]
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cuda_timer(solver):
    import torch
    ext = torch.cuda.ExternalStream(solver.stream())
    return ext, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def barrier(pg):
    if pg:
        import torch.distributed as dist
        dist.barrier()


def aggregate_rate(cells, steps, ws, ms_max):
    """Whole-job cell-steps/s of ws replicas that each advanced `cells`
    cells by `steps` steps, over the slowest rank's time (ms)."""
    return cells * steps * ws / (ms_max * 1e-3)


def max_over_ranks(v, pg):
    if not pg:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_precision(fw, params, depth, phases, precision, K, W, local, pg, autotune=True):
    import torch
    s = fw.Solver(params, precision=precision, device=local)
    s.init(depth, phases=phases)
    t0 = time.perf_counter()
    if isinstance(autotune, dict):
        s.set_tuning({k: tuple(v) if isinstance(v, list) else v for k, v in autotune.items()})
        tuning, tune_s = s.tuning(), 0.0
    else:
        tuning = s.autotune() if autotune else s.tuning()
        tune_s = time.perf_counter() - t0 if autotune else 0.0
    n0 = s.launch_count()
    s.step(2)                       # captures the two-step graph
    per_step = (s.launch_count() - n0) // 2
    if W > 2:
        s.step(W - 2)
    ext, e0, e1 = cuda_timer(s)
    barrier(pg)
    s.sync()
    with ClockSampler(local) as clk:
        e0.record(ext)
        st = s.step(K, check=False)
        e1.record(ext)
        e1.synchronize()
    s.sync()
    barrier(pg)
    ms = e0.elapsed_time(e1)
    return s, {"ms": ms, "status": st, "launches_per_step": per_step, "clocks": clk.summary(),
               "tuning": tuning, "tune_s": tune_s}


def kernel_profile(s, T, cells, faces_x, faces_y, hbm):
    """Average duration of each kernel of a stage (CUDA events on the
    library stream) and its achieved algorithmic bandwidth."""
    out = {}
    for name in PER_STAGE:
        try:
            ms = s.time_kernel(name, nrep=10)
        except Exception:
            continue
        unit = faces_x if name == "flux_x" else faces_y if name == "flux_y" else cells
        b = KERNEL_BYTES[name](T) * unit
        out[name] = {"ms": ms, "bytes": b, "gbs": b / (ms * 1e-3) / 1e9, "frac": b / (ms * 1e-3) / 1e9 / hbm}
    return out


def e2e_run(fw, s, K, f32=True):
    """Per step through the C ABI with pinned host buffers: upload Eta, U,
    V, Ubar, Vbar (one fw_set_fields_f32, or fw_set_fields with f32=False),
    one fw_step, read back Eta, U, V (one fw_get_fields_f32 / fw_get_fields).
    Float host arrays are those of the reference's default single-precision
    build (REAL(SP) = 4 bytes); double ones those of its -DDOUBLE_PRECISION
    build."""
    import numpy as np
    import torch
    import ctypes
    dt_t, dt_n = (torch.float32, 4) if f32 else (torch.float64, 8)
    bufs = {}
    for n in ("Eta", "U", "V", "Ubar", "Vbar"):
        t = torch.empty((s.Nloc, s.Mloc), dtype=dt_t, pin_memory=True)
        a = t.numpy().T  # Fortran-ordered (Mloc, Nloc) view of pinned memory
        a[...] = s.get(n)
        bufs[n] = (t, a)
    L = s.L
    setf, getf = (L.fw_set_fields_f32, L.fw_get_fields_f32) if f32 else (L.fw_set_fields, L.fw_get_fields)
    up, down = ("Eta", "U", "V", "Ubar", "Vbar"), ("Eta", "U", "V")
    up_n = (ctypes.c_char_p * 5)(*[n.encode() for n in up])
    up_p = (ctypes.c_void_p * 5)(*[bufs[n][1].ctypes.data for n in up])
    down_n = (ctypes.c_char_p * 3)(*[n.encode() for n in down])
    down_p = (ctypes.c_void_p * 3)(*[bufs[n][1].ctypes.data for n in down])
    s.sync()
    t0 = time.perf_counter()
    for _ in range(K):
        rc = setf(s.ctx, 5, up_n, up_p)
        assert rc == 0
        s.step(1, check=False)
        rc = getf(s.ctx, 3, down_n, down_p)
        assert rc == 0
    s.sync()
    dt = time.perf_counter() - t0
    nb = s.Mloc * s.Nloc * dt_n
    return dt, 5 * nb, 3 * nb


def link_rates(nbytes, reps=10):
    """Pinned host <-> device copy rates (GB/s) for planes of nbytes, the
    bound of the end-to-end leg's transfers."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, f in (("h2d", lambda: d.copy_(h, non_blocking=True)), ("d2h", lambda: h.copy_(d, non_blocking=True))):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            f()
        torch.cuda.synchronize()
        out[name] = nbytes * reps / (time.perf_counter() - t) / 1e9
    del h, d
    return out


def ensemble_bench(fw, pg, ws, n=512, K=100, W=2, run_seconds=300.0, autotune=True):
    """The 512-run ensemble (planar beaches of uneven size, slope, depth and
    JONSWAP forcing; 1.5e8 cells in all): every member steps concurrently,
    as one parent CUDA graph per two steps (fw_ensemble_run; the headline)
    and round robin on the members' streams (fw_ensemble_step), on the same
    members.  cell-steps/s over K steps after W warm-up steps (host wall
    clock around the call, which waits for every run); runs/hr extrapolates
    to run_seconds of simulated time per run, with each run's step count
    from its own DT and the measured cell-step rate."""
    members = fw.cases.ensemble_members(n, seed=2024)
    t0 = time.perf_counter()
    ens = fw.Ensemble(members, precision="MIXED", autotune=autotune, single_launch=True)
    t_init = time.perf_counter() - t0
    t0 = time.perf_counter()
    ens.step(W, check=False)  # builds the parent graph
    t_graph = time.perf_counter() - t0
    barrier(pg)
    t0 = time.perf_counter()
    st = ens.step(K, check=False)
    wall = max_over_ranks(time.perf_counter() - t0, pg)
    barrier(pg)
    handle, ens.handle = ens.handle, None  # the same members, round robin
    ens.step(W, check=False)
    barrier(pg)
    t0 = time.perf_counter()
    ens.step(K, check=False)
    wall_rr = max_over_ranks(time.perf_counter() - t0, pg)
    barrier(pg)
    ens.handle = handle
    cells = [p["Mglob"] * p["Nglob"] for p, _, _ in members]
    dts = [s.scalar("DT") for s in ens.solvers]
    ens.close()
    rate = sum(cells) * K * ws / wall
    rate_rr = sum(cells) * K * ws / wall_rr
    work = sum(c * run_seconds / dt for c, dt in zip(cells, dts)) / n
    return {"metric": "ensemble runs/hr", "value": 3600.0 * rate / work, "unit": "runs/hr",
            "cell_steps_per_s": rate, "runs": n * ws, "cells_total": sum(cells) * ws,
            "grid_cells_range": [min(cells), max(cells)], "steps_timed": K, "warmup": W,
            "wall_s": wall, "init_s": t_init, "graph_build_s": t_graph,
            "round_robin": {"value": 3600.0 * rate_rr / work, "cell_steps_per_s": rate_rr, "wall_s": wall_rr},
            "statuses_nonzero": sum(1 for v in st if v), "run_seconds": run_seconds,
            "how": "each run is a context with its own arena and autotuned launch shapes; fw_ensemble_run "
                   "advances all runs by two steps per launch of one parent CUDA graph whose children are the "
                   "runs' two-step graphs (round_robin: fw_ensemble_step, the runs' own graphs round robin on "
                   "their streams); runs/hr extrapolates the measured cell-step rate to %g s of simulated time "
                   "per run" % run_seconds}


def c1_full_run(fw):
    """The 250 x 500 planar beach (WK_REG H = 0.3 m, T = 6 s, periodic in y,
    west sponge, breaking on) through its whole 300 s of model time in mixed
    precision and in FP64: the stated eta error of the mixed path over a full
    run, with both wall times."""
    import numpy as np
    params, depth, _ = fw.cases.planar_beach()
    params = fw.with_defaults(params)
    t_end = float(params["TOTAL_TIME"])
    out = {}
    for prec in ("MIXED", "FP64"):
        s = fw.Solver(params, precision=prec)
        s.init(depth)
        n, t0 = 0, time.perf_counter()
        while s.scalar("TIME") < t_end:
            s.step(50)
            n += 50
        out[prec] = {"Eta": s.get("Eta")[3:-3, 3:-3], "MASK": s.get("MASK")[3:-3, 3:-3],
                     "TIME": s.scalar("TIME"), "steps": n, "wall_s": time.perf_counter() - t0}
        s.close()
    m, d = out["MIXED"], out["FP64"]
    wet = (m["MASK"] > 0) & (d["MASK"] > 0)
    diff = (m["Eta"] - d["Eta"])[wet]
    return {"config": "250x500 planar beach, WK_REG H=0.3 m T=6 s, periodic y, 300 s", "t_end_s": t_end,
            "time_mixed_s": m["TIME"], "time_fp64_s": d["TIME"], "steps": d["steps"],
            "eta_rms_mixed_vs_fp64_m": float(np.sqrt(np.mean(diff ** 2))),
            "eta_max_abs_mixed_vs_fp64_m": float(np.abs(diff).max()),
            "eta_rms_signal_m": float(np.sqrt(np.mean(d["Eta"][wet] ** 2))),
            "mask_mismatch_cells": int((m["MASK"] != d["MASK"]).sum()),
            "wall_s": {"MIXED": m["wall_s"], "FP64": d["wall_s"]}}


def precision_report(fw, size=4096, t_end=33.0, t_steady=12.0, t_mean=20.0):
    """The 4096 x 4096 barred beach with rip channels (1:40, bar 1.5 m high
    80 m offshore, JONSWAP Hs = 1.5 m, Tp = 10 s), run to t_end s in mixed
    precision and in FP64: eta RMS over cells wet in both, maximum run-up,
    the time-mean current (Umean, Vmean over [t_steady, t_steady + t_mean])
    and MASK mismatches of mixed against FP64, with both step rates."""
    import numpy as np
    params, depth, phases, rips = fw.cases.barred_beach(size, size, 1.0, seed=2024)
    params = fw.with_defaults(params)
    params.update({"OUT_Hmax": True, "STEADY_TIME": t_steady, "T_INTV_mean": t_mean})
    out = {}
    # FP64_F32DEPTH: FP64 from the depth rounded to float, a change of the
    # inputs at float rounding; its distance from FP64 is what rounding
    # alone grows to by t_end through the run's threshold events (breaking
    # onsets, wet/dry), the floor for any path that stores floats
    for prec in ("MIXED", "FP64", "FP64_F32DEPTH"):
        s = fw.Solver(params, precision=prec[:4] if prec.startswith("FP64") else prec)
        s.init(depth.astype(np.float32).astype(np.float64) if prec == "FP64_F32DEPTH" else depth, phases=phases)
        n = 0
        ext, e0, e1 = cuda_timer(s)
        s.sync()
        e0.record(ext)
        while s.scalar("TIME") < t_end:
            s.step(20)
            n += 20
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec] = {k: s.get(k)[3:-3, 3:-3] for k in ("Eta", "U", "V", "MASK", "HeightMax", "Umean", "Vmean", "AGE")}
        out[prec]["TIME"] = s.scalar("TIME")
        out[prec]["steps"] = n
        out[prec]["rate"] = size * size * n / (ms * 1e-3)
        s.close()
    m, d, r = out["MIXED"], out["FP64"], out["FP64_F32DEPTH"]
    wet = (m["MASK"] > 0) & (d["MASK"] > 0)
    wet_r = (r["MASK"] > 0) & (d["MASK"] > 0)
    floor = {"eta_rms_m": float(np.sqrt(np.mean((r["Eta"] - d["Eta"])[wet_r] ** 2))),
             "eta_max_abs_m": float(np.abs(r["Eta"] - d["Eta"])[wet_r].max()),
             "mask_mismatch_cells": int((r["MASK"] != d["MASK"]).sum()), "steps": r["steps"]}
    cur_d = np.sqrt(d["Umean"] ** 2 + d["Vmean"] ** 2)
    du = np.sqrt((m["Umean"] - d["Umean"]) ** 2 + (m["Vmean"] - d["Vmean"]) ** 2)
    ru_m, ru_d = fw.max_runup(np.pad(m["HeightMax"], 3), depth), fw.max_runup(np.pad(d["HeightMax"], 3), depth)
    # where the difference sits: cells breaking in either run (AGE > 0),
    # widened by 4 cells on every side, against the rest of the wet cells
    brk = (m["AGE"] > 0) | (d["AGE"] > 0)
    zone = brk.copy()
    for _ in range(4):
        z = zone.copy()
        z[1:, :] |= zone[:-1, :]
        z[:-1, :] |= zone[1:, :]
        z[:, 1:] |= zone[:, :-1]
        z[:, :-1] |= zone[:, 1:]
        zone = z
    de2 = ((m["Eta"] - d["Eta"]) ** 2) * wet
    quiet = wet & ~zone
    ad = np.abs(m["Eta"] - d["Eta"])[wet]
    return {
        "metric": "mixed vs FP64 on the 4096x4096 barred beach", "grid": [size, size], "dx_m": 1.0,
        "rip_channels_y_m": rips, "t_end_s": t_end, "time_mixed_s": m["TIME"], "time_fp64_s": d["TIME"],
        "steps_mixed": m["steps"], "steps_fp64": d["steps"],
        "eta_rms_m": float(np.sqrt(np.mean((m["Eta"] - d["Eta"])[wet] ** 2))),
        "eta_max_abs_m": float(np.abs(m["Eta"] - d["Eta"])[wet].max()),
        "eta_rms_signal_m": float(np.sqrt(np.mean(d["Eta"][wet] ** 2))),
        "eta_rms_outside_breaking_m": float(np.sqrt(np.sum(de2[quiet]) / max(1, quiet.sum()))),
        "breaking_zone_cells": int((wet & zone).sum()), "wet_cells": int(wet.sum()),
        "share_of_squared_error_in_breaking_zone": float(np.sum(de2[zone]) / max(np.sum(de2), 1e-300)),
        "eta_abs_diff_percentiles_m": {q: float(np.percentile(ad, float(q))) for q in ("50", "99", "99.9", "99.99")},
        "max_runup_mixed_m": ru_m, "max_runup_fp64_m": ru_d,
        "mean_current_rms_error_m_s": float(np.sqrt(np.mean(du[wet] ** 2))),
        "mean_current_rms_fp64_m_s": float(np.sqrt(np.mean(cur_d[wet] ** 2))),
        "mask_mismatch_cells": int(np.sum(m["MASK"] != d["MASK"])),
        "cell_steps_per_s_mixed": m["rate"], "cell_steps_per_s_fp64": d["rate"],
        "speedup_mixed_over_fp64": m["rate"] / d["rate"],
        "rounding_floor_fp64_from_float_depth": floor,
    }


def fp64_only(fw, size, K, W):
    """The FP64 path alone on the size x size shoal workload: W warm-up
    steps, then K steps timed with CUDA events on the library's stream."""
    import torch
    torch.cuda.set_device(0)
    params, depth, phases = fw.cases.shoal_jonswap(Mglob=size, Nglob=size, seed=2024)
    s = fw.Solver(fw.with_defaults(params), precision="FP64")
    s.init(depth, phases=phases)
    s.step(W)
    ext, e0, e1 = cuda_timer(s)
    s.sync()
    e0.record(ext)
    st = s.step(K, check=False)
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(K, 1)
    s.close()
    return {"metric": "FP64 cell-steps/s", "value": size * size / (ms * 1e-3), "unit": "cell-steps/s",
            "ms_per_step": ms, "steps": K, "warmup": W, "grid": [size, size], "status": st}


def net_report(fw, size=1024, reps=20):
    """The correction network alone, on a size x size coarse grid: the
    forward pass (packing, four tcgen05 convolutions) and one training
    iteration (forward, loss, backward with tcgen05 data and weight
    gradients, Adam) on a batch of 8 tiles of 128 x 128 and on a batch of 8
    whole size x size grids (the full-size training's batch), CUDA events on
    the current stream after 3 warm-up calls.  Tensor work:
    2 x 9 x (16*32 + 32*32 + 32*32 + 32*16) MACs a pixel in the forward pass
    (channels as padded for the tensor cores)."""
    import torch
    torch.cuda.set_device(0)
    net = fw.learned.Net(seed=1)
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn((1, size, size, 5), device="cuda", generator=g)
    for _ in range(3):
        net.forward(x)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        net.forward(x)
    e1.record()
    e1.synchronize()
    ms_fwd = e0.elapsed_time(e1) / reps
    def train_ms(hw):
        xb = torch.randn((8, hw, hw, 5), device="cuda", generator=g)
        tb = torch.randn((8, hw, hw, 3), device="cuda", generator=g)
        wb = torch.ones((8, hw, hw), device="cuda")
        for _ in range(3):
            net.loss_grad(xb, tb, wb)
            net.adam(1e-4)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            net.loss_grad(xb, tb, wb)
            net.adam(1e-4)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    ms_iter = train_ms(128)
    ms_iter_full = train_ms(size)
    net.close()
    macs = 9 * (16 * 32 + 32 * 32 + 32 * 32 + 32 * 16)
    return {"metric": "correction network", "grid": [size, size], "ms_forward": ms_fwd,
            "forward_tflops_padded": 2.0 * macs * size * size / (ms_fwd * 1e-3) / 1e12,
            "ms_train_iteration_batch8_128x128": ms_iter,
            "ms_train_iteration_batch8_%dx%d" % (size, size): ms_iter_full}


def learned_full_report(fw, n_traj=10, steps_per_traj=200, iters=4000, eval_coarse_steps=2000, batch=8,
                        n_train=3, bands=(1, 2)):
    """The learned coarse-grid correction at the configuration's sizes: fine
    runs on 2048 x 2048 cells at dx = 1 m, their coarse twins on 1024 x 1024
    at dx = 2 m; n_traj seeded trajectories (planar, barred and shoal
    bathymetries, JONSWAP Hs 0.5-2 m) of steps_per_traj coarse steps give
    n_traj x steps_per_traj pairs (2000 by default), all made by the solver
    and kept on the GPU; n_train trainings with Adam, each from its own
    initial weights and batch order; then on held-out seeds, per training,
    the one-step error ratio, the eta RMS against the restricted fine run
    after 500 and after eval_coarse_steps coarse steps, and the maximum
    run-up of fine, plain coarse and corrected coarse runs, for each shore
    band of the correction in bands (fw_net_set_shore_band)."""
    import numpy as np
    import torch
    L = fw.learned
    avail_gb = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE") / 1e9
    if avail_gb < 64:
        return {"skipped": "only %.0f GB of host memory available (64 needed)" % avail_gb}

    def dt_for(p, h):
        return round(0.35 * p["DX"] / np.sqrt(9.81 * max(h, 1.0)), 4)

    def hs(seed):
        return float(0.5 + 1.5 * ((seed * 37) % 10) / 9.0)

    def barred(seed):
        p, d, ph, _ = fw.cases.barred_beach(2048, 2048, 1.0, seed=seed, wk_from_shore=300.0, nfreq=16, ntheta=4,
                                            shore_from_east=120.0, Hmo=hs(seed), Sponge_west_width=60.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    def planar(seed):
        p, d, ph = fw.cases.ensemble_members(1, seed=seed, nfreq=16, ntheta=4,
                                             cells_range=(2048 * 2048, 2048 * 2048))[0]
        p["Hmo"] = min(p["Hmo"], 2.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    def shoal(seed):
        p, d, ph = fw.cases.shoal_jonswap(2048, 2048, dx=1.0, seed=seed, Nfreq=16, Ntheta=4, Hmo=hs(seed),
                                          Xc_WK=150.0, Sponge_west_width=80.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    torch.cuda.set_device(0)
    dev = torch.device("cuda")
    kinds = [barred, planar, shoal]
    train_cases = [kinds[k % 3](101 + k) for k in range(n_traj)]
    t0 = time.perf_counter()
    X, T, Wm = [], [], []
    for c in train_cases:
        x, t, w = L.make_pairs(c, steps_per_traj, every=1)
        X.append(torch.from_numpy(x).to(dev))
        T.append(torch.from_numpy(t).to(dev))
        Wm.append(torch.from_numpy(w).to(dev))
        del x, t, w
    npairs = sum(a.shape[0] for a in X)
    t_pairs = time.perf_counter() - t0
    sizes = np.array([a.shape[0] for a in X], dtype=float)
    nets, t_train, losses = [], [], []
    for tr in range(n_train):
        # each training: its own initial weights and batch order
        net = L.Net(seed=tr)
        rng = np.random.default_rng(tr)
        t0 = time.perf_counter()
        lo = []
        for it in range(iters):
            k = rng.choice(len(X), p=sizes / sizes.sum())
            idx = torch.from_numpy(rng.choice(X[k].shape[0], size=batch, replace=False)).to(dev)
            lo.append(net.loss_grad(X[k][idx].contiguous(), T[k][idx].contiguous(), Wm[k][idx].contiguous()))
            net.adam(2e-3 * (0.5 ** (it / max(1, iters // 3))))
        t_train.append(time.perf_counter() - t0)
        losses.append([float(np.mean(lo[:50])), float(np.mean(lo[-50:]))])
        nets.append(net)
    del X, T, Wm
    torch.cuda.empty_cache()

    def ru(o):
        return fw.max_runup(np.pad(o["HeightMax"], 3), o["depth"])

    def rms(a, ref, mask):
        return float(np.sqrt(np.mean((a - ref)[mask] ** 2)))

    n_short = min(500, eval_coarse_steps)
    evals = []
    for name, c in (("barred_held_out", barred(909)), ("planar_held_out", planar(919)), ("shoal_held_out", shoal(929))):
        xh, th, wh = L.make_pairs(c, 100, every=5)
        ratios = []
        for net in nets:
            e0, e1 = L.one_step_error(net, xh, th, wh)
            ratios.append(e1 / e0 if e0 > 0 else None)
        del xh, th, wh
        fine = L.fine_run(c, 2 * eval_coarse_steps, snaps=(2 * n_short,))
        plain, _ = L.rollout(c, eval_coarse_steps, snaps=(n_short,))
        f_short = L.restrict(fine["snaps"][2 * n_short][0])
        f_long = L.restrict(fine["Eta"])
        p_short = plain["snaps"][n_short]
        ev = {"case": name, "coarse_steps": [n_short, eval_coarse_steps],
              "simulated_s": [n_short * 2.0 * c[0]["DT_fixed"], eval_coarse_steps * 2.0 * c[0]["DT_fixed"]],
              "one_step_error_ratio": ratios, "max_runup_fine_m": ru(fine), "max_runup_plain_m": ru(plain),
              "trainings": []}
        for net in nets:
            tr = {}
            for band in bands:
                net.set_shore_band(band)
                corr, applied = L.rollout(c, eval_coarse_steps, net=net, snaps=(n_short,))
                c_short = corr["snaps"][n_short]
                m_short = (p_short[1] > 0) & (c_short[1] > 0)
                m_long = (plain["MASK"] > 0) & (corr["MASK"] > 0)
                tr["band_%d" % band] = {
                    "eta_rms_plain_m": [rms(p_short[0], f_short, m_short), rms(plain["Eta"], f_long, m_long)],
                    "eta_rms_corrected_m": [rms(c_short[0], f_short, m_short), rms(corr["Eta"], f_long, m_long)],
                    "max_runup_corrected_m": ru(corr), "corrections_applied": applied,
                    "rejected_by": corr["rejected"]}
            net.set_shore_band(1)
            ev["trainings"].append(tr)
        evals.append(ev)
    for net in nets:
        net.close()
    return {"metric": "learned coarse-grid correction at full size", "grid_fine": [2048, 2048],
            "grid_coarse": [1024, 1024], "pairs": npairs, "trajectories": n_traj, "pairs_s": t_pairs,
            "train_iters": iters, "batch": batch, "trainings": n_train, "train_s": t_train,
            "loss_first_last": losses, "held_out": evals}


def learned_report(fw, iters=4000, eval_coarse_steps=500, unroll=1, every=2, scale=1, relax=(0.5, 0.25), nudge=None):
    """The learned coarse-grid correction, at reduced training scale: pairs
    (one coarse step of 2 x dx against two fine steps, restricted) from
    seeded planar beaches, barred beaches and a shoal with JONSWAP Hs
    0.5-2 m, all generated by the solver; Adam on the GPU; then on held-out
    seeds: eta RMS against the restricted fine run and the maximum run-up of
    the fine run, the plain coarse run and the corrected coarse run.
    Throughput: the fine 2048 x 2048 run (two fine steps) against the coarse
    1024 x 1024 run plus its correction (one coarse step), both mixed."""
    import numpy as np
    import torch
    L = fw.learned

    def dt_for(p, h):
        return round(0.35 * p["DX"] / np.sqrt(9.81 * max(h, 1.0)), 4)

    def barred(seed, M=256, N=128, shore=40.0, wk=120.0):
        p, d, ph, _ = fw.cases.barred_beach(M, N, 1.0, seed=seed, wk_from_shore=wk, nfreq=16, ntheta=4,
                                            shore_from_east=shore, Hmo=float(0.5 + 1.5 * ((seed * 37) % 10) / 9.0),
                                            Sponge_west_width=30.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    def planar(seed, cells=256 * 128):
        # a planar beach of the ensemble's distribution (grid sides are
        # multiples of 8, so the 2x2 restriction applies)
        p, d, ph = fw.cases.ensemble_members(1, seed=seed, nfreq=16, ntheta=4, cells_range=(cells, cells))[0]
        p["Hmo"] = min(p["Hmo"], 2.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    def shoal(seed, M=256, N=128):
        p, d, ph = fw.cases.shoal_jonswap(M, N, dx=2.0, seed=seed, Nfreq=16, Ntheta=4, Hmo=1.0, Xc_WK=80.0,
                                          Sponge_west_width=40.0)
        p["DT_fixed"] = dt_for(p, float(d.max()))
        return (p, d, ph)

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    # scale x (4 barred beaches, 3 planar beaches of the ensemble's
    # distribution, 1 shoal), seeds disjoint from the held-out 9 and 19
    train_cases = ([barred(s) for s in range(1, 2 + 4 * scale) if s != 9][:4 * scale] +
                   [planar(s) for s in range(11, 11 + 3 * scale) if s != 19] +
                   [shoal(s) for s in range(21, 21 + scale)])
    X, T, Wm = [], [], []
    for c in train_cases:
        x, t, w = L.make_pairs(c, 240, every=every, unroll=unroll, nudge=nudge)
        X.append(x)
        T.append(t)
        Wm.append(w)
    t_pairs = time.perf_counter() - t0
    net = L.Net(seed=0)
    t0 = time.perf_counter()
    losses = L.train(net, X, T, Wm, iters=iters, batch=8, lr=2e-3)
    t_train = time.perf_counter() - t0
    evals = []
    for name, c in (("barred_held_out", barred(9, M=384, N=128, shore=40.0, wk=150.0)), ("planar_held_out", planar(19))):
        xh, th, wh = L.make_pairs(c, 200, every=4)
        e0, e1 = L.one_step_error(net, xh, th, wh)
        fine = L.fine_run(c, 2 * eval_coarse_steps)
        plain, _ = L.rollout(c, eval_coarse_steps)
        corr, applied = L.rollout(c, eval_coarse_steps, net=net)
        f = L.restrict(fine["Eta"])
        m = (plain["MASK"] > 0) & (corr["MASK"] > 0)

        def ru(o):
            return fw.max_runup(np.pad(o["HeightMax"], 3), o["depth"])

        ev = {"case": name, "grid_fine": [c[0]["Mglob"], c[0]["Nglob"]], "coarse_steps": eval_coarse_steps,
              "one_step_error_ratio": e1 / e0 if e0 > 0 else None,
              "eta_rms_plain_m": float(np.sqrt(np.mean((plain["Eta"] - f)[m] ** 2))),
              "eta_rms_corrected_m": float(np.sqrt(np.mean((corr["Eta"] - f)[m] ** 2))),
              "max_runup_fine_m": ru(fine), "max_runup_plain_m": ru(plain),
              "max_runup_corrected_m": ru(corr), "corrections_applied": applied}
        # relaxed corrections: the last layer is linear, so scaling its
        # weights and bias by alpha scales the correction by alpha
        p0 = net.params()
        nw = len(p0) - (9 * 32 * 3 + 3)
        relaxed = {}
        for alpha in relax:
            pa = p0.copy()
            pa[nw:] *= alpha
            net.set_params(pa)
            ca, _ = L.rollout(c, eval_coarse_steps, net=net)
            ma = (plain["MASK"] > 0) & (ca["MASK"] > 0)
            relaxed[str(alpha)] = {"eta_rms_m": float(np.sqrt(np.mean((ca["Eta"] - f)[ma] ** 2))),
                                   "max_runup_m": ru(ca)}
        net.set_params(p0)
        if relaxed:
            ev["relaxed"] = relaxed
        evals.append(ev)
    # throughput at the configuration's sizes
    params, depth, phases = fw.cases.shoal_jonswap(2048, 2048, dx=1.0, seed=5, Nfreq=16, Ntheta=4)
    params = fw.with_defaults(params)
    params["DT_fixed"] = 0.02
    fs = fw.Solver(params, precision="MIXED")
    fs.init(depth, phases=phases)
    fs.step(4)
    ext, e0, e1 = cuda_timer(fs)
    fs.sync()
    e0.record(ext)
    fs.step(20)
    e1.record(ext)
    e1.synchronize()
    ms_fine = e0.elapsed_time(e1) / 20
    fs.close()
    pc, dc = L.coarse_case(params, depth)
    cs = fw.Solver(fw.with_defaults(pc), precision="MIXED")
    cs.init(dc, phases=phases)
    net.correct_run(cs, 4)
    cs.sync()
    t1 = time.perf_counter()
    net.correct_run(cs, 20)  # one graph replay per two (step + correction) pairs
    ms_coarse = (time.perf_counter() - t1) * 1e3 / 20
    cs.close()
    net.close()
    return {"metric": "learned coarse-grid correction", "training_pairs": int(sum(a.shape[0] for a in X)),
            "pairs_unroll": unroll, "pairs_every": every, "pairs_nudge": nudge, "training_cases": len(train_cases),
            "training_iters": iters, "pairs_s": t_pairs, "train_s": t_train,
            "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-50:])),
            "evaluation": evals,
            "ms_fine_2048_two_steps": 2 * ms_fine, "ms_coarse_1024_step_plus_correction": ms_coarse,
            "throughput_ratio": 2 * ms_fine / ms_coarse,
            "scale_note": "training on 8 solver-generated trajectories of about 256x128 fine cells (the "
                          "configuration asks for 2000 pairs at full size); throughput at the full 2048^2 / "
                          "1024^2 sizes"}


def host_info():
    """The host the CPU legs run on: the cores the OS has, the cores this
    process may run on (its affinity mask), and the CPU model."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as fh:
                for ln in fh:
                    if ln.lower().startswith("model name"):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"nproc": os.cpu_count(), "affinity_cores": len(os.sched_getaffinity(0)),
            "cpu_model": model or platform.machine(), "arch": platform.machine()}


def oracle_rate(params, depth, phases, fp32, threads, steps, warmup=1, max_seconds=None):
    """Cell-steps/s of the oracle on the workload: init, warm-up steps, then
    `steps` whole steps (fewer if max_seconds runs out); (rate, steps, s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import fw_oracle
    fw_oracle.build()
    o = fw_oracle.Oracle(params, threads=threads, fp32=fp32)
    o["Depth"][3:-3, 3:-3] = depth
    if phases is not None:
        o.set_phases(phases)
    o.init()
    for _ in range(warmup):
        o.step()
    n, t0 = 0, time.perf_counter()
    while n < steps:
        o.step()
        n += 1
        if max_seconds is not None and time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    o.close()
    return params["Mglob"] * params["Nglob"] * n / dt, n, dt


def cpu_baseline(fw, params, depth, phases, max_seconds=12.0, max_steps=5):
    """The oracle (the C restatement of the reference) on every core this
    process may use, on the same workload: its single-precision build (the
    reference's default REAL(SP) = 4-byte build) as the value, the FP64
    build beside it."""
    host = host_info()
    threads = host["affinity_cores"]
    r32, n32, t32 = oracle_rate(params, depth, phases, True, threads, max_steps, max_seconds=max_seconds)
    r64, n64, t64 = oracle_rate(params, depth, phases, False, threads, max_steps, max_seconds=max_seconds)
    return {"value": r32, "unit": UNIT, "cores": threads, "kind": "port", "dtype": "f32",
            "sample": "%d whole single-precision steps of the %dx%d workload after init and one warm-up step "
                      "(%.1f s), on %d OpenMP threads" % (n32, params["Mglob"], params["Nglob"], t32, threads),
            "fp64": {"value": r64, "unit": UNIT, "dtype": "f64",
                     "sample": "%d whole FP64 steps, the same way (%.1f s)" % (n64, t64)},
            "host": host}


def reference_arm(args, fw, params, depth, phases):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    host = host_info()
    threads = host["affinity_cores"]
    # the reference's default build is single precision (REAL(SP) = 4 bytes,
    # mod_param.F:58-68); the FP64 build is timed beside it on a short sample
    v, n, dt = oracle_rate(params, depth, phases, True, threads, args.steps, warmup=args.warmup)
    v64, n64, dt64 = oracle_rate(params, depth, phases, False, threads, 3, warmup=1, max_seconds=10.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [params["Mglob"], params["Nglob"]], "dx_m": params["DX"],
                   "precision": "FP32 (the reference's default single-precision build)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "dtype": "f32",
                         "sample": "%d whole single-precision steps of the %dx%d workload after %d warm-up "
                                   "steps; the Fortran reference cannot be compiled (no Fortran compiler on "
                                   "either host), so its C restatement (oracle/) runs on %d OpenMP threads, "
                                   "one per core of this process's affinity mask"
                                   % (n, params["Mglob"], params["Nglob"], args.warmup, threads),
                         "host": host},
        "fp64": {"value": v64, "unit": UNIT, "dtype": "f64",
                 "sample": "%d whole FP64 steps after one warm-up step (%.1f s)" % (n64, dt64)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=2048, help="grid edge (2048 for the benchmark)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 512-run ensemble measurement")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes (no fw_autotune)")
    ap.add_argument("--tuning", default=None,
                    help="launch shapes as JSON (the config's launch_shapes of an earlier run) instead of fw_autotune")
    ap.add_argument("--learned-unroll", type=int, default=1,
                    help="learned report: coarse steps unrolled from each restricted fine start")
    ap.add_argument("--learned-every", type=int, default=2,
                    help="learned report: coarse steps between restricted fine starts")
    ap.add_argument("--learned-nudge", type=float, default=None,
                    help="learned report: pairs along one coarse run nudged by this fraction toward the fine run")
    ap.add_argument("--learned-scale", type=int, default=1,
                    help="learned report: multiple of the 8 training cases")
    ap.add_argument("--learned-iters", type=int, default=4000, help="learned reports: Adam iterations")
    ap.add_argument("--net-report", action="store_true",
                    help="time the correction network's forward pass and training iteration")
    ap.add_argument("--learned-full", action="store_true",
                    help="the learned correction trained on 2000 solver-generated pairs at 2048^2 / 1024^2")
    ap.add_argument("--learned-report", action="store_true",
                    help="only the learned coarse-grid correction report (training, held-out error, throughput)")
    ap.add_argument("--precision-report", action="store_true",
                    help="only the 4096x4096 barred-beach mixed-vs-FP64 report (about 10 GPU minutes)")
    ap.add_argument("--no-kernel-profile", action="store_true",
                    help="skip the per-kernel timing (e.g. for an ncu launch list of the stepping only)")
    ap.add_argument("--fp64-only", action="store_true",
                    help="only the FP64 path on the --size workload: --warmup then --steps steps (e.g. for ncu)")
    args = ap.parse_args()
    fw = __graft_entry__.load_package()
    params, depth, phases = fw.cases.shoal_jonswap(Mglob=args.size, Nglob=args.size, seed=2024)
    params = fw.with_defaults(params)
    if args.impl == "reference":
        return reference_arm(args, fw, params, depth, phases)
    if args.net_report:
        print(json.dumps(net_report(fw)), flush=True)
        return 0
    if args.fp64_only:
        print(json.dumps(fp64_only(fw, args.size, args.steps, args.warmup)), flush=True)
        return 0
    if args.learned_full:
        print(json.dumps(learned_full_report(fw, iters=args.learned_iters)), flush=True)
        return 0
    if args.learned_report:
        print(json.dumps(learned_report(fw, iters=args.learned_iters, unroll=args.learned_unroll,
                                        every=args.learned_every, scale=args.learned_scale,
                                        nudge=args.learned_nudge)), flush=True)
        return 0
    if args.precision_report:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(precision_report(fw)), flush=True)
        return 0

    ws, rank, local = dist_env()
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = True
    import torch
    torch.cuda.set_device(local)
    fw.load_library()
    K, W = args.steps, max(args.warmup, 3)
    cells = params["Mglob"] * params["Nglob"]
    hbm, peak_kind = peaks()

    tune_arg = json.loads(args.tuning) if args.tuning else (not args.no_autotune)
    sm, rm = run_precision(fw, params, depth, phases, "MIXED", K, W, local, pg, autotune=tune_arg)
    ms_mixed = max_over_ranks(rm["ms"], pg)
    res64 = None
    if not args.no_fp64:
        s64, r64 = run_precision(fw, params, depth, phases, "FP64", K, W, local, pg, autotune=not args.no_autotune)
        ms64 = max_over_ranks(r64["ms"], pg)
        import numpy as np
        e_m = sm.get("Eta")[3:-3, 3:-3]
        e_d = s64.get("Eta")[3:-3, 3:-3]
        wet = (s64.get("MASK")[3:-3, 3:-3] > 0)
        rms = float(np.sqrt(np.mean((e_m - e_d)[wet] ** 2)))
        mask_m, mask_d = sm.get("MASK"), s64.get("MASK")
        mask_mis = int(np.sum(mask_m != mask_d))
        # where the MASK differs: interior or ghost cells, and how far the
        # FP64 run's total depth eta + h is from the wet/dry threshold there
        mis = mask_m != mask_d
        ghost = np.ones_like(mis)
        ghost[3:-3, 3:-3] = False
        hd = np.asarray(s64.get("Eta")) + np.asarray(s64.get("Depth"))
        mask_detail = {"interior": int((mis & ~ghost).sum()), "ghost": int((mis & ghost).sum()),
                       "abs_total_depth_m_percentiles": (
                           {q: float(np.percentile(np.abs(hd[mis]), float(q))) for q in ("50", "90", "100")}
                           if mis.any() else None)}
        res64 = {"value": aggregate_rate(cells, K, ws, ms64), "ms_per_step": ms64 / K, "dtype": "f64",
                 "step_roofline_frac_hbm": STEP_BYTES["fp64"] * cells / (ms64 / K * 1e-3) / 1e9 / hbm,
                 "eta_rms_mixed_vs_fp64_m": rms, "mask_mismatch_cells": mask_mis,
                 "mask_mismatch_detail": mask_detail,
                 "time_mixed_s": sm.scalar("TIME"), "time_fp64_s": s64.scalar("TIME"),
                 "status": r64["status"]}
        prof64 = {} if args.no_kernel_profile else kernel_profile(
            s64, 8, cells, (params["Mglob"] + 1) * params["Nglob"], params["Mglob"] * (params["Nglob"] + 1), hbm)
        res64["kernels"] = {k: round(v["ms"], 4) for k, v in prof64.items()}
        s64.close()
        # the stated eta error over a whole run: the 250 x 500 planar beach
        # through its 300 s (rank 0 only)
        if rank == 0:
            res64["full_run_250x500"] = c1_full_run(fw)
    e2e_steps = min(K, 10)
    e2e_dt, h2d, d2h = e2e_run(fw, sm, e2e_steps, f32=True)
    e2e64_dt, h2d64, d2h64 = e2e_run(fw, sm, e2e_steps, f32=False)
    link = link_rates(h2d // 5)
    # per-kernel timing last: some kernels update the state in place
    prof = {} if args.no_kernel_profile else kernel_profile(
        sm, 4, cells, (params["Mglob"] + 1) * params["Nglob"], params["Mglob"] * (params["Nglob"] + 1), hbm)
    dom = max(prof, key=lambda k: prof[k]["ms"]) if prof else None
    sm.close()
    ens = None if args.no_ensemble else ensemble_bench(fw, pg, ws, autotune=not args.no_autotune)
    if rank != 0:
        return 0
    value = aggregate_rate(cells, K, ws, ms_mixed)
    step_s = ms_mixed / K * 1e-3
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms_mixed / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 tridiagonal and depth tests)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid": [params["Mglob"], params["Nglob"]], "dx_m": params["DX"],
                   "precision": "MIXED", "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "state (~0.8 GB mixed, ~1.6 GB FP64) exceeds the 129 MB L2; no flush",
                   "launch_shapes": rm["tuning"], "autotune_s": rm["tune_s"]},
        "gpu_launches": rm["launches_per_step"] * K,
        "clocks": rm["clocks"],
        "status": rm["status"],
        "step_roofline": {"bound": "hbm", "bytes_per_cell_step": STEP_BYTES["mixed"],
                          "achieved": STEP_BYTES["mixed"] * cells / step_s / 1e9, "peak": hbm, "unit": "GB/s",
                          "frac": STEP_BYTES["mixed"] * cells / step_s / 1e9 / hbm, "peak_kind": peak_kind},
        "e2e": {"value": cells * e2e_steps / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "what": "per step: Eta,U,V,Ubar,Vbar uploaded as float host arrays (the reference's default "
                        "REAL(SP) build) from pinned memory (one fw_set_fields_f32), fw_step, Eta,U,V read back "
                        "(one fw_get_fields_f32)",
                "double_host": {"value": cells * e2e_steps / e2e64_dt, "h2d_bytes_per_step": h2d64,
                                "d2h_bytes_per_step": d2h64,
                                "what": "the same with double host arrays (a -DDOUBLE_PRECISION host; "
                                        "fw_set_fields / fw_get_fields)"},
                # the transfers' share of a step against the pinned copy rates
                # of this machine's host link
                "transfer_ms_per_step": e2e_dt / e2e_steps * 1e3 - ms_mixed / K,
                "link_gbs": {k: round(v, 1) for k, v in link.items()},
                "link_bound_ms_per_step": (h2d / link["h2d"] + d2h / link["d2h"]) / 1e6},
        "fp64": res64,
        "ensemble": ens,
        "kernels_ms": {k: round(v["ms"], 4) for k, v in prof.items()},
    }
    if dom:
        d = prof[dom]
        unit = ((params["Mglob"] + 1) * params["Nglob"] if dom == "flux_x" else
                params["Mglob"] * (params["Nglob"] + 1) if dom == "flux_y" else cells)
        tpu = TRAFFIC_PER_UNIT_MIXED.get(dom)
        line["roofline"] = {"kernel": dom, "bound": "hbm", "achieved": d["gbs"], "peak": hbm, "unit": "GB/s",
                            "frac": d["frac"], "traffic": tpu * unit if tpu else None, "peak_kind": peak_kind,
                            "algorithmic_bytes_per_launch": d["bytes"], "ms_per_launch": d["ms"],
                            "traffic_from": "ncu dram__bytes_read.sum + dram__bytes_write.sum, 2048x2048 capture, "
                                            "bytes per unit x units of this launch"}
    if not args.no_cpu_baseline and ws == 1:
        line["cpu_baseline"] = cpu_baseline(fw, params, depth, phases)
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
