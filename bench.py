"""Throughput of the fused two-phase D2Q9 LBM step on GB300 (MLUPS).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--dtype f32|f64] [--impl ours|reference]

Workload (the plain FP32 fused kernel at scale): a 4096 x 2048 lattice with
walls at the bottom and top (the walled variant, fingering.py), Zou-He plug
inlet u_x = 0.01 and the reference's velocity-type outlet, seeded random
circular and square blocks with radius / half-side 6..14 placed to porosity
0.7, tau_inv = 0.6, tau_def = 1.0, interfacial tension 5e-4, contact angle
120 deg (psi_wall from the droplet calibration table).  Synthetic, seeded; no dataset involved.

A step is one iteration of the reference's loop body over the whole lattice
(one fused kernel).  `value` is lattice updates per second over all ranks
with the state resident in HBM (18 planes x 8.4 M cells x 4 B = 604 MB read
and written per step, far larger than L2, so no L2 flush is needed).  `e2e`
is the same metric through the host-buffer API: every step uploads the
populations from pinned host memory, advances one iteration and downloads
them again (fd_fused_step_packed_host: the two copy directions and the
kernel pipelined over row chunks).  With --gpus N > 1 each rank runs its own instance (replicas,
weak scaling, no collective on the data path).

The K-step timed region is repeated until the repetitions cover 0.5 s (so the
clock sampler sees the load) and the median repetition is reported.  The
default FP32 line also carries, measured the same way in the same process,
the rest of the metric: `f16` and `bf16` (FP16 / BF16 storage of the same
workload, 76 B per lattice update) and `ensemble` (the batched ensemble of 96
seeded lattices, autotuned tile shape, CUDA-graph replay).

--impl reference times the CPU implementation of the same step (the numpy
oracle, which restates the reference's numpy code operation for operation)
on the host cores: one process per core, each on a 512 x 256 sample of the
same generator.
"""
from __future__ import annotations

import argparse

import numpy as np
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

H_FULL, W_FULL = 2048, 4096
SAMPLE_H, SAMPLE_W = 256, 512
# algorithmic bytes per lattice update: every stored population read once and written once
# (f16 / bf16 keep g_0 in FP32: 17 planes x 2 B + 1 plane x 4 B each way)
BYTES_PER_LU = {"f64": 288, "f32": 144, "f32-exact": 144, "f16": 76, "bf16": 76}
WORKLOAD = "walls_4096x2048_porosity0.7_blocks6-14"
# tau_inv = 0.55 (with tau_def = 1.0) diverges within ~40 steps on this block geometry in the oracle
# itself (the reference algorithm); 0.6 is the closest value that runs thousands of steps.
TAU_INV = 0.6


def workload(H, W, seed=2024):
    from fingering_dynamics_gb300 import geometry as geo
    from fingering_dynamics_gb300.params import from_relaxation_times
    prm = from_relaxation_times(H, W, tau_inv=TAU_INV, tau_def=1.0, sigma=5e-4, contact_angle_deg=120.0,
                                u_in=0.01, variant="walls")
    rects, circles = geo.random_blocks(H, W, 0.7, 6, 14, seed=seed, x_margin=32)
    g = geo.build_geometry(H, W, rects=rects, circles=circles, walls=True)
    return prm, g


def measured_peak():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(key):
    p = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh).get(key)
    return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU (oracle) timing
# ---------------------------------------------------------------------------
def _cpu_sample_worker(args):
    seed, iters, warm = args
    import warnings
    warnings.filterwarnings("ignore")
    from oracle.lbm_oracle import OracleParams, OracleState
    prm, g = workload(SAMPLE_H, SAMPLE_W, seed=seed)
    op = OracleParams(H=prm.H, W=prm.W, variant="walls", tau=prm.tau, eta_n=prm.eta_n, M=prm.M, a=prm.a,
                      kappa=prm.kappa, gamma=prm.gamma, psi_wall=prm.psi_wall, inlet_ux=prm.inlet_ux,
                      outlet_coef=prm.outlet_coef)
    st = OracleState(op, g.solid, prm.initial_psi(g.solid), init_mu=True, init_uy=True)
    for _ in range(warm):
        st.step(g.corner_list, g.circle_masks)
    t0 = time.perf_counter()
    for _ in range(iters):
        st.step(g.corner_list, g.circle_masks)
    t1 = time.perf_counter()
    return t0, t1, iters * prm.H * prm.W


def cpu_baseline(max_seconds=15.0):
    """One core, the oracle on a 512 x 256 sample, until ~max_seconds."""
    import warnings
    warnings.filterwarnings("ignore")
    from oracle.lbm_oracle import OracleParams, OracleState
    prm, g = workload(SAMPLE_H, SAMPLE_W)
    op = OracleParams(H=prm.H, W=prm.W, variant="walls", tau=prm.tau, eta_n=prm.eta_n, M=prm.M, a=prm.a,
                      kappa=prm.kappa, gamma=prm.gamma, psi_wall=prm.psi_wall, inlet_ux=prm.inlet_ux,
                      outlet_coef=prm.outlet_coef)
    st = OracleState(op, g.solid, prm.initial_psi(g.solid), init_mu=True, init_uy=True)
    st.step(g.corner_list, g.circle_masks)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < max_seconds and n < 400:
        st.step(g.corner_list, g.circle_masks)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": round(n * prm.H * prm.W / dt / 1e6, 4), "unit": "MLUPS", "cores": 1, "kind": "port",
            "sample": f"numpy oracle, {SAMPLE_W}x{SAMPLE_H} lattice of the same generator, {n} steps in {dt:.1f} s, "
                      f"1 process"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    iters = max(1, args.steps)
    ctx = mp.get_context("spawn")
    t_start = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_sample_worker, [(1000 + i, iters, max(1, args.warmup)) for i in range(cores)])
    t0 = min(r[0] for r in res)
    t1 = max(r[1] for r in res)
    cells = sum(r[2] for r in res)
    mlups = cells / (t1 - t0) / 1e6
    ms = (t1 - t0) / iters * 1e3
    sample = (f"numpy oracle (the reference's numpy step restated op for op), {cores} processes x "
              f"{SAMPLE_W}x{SAMPLE_H} samples of the same generator, {iters} timed steps each")
    line = {"metric": "MLUPS", "value": round(mlups, 4), "unit": "MLUPS", "n_gpus": args.gpus, "steps": iters,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"{SAMPLE_W}x{SAMPLE_H}", "variant": "walls"},
            "cpu_baseline": {"value": round(mlups, 4), "unit": "MLUPS", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(mlups, 4), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(time.perf_counter() - t_start, 1)}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# replicas across ranks (host logic, any torch.distributed backend)
# ---------------------------------------------------------------------------
def replica_seed(rank: int) -> int:
    """Geometry seed of rank `rank`'s lattice: every rank runs its own
    instance of the workload (replicas, no data-path collective)."""
    return 2024 + rank


def max_over_ranks(values, device="cpu"):
    """Element-wise max of `values` over all ranks of the default process
    group (the slowest rank bounds the job's time); identity without one."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def job_mlups(world: int, cells: int, steps: int, ms_total: float) -> float:
    """Whole-job lattice updates per second: all ranks' cells over the
    slowest rank's time."""
    return world * cells * steps / (ms_total / 1e3) / 1e6


MIN_TIMED_S = 0.5  # the K-step timed region is repeated until the repetitions cover at least this long


def timed_repetitions(run_steps, stream, min_s=MIN_TIMED_S, max_reps=5000, barrier=None):
    """Milliseconds of each repetition of `run_steps()` (one timed region of K
    steps, CUDA events on `stream`, synchronised and, with `barrier`, a barrier
    over ranks on both sides), repeated until the repetitions cover `min_s`
    seconds.  With several ranks every rank stops after the same repetition."""
    import torch
    out = []
    total = 0.0
    while len(out) < max_reps:
        torch.cuda.synchronize()
        if barrier is not None:
            barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run_steps()
        e1.record(stream)
        torch.cuda.synchronize()
        if barrier is not None:
            barrier()
        out.append(e0.elapsed_time(e1))
        total += out[-1]
        done = total >= min_s * 1e3
        if barrier is not None:
            done = max_over_ranks([float(done)], device=f"cuda:{torch.cuda.current_device()}")[0] > 0
        if done:
            break
    return out


def roofline(dtype, cells, ms_step):
    alg_bytes = BYTES_PER_LU[dtype] * cells
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg_bytes}


def measure_single(prm, g, dtype, steps, warmup, rows=0, rounding="stochastic"):
    """A storage type on the single-lattice workload: `warmup` steps, then the
    K-step timed region repeated (timed_repetitions); median ms per step."""
    import torch
    from fingering_dynamics_gb300.lattice import Lattice
    lat = Lattice(prm, g, dtype=dtype, rounding=rounding)
    lat.enter_fused()
    lat.advance(warmup, rows)
    stream = torch.cuda.current_stream()
    with ClockSampler(torch.cuda.current_device()) as clk:
        reps = timed_repetitions(lambda: lat.advance(steps, rows), stream)
    ms_step = statistics.median(reps) / steps
    lat.exit_fused()
    finite = bool(torch.isfinite(lat.psi).all().item())
    del lat
    torch.cuda.empty_cache()
    return {"dtype": dtype, "value": round(prm.H * prm.W / (ms_step / 1e3) / 1e6, 1), "unit": "MLUPS",
            "ms_per_step": round(ms_step, 4), "timed_repetitions": len(reps), "steps_per_repetition": steps,
            "roofline": roofline(dtype, prm.H * prm.W, ms_step),
            "rounding": rounding if dtype in ("f16", "bf16") else None, "state_finite_after_timing": finite,
            "gpu_launches_per_repetition": steps, "clocks": clk.summary()}


ENSEMBLE_SETTLE_STEPS = 200  # before timing, so that members that diverge at once are quarantined


def measure_ensemble(steps, warmup, members=96, dtype="f32", family="config", seed=2024):
    """The batched ensemble (seeded lattices of uneven size, geometry and
    parameters; one persistent launch per iteration replayed from a CUDA graph;
    tile shape autotuned on the ensemble): aggregate MLUPS, median over
    repetitions of the K-step timed region.  Members that meet a non-finite
    cell are quarantined by the batch (skipped from then on); the value counts
    only the cells of members still stepping at the end of the timed region."""
    import torch
    from fingering_dynamics_gb300.ensemble import Ensemble, ensemble_specs
    specs = ensemble_specs(members, seed=seed, family=family)
    ens = Ensemble([s.build() for s in specs], dtype=dtype)
    ens.step(ENSEMBLE_SETTLE_STEPS)
    settled = ens.member_status()
    tuned = ens.autotune(steps=10)
    ens.step(warmup)
    with ClockSampler(torch.cuda.current_device()) as clk:
        reps = timed_repetitions(lambda: ens.step(steps, use_graph=True), ens.stream)
    ms_step = statistics.median(reps) / steps
    quarantined = ens.member_status()
    active_cells = sum(lat.H * lat.W for lat, q in zip(ens.lattices, quarantined) if not q)
    out = {"dtype": dtype, "members": members, "family": family, "cells": ens.cells,
           "active_cells": active_cells, "members_quarantined_before_timing": int(sum(settled)),
           "members_quarantined": int(sum(quarantined)), "members_finite": members - int(sum(quarantined)),
           "settle_steps": ENSEMBLE_SETTLE_STEPS,
           "value": round(active_cells / (ms_step / 1e3) / 1e6, 1), "unit": "MLUPS", "ms_per_step": round(ms_step, 4),
           "timed_repetitions": len(reps), "steps_per_repetition": steps,
           "roofline": roofline(dtype, active_cells, ms_step),
           "tile_shape": {"band_width": ens.config[0], "rows_per_strip": ens.config[1], "cells_per_thread": 1},
           "autotune_mlups": {f"{b}x{r}": round(v, 1) for (b, r), v in tuned.items()},
           "graph": True, "gpu_launches_per_repetition": steps,
           "clocks": clk.summary()}
    ens.close()
    del ens
    torch.cuda.empty_cache()
    return out


# ---------------------------------------------------------------------------
# GPU timing
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300.lattice import Lattice
    build.build()
    prm, g = workload(args.H, args.W, seed=replica_seed(rank))
    lat = Lattice(prm, g, dtype=args.dtype, device=f"cuda:{local}", rounding=args.rounding)
    H, W = prm.H, prm.W
    lat.enter_fused()
    for _ in range(args.warmup):
        lat.advance(1, args.rows)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    barrier()
    # the K-step timed region (synchronize and barrier on both sides), repeated
    # until the repetitions cover MIN_TIMED_S; the median repetition is reported
    with ClockSampler(local) as clk:
        def region():
            for _ in range(args.steps):
                lat.advance(1, args.rows)
        reps = timed_repetitions(region, stream, barrier=barrier if world > 1 else None)
    ms_total = statistics.median(reps)
    clocks = clk.summary()
    lat.exit_fused()
    finite = bool(torch.isfinite(lat.psi).all().item())
    lat.enter_fused()

    # end to end through the host-buffer API: the state in pinned host memory,
    # every step uploaded, advanced one iteration and downloaded again (packed
    # storage: one pipelined fd_fused_step_packed_host call per step; FP64:
    # upload, fused step, download)
    state = lat.current_buffer()
    e2e_steps = max(3, min(args.steps, 20))
    e2e_s = float("nan")

    def host_step(host):
        if lat.storage is not None and not args.e2e_serial:
            lat.advance_host(host, chunk_rows=args.e2e_chunk_rows)
        else:
            lat.upload_populations(host)
            lat.advance(1, args.rows)
            lat.download_populations(host)

    if not args.no_e2e:
        host = torch.empty(state.shape, dtype=state.dtype, pin_memory=True)
        host.copy_(state)
        for _ in range(2):
            host_step(host)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host_step(host)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0

    ms_total, e2e_s = max_over_ranks([ms_total, e2e_s], device=f"cuda:{local}")
    if rank == 0:

        ms_step = ms_total / args.steps
        cells = H * W
        mlups = job_mlups(world, cells, args.steps, ms_total)
        alg_bytes = BYTES_PER_LU[args.dtype] * cells
        achieved = alg_bytes / (ms_step / 1e3) / 1e9
        peak, peak_kind = measured_peak()
        pop_bytes = int(state.numel() * state.element_size())
        line = {
            "metric": "MLUPS", "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
            "config": {"workload": WORKLOAD if (H, W) == (H_FULL, W_FULL) else f"walls_{W}x{H}_porosity0.7_blocks6-14",
                       "H": H, "W": W, "variant": "walls", "porosity": round(g.porosity, 4),
                       "blocks": len(g.rects) + len(g.circles),
                       "tau_inv": TAU_INV, "tau_def": 1.0, "sigma": 5e-4, "contact_angle_deg": 120, "u_in": 0.01,
                       "l2": "inputs larger than L2 (populations 2 x %d MB)" % (pop_bytes // 2 ** 20),
                       "parallelism": f"replicas{world}", "rows_per_warp": args.rows or "auto",
                       "rounding": args.rounding if args.dtype in ("f16", "bf16") else None,
                       "state_finite_after_timing": finite},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                         "traffic": committed_traffic(f"fused_{args.dtype}_{W}x{H}"),
                         "algorithmic_bytes_per_launch": alg_bytes},
            "e2e": None if args.no_e2e else {
                "value": round(world * cells * e2e_steps / e2e_s / 1e6, 1), "unit": "MLUPS",
                "h2d_bytes_per_step": pop_bytes, "d2h_bytes_per_step": pop_bytes,
                "path": "serial" if (args.e2e_serial or lat.storage is None) else
                        f"pipelined host step, chunk rows {args.e2e_chunk_rows or 'auto'}"},
            "gpu_launches": args.steps,
            "clocks": clocks,
            "timed_repetitions": {"count": len(reps), "steps_each": args.steps,
                                  "ms_median": round(statistics.median(reps), 4), "ms_min": round(min(reps), 4),
                                  "ms_max": round(max(reps), 4)},
            # fluid cells only (the metric counts every cell, solid ones too, as the reference streams them)
            "mflups_fluid": round(mlups * g.porosity, 1),
        }
        if not args.no_extras and args.dtype == "f32" and world == 1:
            # the rest of the metric on the same box and workload: reduced-precision storage and the batch
            for d in ("f16", "bf16"):
                sub = measure_single(prm, g, d, args.steps, args.warmup, args.rows, args.rounding)
                sub["ratio_to_f32"] = round(sub["value"] / mlups, 3)
                line[d] = sub
            line["ensemble"] = measure_ensemble(args.steps, args.warmup)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_ensemble(args):
    """The batched ensemble: --members seeded independent lattices of uneven
    size, geometry and parameters (--family), advanced by one persistent
    batched launch per iteration (CUDA-graph replay), tile shape chosen by the
    autotuner, diverging members quarantined; aggregate MLUPS over the members
    still stepping."""
    from fingering_dynamics_gb300 import build
    build.build()
    sub = measure_ensemble(args.steps, args.warmup, members=args.members, dtype=args.dtype, family=args.family)
    line = {"metric": "MLUPS", "value": sub["value"], "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sub["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
            "config": {"workload": f"ensemble_{args.members}_members", **{k: v for k, v in sub.items() if k not in (
                "value", "unit", "ms_per_step", "roofline", "clocks")},
                       "rounding": args.rounding if args.dtype in ("f16", "bf16") else None},
            "roofline": sub["roofline"], "gpu_launches": args.steps, "clocks": sub["clocks"]}
    print(json.dumps(line), flush=True)
    return 0


def run_precision(args):
    """Reduced-precision storage: error against the FP64 path on a 1024 x 256
    instance of the same generator (max |dpsi|, colour-mass drift, saturation
    and tip error, breakthrough iteration), one line per run."""
    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300.precision import precision_study
    build.build()
    H, W = (256, 1024) if (args.H, args.W) == (H_FULL, W_FULL) else (args.H, args.W)
    prm, g = workload(H, W)
    t0 = time.perf_counter()
    res = precision_study(prm, g, dtypes=("f32", "f16", "bf16", "f16/nearest", "bf16/nearest"), steps=args.steps,
                          every=args.every)
    if args.out:
        with open(args.out, "w") as fh:
            json.dump(res, fh)
    per = {d: {k: v for k, v in r.items() if k != "curve"} for d, r in res["per_dtype"].items()}
    line = {"metric": "max |psi - psi_fp64| over fluid cells, first %d iterations" % res["window"],
            "value": per["f16"]["max_dpsi_window"], "unit": "psi", "higher_is_better": False, "n_gpus": 1,
            "steps": args.steps, "dtype": "f16", "data": "synthetic",
            "config": {"workload": f"walls_{W}x{H}_porosity0.7_blocks6-14", "H": H, "W": W, "every": args.every,
                       "reference": "FP64 fused kernel (bitwise equal to the numpy oracle)"},
            "breakthrough_f64": res["breakthrough_f64"], "per_dtype": per,
            "wall_s": round(time.perf_counter() - t0, 1)}
    print(json.dumps(line), flush=True)
    return 0


def run_accelerated(args):
    """The surrogate-accelerated ensemble against the plain batched LBM on the
    held-out members of the surrogate workload (same generator and seeds; the
    last 10% of --members), with a network trained and saved by
    `--workload surrogate --save-net`."""
    import torch
    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300.ensemble import ensemble_specs
    from fingering_dynamics_gb300.surrogate import UNet, accelerated_ensemble, breakthrough_race
    build.build()
    if not args.load_net:
        raise SystemExit("--workload accelerated needs --load-net (a network saved by --workload surrogate --save-net)")
    H, W, jump = 256, 512, 200
    M = args.members
    specs = ensemble_specs(M, seed=2024, sizes_w=(W,), sizes_h=(H,))
    held = max(1, M // 10)
    net = UNet((32, 64, 128, 256), params=dict(np.load(args.load_net)), conv=args.conv)
    members = [specs[i].build() for i in range(M - held, M)][:args.batch]
    # pick the convolution kernels for the batch shape before the timed runs
    net.predict(torch.zeros((len(members), H, W, 16), dtype=torch.bfloat16, device="cuda"))
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        acc = {r: accelerated_ensemble(net, members, rounds=5, jump=jump, restart=r)
               for r in ("regularised", "equilibrium")}
        race = breakthrough_race(net, members, max_rounds=args.max_rounds, jump=jump) if args.max_rounds else None
    line = {"metric": "surrogate-accelerated ensemble speed-up over the plain batched LBM, same horizon",
            "value": round(acc["regularised"]["speedup"], 3), "unit": "x", "higher_is_better": True, "n_gpus": 1,
            "steps": 5, "warmup": 0, "dtype": "bf16 network, f32 lattices", "data": "synthetic (held-out geometries)",
            "config": {"workload": f"accelerated_{len(members)}_members_{W}x{H}", "rounds": 5,
                       "jumps_per_check": 5, "jump": jump, "tolerance": 0.02, "restart": "regularised"},
            "accelerated_ensemble": acc["regularised"], "accelerated_ensemble_equilibrium_restart": acc["equilibrium"],
            "breakthrough_race": race, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_surrogate(args):
    """The learned surrogate at 512 x 256.  Trajectories of
    a seeded ensemble (batched LBM, one frame every 200 iterations), the last
    10% of geometries held out; AdamW training of the U-Net (32/64/128/256)
    with the project's tensor-core kernels, timed with CUDA events; held-out
    error against persistence, autoregressive saturation error, and the time
    of one jump against 200 batched LBM iterations of the same members."""
    import torch
    from fingering_dynamics_gb300 import build
    from fingering_dynamics_gb300.ensemble import Ensemble, ensemble_specs
    from fingering_dynamics_gb300.surrogate import (UNet, accelerated_ensemble, evaluate, expand,
                                                    generate_trajectories, rollout_saturation_error, train)
    build.build()
    H, W, jump = 256, 512, 200
    M = args.members
    specs = ensemble_specs(M, seed=2024, sizes_w=(W,), sizes_h=(H,))
    held = max(1, M // 10)
    t0 = time.perf_counter()
    frames, finite = generate_trajectories(specs, n_frames=args.frames, jump=jump)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    fin = finite.cpu().numpy()
    train_idx = [i for i in range(M - held) if fin[i]]
    test_idx = [i for i in range(M - held, M) if fin[i]]
    train_f, test_f = frames[train_idx], frames[test_idx]
    net = UNet((32, 64, 128, 256), seed=0, conv=args.conv)
    train(net, train_f, steps=args.warmup, batch=args.batch, seed=1)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        hist = train(net, train_f, steps=args.train_steps, batch=args.batch, lr=1e-3, lr_end=5e-5, seed=2,
                     log_every=max(1, args.train_steps // 10))
        e1.record(stream)
        torch.cuda.synchronize()
    ms_step = e0.elapsed_time(e1) / args.train_steps
    flops_step = 3.0 * net.flops_forward(args.batch, H, W)
    tflops = flops_step / (ms_step / 1e3) / 1e12
    if args.save_net:
        np.savez(args.save_net, **net.state_dict())
    ev = evaluate(net, test_f)
    roll = rollout_saturation_error(net, test_f, start=0, jumps=5)
    # one jump of `batch` members: surrogate forward vs 200 batched LBM iterations
    nb = min(args.batch, M)
    ens = Ensemble([s.build() for s in specs[:nb]])
    ens.step(5)
    t_lbm = ens.time_steps(jump, use_graph=True)
    ens.close()
    x = expand(frames[:nb, 0])
    for _ in range(3):
        net.forward(x)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(10):
        net.forward(x)
    f1.record(stream)
    torch.cuda.synchronize()
    t_sur = f0.elapsed_time(f1) / 10 / 1e3
    del frames, train_f, test_f, x
    torch.cuda.empty_cache()
    accel = accelerated_ensemble(net, [specs[i].build() for i in test_idx[:args.batch]], rounds=5, jump=jump)
    peak = None
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        peak = float(json.load(open(p))["bf16_tflops_sustained"])
    peak_kind = "measured (sustained)" if peak else "fallback"
    peak = peak or 1700.0
    line = {"metric": "surrogate training throughput (tensor-core convolutions, fwd + data + weight gradients)",
            "value": round(tflops, 2), "unit": "TFLOP/s", "higher_is_better": True, "n_gpus": 1,
            "steps": args.train_steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "dtype": "bf16",
            "data": "synthetic (batched-LBM trajectories)",
            "config": {"workload": f"unet_{W}x{H}_batch{args.batch}", "widths": [32, 64, 128, 256],
                       "conv_kernel": args.conv,
                       "conv_choice": {"x".join(map(str, k)): v for k, v in net.conv_choice.items()},
                       "optimizer": "AdamW, lr 1e-3 -> 5e-5 cosine, weight decay 1e-2",
                       "params": net.n_params, "members": M, "held_out_members": len(test_idx),
                       "train_members": len(train_idx), "frames_per_member": args.frames, "jump": jump,
                       "train_pairs": len(train_idx) * (args.frames - 1),
                       "flops_per_step": flops_step, "data_generation_s": round(t_data, 1)},
            "roofline": {"bound": "tensor", "achieved": round(tflops, 2), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(tflops / peak, 4), "peak_kind": peak_kind, "traffic": None},
            "loss_history": hist, "held_out": ev, "rollout_saturation_rel_error": roll,
            "accelerated_ensemble": accel,
            "jump_vs_lbm": {"members": nb, "lbm_200_iterations_ms": round(t_lbm * 1e3, 3),
                            "surrogate_jump_ms": round(t_sur * 1e3, 3), "speedup": round(t_lbm / t_sur, 2),
                            "speedup_with_judge": round(6 * t_lbm / (6 * t_sur + t_lbm), 2)},
            "gpu_launches": None, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_convs(args):
    """Every convolution shape of the surrogate's training step (forward and
    data gradient, batch `--batch` at 512 x 256): the warp-level, the tcgen05
    and (widths that are multiples of 128) the TMA-fed tcgen05 kernel timed
    with CUDA events, one JSON line per shape."""
    import ctypes as C
    import torch
    from fingering_dynamics_gb300 import _lib as L
    from fingering_dynamics_gb300 import build
    build.build()

    def p(t):
        return C.c_void_p(t.data_ptr())
    N = args.batch
    shapes = [(256, 512, 16, 32), (256, 512, 32, 32), (128, 256, 32, 64), (128, 256, 64, 64), (64, 128, 64, 128),
              (64, 128, 128, 128), (32, 64, 128, 256), (32, 64, 256, 256), (64, 128, 384, 128),
              (128, 256, 192, 64), (256, 512, 96, 32), (256, 512, 32, 16), (256, 512, 32, 96),
              (128, 256, 64, 192), (64, 128, 128, 384), (32, 64, 256, 128)]
    for (H, W, ci, co) in shapes:
        x = torch.randn(N, H, W, ci, device="cuda").to(torch.bfloat16)
        w = (0.1 * torch.randn(co, 3, 3, ci, device="cuda")).to(torch.bfloat16)
        y = torch.empty(N, H, W, co, device="cuda", dtype=torch.bfloat16)
        z = torch.empty_like(y)
        fl = 2.0 * 9 * ci * co * N * H * W
        line = {"metric": "conv3x3 throughput", "unit": "TFLOP/s", "shape": [N, H, W, ci, co]}
        for fn, key in (("sg_conv3x3", "mma"), ("sg_conv3x3_tc", "tcgen05"), ("sg_conv3x3_tma", "tma"),
                        ("sg_conv3x3_tma_ws", "tma_ws")):
            if key.startswith("tma") and W % 128:
                continue
            for _ in range(args.warmup):
                L.call(fn, p(x), N, H, W, ci, p(w), None, co, 1, p(z), p(y), None)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                L.call(fn, p(x), N, H, W, ci, p(w), None, co, 1, p(z), p(y), None)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            line[key] = {"us": round(ms * 1e3, 1), "tflops": round(fl / ms / 1e9, 1)}
        # the weight gradient of the same shape (dz = y here: same layout as the real gradient)
        nparts = max(int(L.lib().sg_wgrad_partial_floats(N, H, W, ci, co)), 8 * co * 9 * ci)
        part = torch.empty(nparts, dtype=torch.float32, device="cuda")
        dw = torch.empty(co * 9 * ci, dtype=torch.float32, device="cuda")
        for fn, key in (("sg_conv3x3_wgrad", "wgrad_mma"), ("sg_conv3x3_wgrad_tc", "wgrad_tcgen05")):
            if key == "wgrad_tcgen05" and W % 128:
                continue
            wa = (p(x), p(y), N, H, W, ci, co, p(dw), p(part), part.numel(), 0, None)
            for _ in range(args.warmup):
                L.call(fn, *wa)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                L.call(fn, *wa)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            line[key] = {"us": round(ms * 1e3, 1), "tflops": round(fl / ms / 1e9, 1)}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--dtype", default="f32", choices=sorted(BYTES_PER_LU))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rows", type=int, default=0,
                    help="strip height of the staged kernel, rows per warp of the others (0 = automatic)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end measurement")
    ap.add_argument("--no-extras", action="store_true",
                    help="single workload: skip the f16 / bf16 and ensemble sub-records of the default line")
    ap.add_argument("--e2e-chunk-rows", type=int, default=0,
                    help="e2e: rows per chunk of the pipelined host step (0: automatic)")
    ap.add_argument("--e2e-serial", action="store_true",
                    help="e2e: upload, step and download one after the other instead of the pipelined host step")
    ap.add_argument("--H", type=int, default=H_FULL, help="lattice rows (default: the 4096 x 2048 workload)")
    ap.add_argument("--W", type=int, default=W_FULL, help="lattice columns")
    ap.add_argument("--workload", default="single",
                    choices=["single", "ensemble", "precision", "surrogate", "surrogate-convs", "accelerated"],
                    help="single 4096 x 2048 lattice (default), the batched ensemble, or the error study of "
                         "reduced-precision storage against the FP64 path (1024 x 256, --steps iterations)")
    ap.add_argument("--rounding", default="stochastic", choices=["stochastic", "nearest"],
                    help="rounding of FP16/BF16 population stores")
    ap.add_argument("--every", type=int, default=500, help="precision study: iterations between comparisons")
    ap.add_argument("--out", default=None, help="precision study: write the full curves to this JSON file")
    ap.add_argument("--members", type=int, default=96, help="ensemble members (surrogate: trajectory members)")
    ap.add_argument("--frames", type=int, default=41, help="surrogate: frames per member (one per 200 iterations)")
    ap.add_argument("--train-steps", type=int, default=1000, help="surrogate: timed AdamW steps")
    ap.add_argument("--batch", type=int, default=32, help="surrogate: training batch")
    ap.add_argument("--conv", default="auto", choices=["auto", "mma", "tcgen05", "tma", "tma_ws"],
                    help="surrogate: forward / data-gradient convolution kernel (auto: the faster per shape)")
    ap.add_argument("--save-net", default=None, help="surrogate: write the trained network's weights (.npz) here")
    ap.add_argument("--load-net", default=None,
                    help="accelerated: the trained network's weights (.npz, as written by --save-net)")
    ap.add_argument("--max-rounds", type=int, default=0,
                    help="accelerated: also race plain and accelerated runs to breakthrough, at most this many "
                         "rounds of 1200 iterations (0: skip)")
    ap.add_argument("--family", default="config", choices=["config", "stable", "spec"],
                    help="ensemble parameter family (spec: the configuration's literal ranges)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.workload == "surrogate-convs":
        return run_convs(args)
    if args.workload == "accelerated":
        return run_accelerated(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
