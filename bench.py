#!/usr/bin/env python3
"""Benchmark of the StormLab model step on GB300: batched / served cell-steps/s beside the plain single-run step.

One JSON line on rank 0. A "step" is one model time step (dt = 3 s) of every run in the workload.
Headline (`value`): the batched ensemble — 64 members on the standard 40x32x50 grid, seeded
soundings, advanced together through one CUDA graph per step; inputs resident in HBM (213 MB per field set, larger
than the 129 MB L2, so no flush is needed between steps). `e2e`: the same metric through the C ABI with host
buffers: every step writes all members' fields from pinned host memory, steps, and reads them back
(sg_batch_step_round_trips over the timed steps, the members in four groups whose copies overlap the other groups'
steps; beside it one sg_batch_step_io call a step, and separate write / step / read calls).
Beside it: the plain single-run step on the standard, large (80x64x50) and stress (320x256x80) grids.
`--impl reference`: the reference's algorithm on the host cores (the oracle port) on a bounded sample of the same
workload (one member per host core, spun up like the GPU arm's), timed two ways (every step split over all threads;
one member per thread) and reported as the faster.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s batched vs plain GPU step at <=1e-5 rel-L2; serve p50/p99 s/run"
MEMBERS = 64
# Groups of the e2e leg's sg_batch_step_io call (16 members each): the fastest of 1, 2, 4 and 8 on GB300.
E2E_GROUPS = 4
# The dominant kernel: the WENO5 transport of the 9 monotone fields (rain, snow, graupel, hail, q, cloud, ice,
# iceNumber, cold), one launch per RK3 stage. Algorithmic bytes per cell and launch: each field read once and written
# once (4 + 4 B), the step-start value read in stages 2 and 3 (4 B), the projected face fluxes (mx, my, mz, div: 16 B);
# mean over the three stages = (9 * 8 + 16 + 2 * (9 * 12 + 16)) / 3.
TRANSPORT_BYTES_PER_CELL = (9 * 8 + 16 + 2 * (9 * 12 + 16)) / 3
# Algorithmic bytes per cell and launch of every kernel (FP32 fields 4 B; inputs read once, outputs written once):
# the denominators of the per-kernel HBM roofline. Spectra and solver factors per cell of the 40-wide grid: a half
# spectrum is (nx/2 + 1)/nx complex values per node (4.2 B), the sweep's FP64 factors 3 x 8 B per mode (12.6 B).
KERNEL_BYTES_PER_CELL = {
    "fall_courant": 16, "sediment": 32,                                   # 4 falling fields in (and out)
    "face_div_xfft": 12 + 4.2, "pres_div_xfft": 12 + 4.2,                 # u, v, w in; half spectrum out
    "face_modes": 8.4 + 12.6, "pres_modes": 8.4 + 12.6,                   # spectrum in and out, FP64 factors
    "face_xifft": 4.2 + 4, "pres_xifft": 4.2 + 4,                         # spectrum in, potential / pressure out
    "face_correct": 16 + 16,                                              # u, v, w, phi in; float4 faces out
    "pres_correct": 16 + 12, "pres_correct_final": 16 + 12,               # p, u, v, w in; u, v, w out
    "transport_weno": TRANSPORT_BYTES_PER_CELL,
    "transport_dynamics": (80 + 96 + 96) / 3,                             # u, v, w, theta' r/w, faces, buoyancy inputs, start values
    "fill_partial": 28, "physics": 104, "viscosity": 36, "mix": 72,
    # the final projection's refinement: the residual (u, v, w, p in; the residual out), the second solve (right-hand
    # side in), the correction (u, v, w, p1, p2 in; u, v, w out)
    "refine_residual": 16 + 4, "refine_div_xfft": 4 + 4.2, "refine_modes": 8.4 + 12.6,
    "refine_xifft": 4.2 + 4, "refine_correct": 20 + 12,
}
# Algorithmic bytes of one whole step per cell, pass by pass (each global pass reads its inputs once and writes its
# outputs once, FP32 4 B): sedimentation 32, face projection 72, RK3 transport 464, three pressure projections 252,
# positivity rescale 64, physics 104, viscosity 36, mixing and drag 72.
STEP_BYTES_PER_CELL = 32 + 72 + 464 + 252 + 64 + 104 + 36 + 72


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--members", type=int, default=MEMBERS)
    p.add_argument("--spinup", type=int, default=300, help="untimed steps before the warm-up (15 simulated minutes), so the "
                   "timed steps see a developed storm with cloud and precipitation rather than the quiescent start")
    p.add_argument("--quick", action="store_true", help="skip the serving and stress-grid legs")
    p.add_argument("--moments", type=int, default=1, choices=[1, 2],
                   help="with --ncu-window: the ensemble in the one- or two-moment configuration (two-moment rain, graupel and hail; the timed headline is one-moment)")
    p.add_argument("--ncu-window", action="store_true",
                   help="profiling driver: set up and spin up the ensemble, then run --steps eager steps between "
                        "cudaProfilerStart/Stop (for ncu --profile-from-start off) and exit without timing")
    return p.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def rank_members(grid, members: int, rank: int):
    """Replicas only: each rank steps its own ensemble, seeded by its rank; no data crosses ranks."""
    from meteolab_gb300.scenarios import ensemble_members
    return ensemble_members(grid, members, seed=2026 + rank)


def job_value(cells_per_rank: int, world: int, steps: int, ms_max: float) -> float:
    """Whole-job cell-steps/s: every rank's cells over the slowest rank's time."""
    return cells_per_rank * world * steps / (ms_max * 1e-3)


def barrier(pg):
    if pg:
        pg.barrier()


def allmax(pg, x: float) -> float:
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """SM clock and clock-event (throttle) reasons sampled during the timed region: through NVML's read-only queries
    every few milliseconds on a sampling thread (the timed call releases the GIL), so even a region of a few tens of
    milliseconds has samples; nvidia-smi at 200 ms where NVML cannot be loaded."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits (nvml.h): SW power cap, HW slowdown, SW thermal, HW thermal
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, device: int):
        self.device, self.proc, self.lines, self.first = device, None, [], 0
        self.nvml, self.samples, self.max_mhz, self.stop = None, [], None, threading.Event()

    def _nvml_open(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        handle = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.device), ctypes.byref(handle)) != 0:
            return None
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(handle, 1, ctypes.byref(mx)) == 0:  # 1: NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, handle, reasons

    def _nvml_loop(self):
        import ctypes
        lib, handle, reasons = self.nvml
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(handle, 1, ctypes.byref(clk)) == 0 and reasons(handle, ctypes.byref(rs)) == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            time.sleep(.005)

    def __enter__(self):
        try:
            self.nvml = self._nvml_open()
        except Exception:
            self.nvml = None
        if self.nvml:
            self.reader = threading.Thread(target=self._nvml_loop, daemon=True)
            self.reader.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=lambda: self.lines.extend(self.proc.stdout), daemon=True)
            self.reader.start()
            # the timed region starts once sampling has (nvidia-smi takes a moment to print its first line)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(.02)
            self.first = len(self.lines)  # samples from here on fall in the timed region
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml:
            self.stop.set()
            self.reader.join(timeout=2)
            try:
                self.nvml[0].nvmlShutdown()
            except Exception:
                pass
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()
            self.reader.join(timeout=2)

    def summary(self):
        if self.nvml:
            sm = [c for c, _ in self.samples]
            reasons = sorted(n for n, b in self.BITS.items() if any(r & b for _, r in self.samples))
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz, "reasons": reasons,
                    "samples": len(sm), "source": "nvml, 5 ms"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.first:] or self.lines[-1:]  # (a region shorter than the sampling interval: the last sample)
        for line in lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi, 200 ms"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dram_profile():
    """Per-kernel DRAM bytes and GB/s of one step from the committed ncu launch list, if there is one."""
    try:
        with open(os.path.join(ROOT, "profiles", "step_dram_ensemble64.json")) as f:
            return json.load(f)["kernels"]
    except Exception:
        return None


def traffic_per_cell():
    """DRAM bytes per cell of one transport launch from the committed ncu summary, if there is one."""
    try:
        with open(os.path.join(ROOT, "profiles", "transport_traffic.json")) as f:
            return float(json.load(f)["dram_bytes_per_cell"])
    except Exception:
        return None


def cpu_strategies(specs, steps: int, threads: int):
    """The reference's algorithm (the oracle port: FP32 fields, FP64 arithmetic, the reference's task order) on the host
    cores, two ways over the same member states, wall-clock measured:
      * "openmp": the members one after another, each step split over all threads (the reference's in-step tasks,
        src/core/threads.ts; its `npm run bench` times one run this way);
      * "pool": one member per worker thread, all at once, each single-threaded (the reference's ensemble runner,
        runPool, src/ensemble/pool.ts:19-47: one run per worker).
    Returns {strategy: (cell-steps/s, ms per step of the whole sample)}."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from concurrent.futures import ThreadPoolExecutor
    cells = sum(s.grid.n for s in specs)
    out = {}
    models = [pyoracle.OracleModel(s, threads=threads) for s in specs]
    for m in models:
        m.step(3.0, 1)  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        for m in models:
            m.step(3.0, 1)
    el = time.perf_counter() - t0
    out["openmp"] = (cells * steps / el, el * 1e3 / steps)
    models = [pyoracle.OracleModel(s, threads=1) for s in specs]
    with ThreadPoolExecutor(max_workers=len(models)) as ex:  # ctypes calls run without the GIL
        list(ex.map(lambda m: m.step(3.0, 1), models))
        t0 = time.perf_counter()
        list(ex.map(lambda m: m.step(3.0, steps), models))
        el = time.perf_counter() - t0
    out["pool"] = (cells * steps / el, el * 1e3 / steps)
    return out


def cpu_summary(strategies, threads: int, sample: str) -> dict:
    best = max(strategies, key=lambda k: strategies[k][0])
    return {"value": strategies[best][0], "unit": "cell-steps/s", "cores": threads, "kind": "port", "strategy": best,
            "strategies": {k: {"cell_steps_s": v[0], "ms_per_step": v[1]} for k, v in strategies.items()},
            "sample": sample}


def cpu_baseline(states, steps: int = 30):
    """The CPU baseline beside the GPU figures: both strategies of cpu_strategies on the GPU arm's own spun-up member
    states (the first `threads` members), `steps` steps each; and the lightning's field solve restated with numpy."""
    import numpy as np
    threads = os.cpu_count() or 1
    specs = states[:threads]
    st = cpu_strategies(specs, steps, threads)
    out = cpu_summary(st, threads, f"{len(specs)} of the ensemble's 40x32x50 members from the GPU arm's spun-up states, {steps} "
                                   f"steps per strategy; reference algorithm restated in C++ (oracle)")
    # the lightning's field solve (ElectricSolver.solve) restated with numpy's FFT, one thread, on the same grid
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import electric
    grid = specs[0].grid
    rho = np.random.default_rng(1).standard_normal(grid.n) * 1e-10
    electric.solve(grid, rho)
    k, t1 = 0, time.perf_counter()
    while time.perf_counter() - t1 < .5:
        electric.solve(grid, rho)
        k += 1
    out["electric_solve_ms"] = (time.perf_counter() - t1) / k * 1e3
    return out


def electrified_leg(ctx, members, runs, steps: int, build: int = 200, cpu_steps: int = 10):
    """Electrification and lightning on: the first 16 ensemble members as the timed steps left them (developed storms),
    electrified, their charge built over `build` untimed steps; then `steps` timed steps of the batch (device work and
    the host-stepped flash stages included) beside the same states without electrification; flashes counted from the
    runs' charge budgets. CPU: the oracle with lightning on from the same states (charges included), pool strategy."""
    import dataclasses
    from meteolab_gb300.scenarios import CARRIED, CHARGES, RunSpec
    k = min(16, len(runs))
    base = [RunSpec(m.grid, m.env, m.switches, r.read(), m.seed, m.label) for m, r in zip(members[:k], runs[:k])]
    elec = [RunSpec(s.grid, s.env, dataclasses.replace(s.switches, lightning=1), s.fields, s.seed, s.label) for s in base]
    er = [ctx.create(s) for s in elec]
    ctx.time_steps(er, build)
    before = [r.charge() for r in er]
    ms = ctx.time_steps(er, steps)
    after = [r.charge() for r in er]
    flashes = sum(a["flashes_ic"] + a["flashes_cg"] - b["flashes_ic"] - b["flashes_cg"] for a, b in zip(after, before))
    cg = sum(a["flashes_cg"] - b["flashes_cg"] for a, b in zip(after, before))
    total_flashes = sum(a["flashes_ic"] + a["flashes_cg"] for a in after)
    states = [RunSpec(s.grid, s.env, s.switches, r.read(list(CARRIED) + list(CHARGES)), s.seed, s.label) for s, r in zip(elec, er)]
    for r in er:
        r.retire()
    pr = [ctx.create(s) for s in base]
    ctx.time_steps(pr, 3)
    ms_plain = ctx.time_steps(pr, steps)
    for r in pr:
        r.retire()
    cells = sum(s.grid.n for s in elec)
    threads = os.cpu_count() or 1
    cpu = cpu_strategies(states[:threads], cpu_steps, threads)
    best = max(cpu, key=lambda key: cpu[key][0])
    return {"members": k, "grid": "40x32x50", "charge_build_steps": build, "timed_steps": steps,
            "ms_per_step": ms / steps, "cell_steps_s": cells * steps / (ms * 1e-3),
            "without_lightning_ms_per_step": ms_plain / steps, "flashes_timed": flashes, "cg_flashes_timed": cg,
            "flashes_since_electrified": total_flashes,
            "cpu_baseline": {"value": cpu[best][0], "unit": "cell-steps/s", "cores": threads, "kind": "port", "strategy": best,
                             "sample": f"the same {min(threads, k)} electrified member states, {cpu_steps} steps, oracle with lightning on"}}


def two_moment_specs(members, runs):
    """The ensemble's members as the timed steps left them, in the reference's two-moment configuration (SimConfig.moments
    2: two-moment rain, graupel and hail, src/core/model.ts:331): the drop number started as the reference starts rain
    without one (Marshall-Palmer's), graupel's and hail's number and volume as the one-moment classes of the same mass."""
    import dataclasses
    import numpy as np
    from meteolab_gb300.scenarios import RunSpec, exponential_ice_moments, marshall_palmer_number
    specs = []
    for m, r in zip(members, runs):
        f = r.read()
        rho = np.repeat(np.asarray(m.env.rho), m.grid.layer)
        f["rainNumber"] = marshall_palmer_number(f["rain"], rho)
        for kind in ("graupel", "hail"):
            f[kind + "Number"], f[kind + "Volume"] = exponential_ice_moments(f[kind], rho, kind)
        specs.append(RunSpec(m.grid, m.env, dataclasses.replace(m.switches, rain_moments=2, ice_moments=2), f, m.seed, m.label))
    return specs


def two_moment_leg(ctx, members, runs, steps: int, cpu_steps: int = 10):
    """The two-moment configuration (two_moment_specs) of the ensemble: `steps` timed graph steps of the whole batch
    beside its one-moment steps; CPU: the oracle in the same configuration from the same states, pool strategy."""
    from meteolab_gb300.scenarios import RunSpec
    specs = two_moment_specs(members, runs)
    tr = [ctx.create(s) for s in specs]
    ctx.time_steps(tr, 5)
    ms = ctx.time_steps(tr, steps)
    prof = ctx.profile(tr, 2)
    cells = sum(s.grid.n for s in specs)
    states = [RunSpec(s.grid, s.env, s.switches, r.read(list(s.fields)), s.seed, s.label) for s, r in zip(specs, tr)]
    for r in tr:
        r.retire()
    threads = os.cpu_count() or 1
    cpu = cpu_strategies(states[:threads], cpu_steps, threads)
    best = max(cpu, key=lambda key: cpu[key][0])
    return {"members": len(specs), "grid": "40x32x50", "config": "SimConfig.moments 2: two-moment rain, graupel and hail",
            "timed_steps": steps, "ms_per_step": ms / steps,
            "cell_steps_s": cells * steps / (ms * 1e-3),
            "kernels_ms_per_launch": {k: round(v[0], 5) for k, v in prof.items()},
            "cpu_baseline": {"value": cpu[best][0], "unit": "cell-steps/s", "cores": threads, "kind": "port", "strategy": best,
                             "sample": f"{min(threads, len(states))} of the members, {cpu_steps} steps, oracle in the two-moment configuration"}}


def reference_arm(args, rank, pg):
    """--impl reference: the reference's algorithm on the host cores (the oracle port; no GPU, none of this package's
    device code) on a bounded sample of the workload: the first `threads` members of the same seeded 64-member ensemble,
    spun up --spinup steps in the pool strategy (untimed), then W warm-up and K timed steps in each strategy of
    cpu_strategies; the faster is the line's value. ms_per_step is the measured wall time of one step of the sample."""
    if rank != 0:
        return
    from meteolab_gb300.grid import DEFAULT_GRID, create_grid
    from meteolab_gb300.scenarios import CARRIED, RunSpec, ensemble_members
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from concurrent.futures import ThreadPoolExecutor
    threads = os.cpu_count() or 1
    grid = create_grid(DEFAULT_GRID)
    members = ensemble_members(grid, args.members, seed=2026)[:min(threads, args.members)]
    if args.spinup:  # the GPU arm's spun-up state: storms with cloud and precipitation
        models = [pyoracle.OracleModel(s, threads=1) for s in members]
        with ThreadPoolExecutor(max_workers=len(models)) as ex:
            list(ex.map(lambda m: m.step(3.0, args.spinup), models))
        members = [RunSpec(s.grid, s.env, s.switches, {k: m.get(k).astype("float32") for k in CARRIED}, s.seed, s.label)
                   for s, m in zip(members, models)]
        del models
    if args.warmup:
        cpu_strategies(members, max(1, args.warmup // 2), threads)
    st = cpu_strategies(members, args.steps, threads)
    cpu = cpu_summary(st, threads, f"{len(members)} of the {args.members} ensemble members (40x32x50), spun up {args.spinup} steps, "
                                   f"{args.steps} timed steps per strategy; reference algorithm restated in C++ (oracle)")
    value = cpu["value"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": cpu["strategies"][cpu["strategy"]]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded soundings, ellipsoid bubble)",
            "config": {"workload": f"ensemble {args.members} x 40x32x50, sampled: the first {len(members)} members, "
                                   f"all of them every timed step", "cores": threads, "spinup_steps": args.spinup},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def terrain_leg(ctx, grid, calls: int = 10):
    """The terrain's two masked solves on the standard grid over a 1 km hill (5 km half-width), a 10 +- 2 m/s westerly
    with random vertical motion: MaskedProjection.project (the pressure, to 1e-6) and the transport's
    setVelocityMasked (the faces, to 1e-10), each one call with its host copies; median wall time of `calls` calls
    after one warm-up, with the iterations each took."""
    import numpy as np
    from meteolab_gb300.runtime import MaskedProjection, TerrainFaces, terrain_heights
    try:
        h = terrain_heights({"kind": "hill", "height": 1, "width": 5}, grid)
        rho = 1.2 * np.exp(-np.asarray(grid.zs) / 9000)
        rng = np.random.default_rng(1)
        u0 = (10 + rng.normal(0, 2, grid.n)).astype(np.float32)
        v0 = rng.normal(0, 2, grid.n).astype(np.float32)
        w0 = rng.normal(0, 1, grid.n).astype(np.float32)
        cells = grid.nx * grid.ny * (grid.nz - 1)
        m, f = MaskedProjection(ctx, grid, rho, h), TerrainFaces(ctx, grid, rho, h)
        proj, faces = [], []
        for k in range(calls + 1):
            u, v, w, p = u0.copy(), v0.copy(), w0.copy(), np.zeros(cells)
            t0 = time.perf_counter()
            m.project(u, v, w, 3.0, p)
            proj.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            f.set_velocity_masked(u0, v0, w0)
            faces.append(time.perf_counter() - t0)
        out = {"grid": "40x32x50", "form": "hill 1 km, half-width 5 km",
               "projection": {"ms_per_call": 1e3 * float(np.median(proj[1:])), "iterations": m.iterations, "residual": m.residual},
               "faces": {"ms_per_call": 1e3 * float(np.median(faces[1:])), "iterations": f.iterations, "residual": f.residual}}
        m.close(); f.close()
        return out
    except Exception as e:  # the headline does not depend on this leg
        return {"error": str(e)}


def serving_leg(ctx, rate: float, count: int, quantum: int):
    """The serving configuration: an open Poisson stream of requests (seeded soundings, standard or large grid 3:1,
    400-1200 steps) through the continuous-batching loop. Time-to-completion runs from a request's arrival to its
    collected result; per-step latency is an iteration's wall time over the steps it advanced."""
    import numpy as np
    from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, create_grid
    from meteolab_gb300.runtime import Server
    from meteolab_gb300.scenarios import serving_requests
    reqs = serving_requests(create_grid(DEFAULT_GRID), create_grid(LARGE_GRID), count, rate)
    srv = Server(ctx, max_active=256)
    srv.set_quantum(quantum)
    done_at, step_ms, cells_steps = {}, [], 0
    nxt, active, queued = 0, 0, 0
    t0 = time.perf_counter()
    while len(done_at) < count:
        now = time.perf_counter() - t0
        while nxt < count and reqs[nxt][0] <= now:
            _, spec, steps = reqs[nxt]
            srv.submit(spec, steps, nxt)
            nxt += 1
        if active or queued or nxt > len(done_at) + active:
            ts = time.perf_counter()
            tags, active, queued = srv.iterate()
            te = time.perf_counter()
            k = srv.last_steps
            if k:
                step_ms.append((te - ts) * 1e3 / k)
            for t in tags:
                srv.collect(t, reqs[t][1].grid.n)
                done_at[t] = time.perf_counter() - t0
                cells_steps += reqs[t][1].grid.n * reqs[t][2]
        else:
            time.sleep(max(0.0, min(0.01, reqs[nxt][0] - now)))
    wall = time.perf_counter() - t0
    srv.close()
    ttc = np.array([done_at[t] - reqs[t][0] for t in range(count)])
    return {"rate_per_s": rate, "requests": count, "quantum_steps": quantum, "wall_s": wall,
            "p50_s": float(np.percentile(ttc, 50)), "p99_s": float(np.percentile(ttc, 99)),
            "step_latency_p50_ms": float(np.percentile(step_ms, 50)), "step_latency_p99_ms": float(np.percentile(step_ms, 99)),
            "cell_steps_s": cells_steps / wall}


def uneven_leg(ctx, steps: int, spinup: int):
    """48 standard + 16 large runs of a CAPE x shear regime grid in the same launches."""
    from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, create_grid
    from meteolab_gb300.scenarios import regime_runs
    specs = regime_runs(create_grid(DEFAULT_GRID), create_grid(LARGE_GRID))
    runs = [ctx.create(s) for s in specs]
    if spinup:
        ctx.time_steps(runs, spinup)
        ctx.set_transport_shape(0)  # tuned on the developed storms
    ctx.time_steps(runs, 3)
    ms = ctx.time_steps(runs, steps)
    cells = sum(r.grid.n for r in runs)
    tile = ctx.transport_shape(runs)
    # each size alone (its own plan, graph and tuned tile), from the same states: the per-size throughput, and what
    # mixing the sizes in one launch costs or saves
    alone = {}
    for name, nx in (("standard", 40), ("large", 80)):
        part = [r for r in runs if r.grid.nx == nx]
        ctx.time_steps(part, 3)
        pms = ctx.time_steps(part, steps)
        alone[name] = {"runs": len(part), "cell_steps_s": sum(r.grid.n for r in part) * steps / (pms * 1e-3),
                       "ms_per_step": pms / steps}
    for r in runs:
        r.retire()
    v = cells * steps / (ms * 1e-3)
    # Work items are per run, so no run is padded to another's size; the transport tiles overhang no grid edge
    # when the tile width divides the grid widths.
    waste = 0.0 if all(nx % tile[0] == 0 and ny % tile[1] == 0 for nx, ny in ((40, 32), (80, 64))) else None
    capes = [s.meta["cape"] for s in specs]
    return {"runs": "48 x 40x32x50 + 16 x 80x64x50", "cell_steps_s": v, "ms_per_step": ms / steps,
            "regime": {"ml_cape_j_per_kg": {"min": min(capes), "max": max(capes)},
                       "points": [[s.label, s.grid.nx, round(s.meta["cape"]), round(s.meta["shear"], 1), round(s.meta["lid_k"], 2),
                                   round(s.meta["lid_km"], 2)] for s in specs],
                       "point_fields": ["label", "nx", "ml_cape", "shear06", "lid_K", "lid_km"]},
            "alone": alone, "mixed_vs_sizes_alone": (alone["standard"]["ms_per_step"] + alone["large"]["ms_per_step"]) / (ms / steps),
            "padding_waste": waste, "transport_tile": list(tile)}


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        reference_arm(args, rank, pg)
        return
    from meteolab_gb300 import build
    build.build()
    import numpy as np
    import torch
    from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, STRESS_GRID, create_grid
    from meteolab_gb300.runtime import Context
    from meteolab_gb300.scenarios import CARRIED, baseline_run, ensemble_members

    ctx = Context(local)
    grid = create_grid(DEFAULT_GRID)
    members = rank_members(grid, args.members, rank)
    runs = [ctx.create(s) for s in members]
    cells = sum(r.grid.n for r in runs)

    # ---- headline: the batched ensemble from its CUDA graph, device time, inputs resident
    if args.spinup:
        ctx.time_steps(runs, args.spinup)
        ctx.set_transport_shape(0)  # tune the transport again, on the developed storms rather than the quiescent start
    if args.ncu_window:
        if args.moments == 2:  # the same states in the two-moment configuration (two_moment_specs)
            specs = two_moment_specs(members, runs)
            for r in runs:
                r.retire()
            runs = [ctx.create(s) for s in specs]
        ctx.time_steps(runs, 1, graph=False)  # plans and tuning outside the window
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        ctx.time_steps(runs, args.steps, graph=False)
        torch.cuda.profiler.stop()
        print(json.dumps({"ncu_window": True, "members": args.members, "steps": args.steps, "transport_tile": ctx.transport_shape(runs)}))
        return
    ctx.time_steps(runs, max(3, args.warmup))
    barrier(pg)
    with Clocks(local) as clk:
        ms = ctx.time_steps(runs, args.steps)
    ms = allmax(pg, ms)
    value = job_value(cells, world, args.steps, ms)

    tile = ctx.transport_shape(runs)
    bulk = ctx.transport_bulk(runs)
    # ---- kernel profile (eager, CUDA events per launch) and the roofline of the transport
    prof = ctx.profile(runs, 2)
    hbm, peak_kind = peaks()
    tr_ms = prof.get("transport_weno", (None, 0))[0]
    achieved = cells * TRANSPORT_BYTES_PER_CELL / (tr_ms * 1e-3) / 1e9 if tr_ms else None
    tpc = traffic_per_cell()
    launches_per_step = sum(v[1] for v in prof.values())

    # ---- e2e through the C ABI with a pinned host buffer: all fields of all runs written from it, one step, all read
    # back into it, every step. Headline: sg_batch_step_round_trips over the timed steps (the runs in E2E_GROUPS groups
    # whose copies overlap the other groups' steps, pipelined across steps); beside it one sg_batch_step_io call a step
    # and the same round trip as three separate calls (write, step, read).
    packed = torch.empty(cells * len(CARRIED), dtype=torch.float32, pin_memory=True).numpy()
    ctx.read_packed(runs, packed)
    def e2e_serial():
        ctx.write_packed(runs, packed)
        ctx.batch_step(runs, 1, wait=False)
        ctx.read_packed(runs, packed)
    def e2e_io():
        ctx.batch_step_io(runs, packed, steps=1, groups=E2E_GROUPS)
    e2e_n = max(3, args.steps // 4)
    e2e_values = {}
    for name, fn in (("io", e2e_io), ("serial", e2e_serial)):
        for _ in range(2):
            fn()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(e2e_n):
            fn()
        e2e_s = allmax(pg, time.perf_counter() - t0)
        e2e_values[name] = cells * world * e2e_n / e2e_s
    # the same round trip every step, e2e_n steps in one call: the groups pipeline across steps
    ctx.batch_round_trips(runs, packed, steps=2, groups=E2E_GROUPS)
    barrier(pg)
    t0 = time.perf_counter()
    ctx.batch_round_trips(runs, packed, steps=e2e_n, groups=E2E_GROUPS)
    e2e_s = allmax(pg, time.perf_counter() - t0)
    e2e_values["round_trips"] = cells * world * e2e_n / e2e_s
    e2e_value = e2e_values["round_trips"]
    bytes_io = cells * 4 * len(CARRIED)

    # ---- plain single-run steps (eager launches and from a graph) on the standard, large and stress grids
    plain = {}
    for name, opts in (("standard", DEFAULT_GRID), ("large", LARGE_GRID)) + ((("stress", STRESS_GRID),) if not args.quick else ()):
        spec = baseline_run(create_grid(opts), seed=3)
        r = ctx.create(spec)
        if args.spinup:
            ctx.time_steps([r], args.spinup)
            ctx.set_transport_shape(0)  # tuned on the developed storm
        ctx.time_steps([r], 3, graph=False)
        n = max(5, args.steps // 2)
        eager = ctx.time_steps([r], n, graph=False)
        ctx.time_steps([r], 3)
        graphed = ctx.time_steps([r], n)
        plain[name] = {"cells": spec.grid.n, "eager_cell_steps_s": spec.grid.n * n / (eager * 1e-3),
                       "graph_cell_steps_s": spec.grid.n * n / (graphed * 1e-3), "graph_ms_per_step": graphed / n}
        r.retire()

    # ---- the lightning's field solve (ElectricSolver) on the standard grid: one call with its host copies (FP64 in,
    # FP64 out), wall time per solve
    from meteolab_gb300.runtime import ElectricSolver
    es = ElectricSolver(ctx, grid)
    rho = np.random.default_rng(1).standard_normal(grid.n) * 1e-10
    phi = np.empty_like(rho)
    for _ in range(5):
        es.solve(rho, phi)
    t0, k = time.perf_counter(), 100
    for _ in range(k):
        es.solve(rho, phi)
    electric_ms = (time.perf_counter() - t0) / k * 1e3
    es.close()

    terrain = terrain_leg(ctx, grid)

    uneven = uneven_leg(ctx, max(5, args.steps // 2), args.spinup)
    electrified = electrified_leg(ctx, members, runs, max(10, args.steps // 4)) if rank == 0 else None
    two_moment = two_moment_leg(ctx, members, runs, max(10, args.steps // 4)) if rank == 0 else None
    serving = None if args.quick else serving_leg(ctx, rate=4.0, count=32, quantum=10)
    # the serving configuration's range of arrival rates (0.5 to 8 runs/s), each with about 8-12 s of arrivals
    serving_rates = None if args.quick else [serving_leg(ctx, rate=r, count=c, quantum=10) for r, c in ((0.5, 6), (2.0, 16), (8.0, 64))]
    # the CPU baseline on the ensemble's states as the timed GPU steps left them (developed storms)
    cpu = None
    if rank == 0:
        from meteolab_gb300.scenarios import RunSpec
        k = min(os.cpu_count() or 1, len(runs))
        states = [RunSpec(m.grid, m.env, m.switches, r.read(), m.seed, m.label) for m, r in zip(members[:k], runs[:k])]
        cpu = cpu_baseline(states)
    for r in runs:
        r.retire()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Weisman-Klemp-type soundings (surface qv 11-16 g/kg, 0-6 km shear 0-30 m/s, veering 0-90 deg), "
                "1-3 K ellipsoid bubble, +-0.1 K noise below 1 km",
        "config": {"workload": f"ensemble {args.members} x 40x32x50 per GPU, one CUDA graph per step", "cells_per_gpu": cells,
                   "spinup_steps": args.spinup, "transport_tile": {"x": tile[0], "y": tile[1], "weno_fields_per_item": tile[2], "weno_blocks_per_sm": tile[3]},
                   "transport_copies": "TMA bulk copies by two producer warps" if bulk else "per-thread cp.async",
                   "l2": "inputs larger than L2 (213 MB per field set)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "cell-steps/s", "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                "call": f"sg_batch_step_round_trips, {e2e_n} steps a call, every step's fields written from and read back to "
                        f"pinned host memory, {E2E_GROUPS} groups", "call_a_step_value": e2e_values["io"],
                "serial_calls_value": e2e_values["serial"]},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm if achieved else None,
                     "traffic": tpc * cells if tpc else None, "kernel": "k_transport<WENO> (9 fields, one RK3 stage)", "peak_kind": peak_kind,
                     "bytes_per_cell_per_launch": TRANSPORT_BYTES_PER_CELL},
        "step_roofline": {"bytes_per_cell_step": STEP_BYTES_PER_CELL, "achieved": value / world * STEP_BYTES_PER_CELL / 1e9,
                          "peak": hbm, "unit": "GB/s", "frac": value / world * STEP_BYTES_PER_CELL / 1e9 / hbm},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "plain_single_run": plain,
        "batched_vs_plain_standard": value / world / plain["standard"]["graph_cell_steps_s"],
        "uneven_batch": uneven,
        "electric_solve": {"grid": "40x32x50", "ms_per_solve": electric_ms, "host_io_bytes": 2 * grid.n * 8},
        "terrain": terrain,
        "electrified": electrified,
        "two_moment": two_moment,
        "serving": serving,
        "serving_rates": serving_rates,
        "kernels_ms_per_launch": {k: round(v[0], 5) for k, v in prof.items()},
        # each kernel's algorithmic bytes over its event-timed launch (L2 hits can put a kernel above its DRAM rate)
        "kernels_algorithmic_gbs": {k: round(cells * KERNEL_BYTES_PER_CELL[k] / (v[0] * 1e-3) / 1e9, 1)
                                    for k, v in prof.items() if k in KERNEL_BYTES_PER_CELL and v[0] > 0},
        # the measured DRAM bytes and GB/s of every kernel (ncu, profiles/step_launches_ensemble64.md)
        "kernels_dram_ncu": dram_profile(),
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
