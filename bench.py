#!/usr/bin/env python3
"""Benchmark of the GB300 2D Barnes-Hut step (one JSON line on rank 0).

Workload: 2D-projected Plummer sphere, N = 2^20, a = 1, M = 1, equal masses,
eps = 0.01, dt = 1e-4, theta = 0.5 (seeded synthetic input).  A "step" is one
full pass of the pipeline: box, keys, radix sort, reorder, tree, moments,
force walk fused with the integration.

  value   steps/s of the MIXED engine (quadrupole walk, compensated sums,
          hi/lo positions) replayed as a CUDA graph, inputs resident in HBM,
          CUDA events per step, L2 flushed between timed steps.
  e2e     the same metric through the C ABI with host buffers: every step
          copies in from pinned host memory the state the reference's reset()
          uploads (x, y, vx, vy, ax, ay, mass), steps, and reads the
          positions back.
  roofline  the force walk (k_walk_acc alone) against the measured FP32 FMA
          peak, 14 flops per body-node interaction; the executed count with
          quadrupole cells at 33 flops beside it, and per-phase HBM fractions.
  reference_mode  the reference's own walk rule (monopole warp vote) on the
          GPU, same workload: the like-for-like figure for the reference arm.
  dropin  the reference's own update() order through the nine drop-in
          wrappers (Particle_cuda.cuh) on arrays of its layout, same workload.
  ensemble  256 systems, N log-uniform in [2^10, 2^17]: the batched MIXED
          engine against one PLAIN handle per system.

--impl reference times the reference's algorithm on the host cores (the CPU
restatement in oracle/, the reference having no CPU path) on the same
workload.  With torchrun (N > 1) every rank runs an independent replica.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s & interactions/s, N=2^20 Plummer θ=0.5, mixed vs plain FP32 at ≤1e-3 err"
WORKLOAD = "plummer2d_2^20"
N_BODIES = 1 << 20
EPS = 0.01
DT = 1e-4
THETA = 0.5
# kernels of one replayed step at 2^20: keys, 3 x (hist, scan, scatter), fixup, reorder,
# build, moments, records, frontier, walk (the box is the one the last walk folded; the
# full-sort fallback sits behind a conditional node that these inputs never switch on; no
# bootstrap pass after the first step)
LAUNCHES_PER_STEP = 17


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def wait_first_sample(self, timeout=5.0):
        """Block until nvidia-smi has written its first sample (it takes a
        moment to start), so that the samples cover the region that follows."""
        t0 = time.perf_counter()
        while self.proc and time.perf_counter() - t0 < timeout:
            if os.path.getsize(self.path) > 0:
                return
            time.sleep(0.02)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v == "Active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])),
                "sm_max_mhz": float(max(r[1] for r in rows)),
                "power_w_max": float(max(r[2] for r in rows)),
                "samples": len(rows), "reasons": reasons}


def run_engine(args):
    import torch

    from stellarsolver_gb300 import bh, models, roofline

    world, rank, local = dist_init()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    sp = ctypes_stream(stream)
    hbm_peak, hbm_kind = roofline.hbm_peak()

    x, y, vx, vy, m = models.plummer(N_BODIES, models.SEED_BASE + 1)
    n = len(x)
    eps2 = EPS * EPS
    common = dict(theta=THETA, eps2=eps2, gravity=1.0, timestep=DT, dampening=1.0,
                  leaf_bucket=args.bucket)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def timed_steps(s, k):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(k)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            s.step(1, sp)
            b.record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / 1e3

    result = {}
    # ---------------------------------------------------------------- force error
    idx = np.sort(np.random.default_rng(7).choice(n, size=4096, replace=False)).astype(np.int32)
    errors = {}
    inter = {}
    for mode in ("mixed", "plain"):
        with bh.BarnesHutSystem(n, device=local, mode=mode, **common) as s:
            s.set_state(x, y, vx, vy, m)
            if mode == "mixed":
                rx, ry = s.direct_sum_f64(idx)
            s.step(1)
            s.sync()
            ax, ay = s.get_accel()
            inter[mode] = s.stats()["interactions"]
        rel = np.hypot(ax[idx] - rx, ay[idx] - ry) / np.hypot(rx, ry)
        errors[mode] = {"rms_rel": float(np.sqrt(np.mean(rel ** 2))), "max_rel": float(rel.max())}

    # ---------------------------------------------------------------- steps/s
    sysm = bh.BarnesHutSystem(n, device=local, mode=args.mode, use_graph=True, **common)
    sysm.set_state(x, y, vx, vy, m)
    tuned = None
    if not args.no_autotune and args.mode != "reference":
        tuned = sysm.autotune(sp)
    for _ in range(args.warmup):
        sysm.step(1, sp)
    sysm.sync(sp)
    barrier()

    def hold_load(seconds):
        """Untimed graph steps for `seconds` (clock samples under load)."""
        t_end = time.perf_counter() + seconds
        while time.perf_counter() < t_end:
            for _ in range(20):
                sysm.step(1, sp)
            torch.cuda.synchronize()

    with ClockSampler(local) as clk:
        # the timed steps last a few tens of ms, less than the 200 ms sampling
        # period: the samples span a window of load around them
        clk.wait_first_sample()
        hold_load(0.5)
        sysm.sync(sp)
        st0 = sysm.get_state()
        barrier()
        t_wall0 = time.perf_counter()
        secs = timed_steps(sysm, args.steps)
        t_wall = time.perf_counter() - t_wall0
        barrier()
        sysm.sync(sp)
        st1 = sysm.get_state()
        hold_load(0.3)
    stats = sysm.stats()
    clocks = clk.summary()
    clocks["window"] = "0.5 s of untimed steps, the timed steps, 0.3 s of untimed steps"
    if world > 1:
        t = torch.tensor([secs], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        secs = float(t.item())
    value = world * args.steps / secs
    ms_per_step = 1e3 * secs / args.steps
    p0 = np.array([np.sum(st0["m"].astype(np.float64) * st0["vx"]),
                   np.sum(st0["m"].astype(np.float64) * st0["vy"])])
    p1 = np.array([np.sum(st1["m"].astype(np.float64) * st1["vx"]),
                   np.sum(st1["m"].astype(np.float64) * st1["vy"])])
    pscale = float(np.sum(st0["m"].astype(np.float64) * np.hypot(st0["vx"], st0["vy"])))

    # plain FP32 side by side: graph replay, and the single-system path without a graph
    sides = {}
    for label, kw in (("plain_graph", dict(mode="plain", use_graph=True)),
                      ("plain_single_system_nograph", dict(mode="plain", use_graph=False))):
        with bh.BarnesHutSystem(n, device=local, **kw, **common) as s:
            s.set_state(x, y, vx, vy, m)
            for _ in range(args.warmup):
                s.step(1, sp)
            s.sync(sp)
            sides[label] = args.steps / timed_steps(s, args.steps)

    # ---------------------------------------------------------------- per-phase roofline
    phase_ms = np.zeros(bh.PHASES_N, np.float32)
    prof_steps = max(3, min(args.steps, 10))
    for _ in range(prof_steps):
        flush.zero_()
        sysm.step_profiled(phase_ms, sp)
    phase_ms /= prof_steps
    sysm.sync(sp)
    walk_ms = float(phase_ms[bh.PHASES.index("walk")])  # k_walk_acc alone
    peaks = bh.measure_fp32_peaks(local)
    fp32_peak = max(peaks.values())
    walk_flops = roofline.walk_flops(stats)  # 14 per interaction
    walk_flops_mp = roofline.walk_flops_with_multipole(stats)
    achieved = walk_flops / (walk_ms * 1e-3) / 1e12
    achieved_mp = walk_flops_mp / (walk_ms * 1e-3) / 1e12
    traffic = recorded_traffic("walk")
    pb = roofline.phase_bytes(n, args.mode == "mixed", passes=roofline.high_passes(n),
                              accuracy=args.mode != "reference")
    phases = {}
    for i, name in enumerate(bh.PHASES):
        ms = float(phase_ms[i])
        entry = {"ms": round(ms, 4)}
        if name in pb:
            gbs = pb[name] / (ms * 1e-3) / 1e9 if ms > 0 else None
            entry.update({"algorithmic_bytes": pb[name], "GB/s": round(gbs, 1) if gbs else None,
                          "frac_hbm": round(gbs / hbm_peak, 4) if gbs else None})
        phases[name] = entry

    # ---------------------------------------------------------------- e2e through the C ABI
    e2e = run_e2e(bh, torch, stream, sp, n, x, y, vx, vy, m, sysm.params, local, args)
    sysm.close()
    # the reference's own rule on the GPU (REFERENCE mode: monopole warp-vote walk,
    # the interaction set of kernels.cu:340-435), same workload, graph replay: the
    # like-for-like figure beside the --impl reference arm
    with bh.BarnesHutSystem(n, device=local, mode="reference", use_graph=True, **common) as s:
        s.set_state(x, y, vx, vy, m)
        for _ in range(args.warmup):
            s.step(1, sp)
        s.sync(sp)
        ref_secs = timed_steps(s, args.steps)
        ref_inter = s.stats(sp)["interactions"]
    reference_mode = {"steps_per_s": round(args.steps / ref_secs, 3),
                      "ms_per_step": round(1e3 * ref_secs / args.steps, 4),
                      "interactions_per_step": ref_inter,
                      "rule": "reference warp vote (monopole, kernels.cu:395-411), CUDA graph, "
                              "L2 flushed before every timed step"}
    # the drop-in path: the reference's own update() order through the nine
    # C-linkage wrappers on arrays of its layout (m = 2n + 12000), same workload
    dropin = run_dropin(torch, stream, sp, flush, n, x, y, vx, vy, m, args)
    ens = None
    if not args.no_ensemble:
        ens = run_ensemble(bh, torch, stream, sp, local, world, rank, args)

    result = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded 2D Plummer, models.plummer)",
        "config": {"workload": WORKLOAD, "n_bodies": n, "theta": THETA, "eps": EPS, "dt": DT,
                   "mode": args.mode, "walk_shape": tuned or "defaults", "cuda_graph": True,
                   "l2": "flushed (256 MB write) before every timed step",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "timed_wall_s_incl_flush": round(t_wall, 3)},
        "interactions_per_step": stats["interactions"],
        "cell_interactions_per_step": stats["cell_interactions"],
        "walk_flops_per_step": walk_flops,
        "walk_flops_with_multipole_per_step": walk_flops_mp,
        "interactions_per_s": round(stats["interactions"] * value / world, 1) * world,
        "force_error_vs_fp64": errors,
        "plain_fp32": {"steps_per_s_graph": round(sides["plain_graph"], 3),
                       "steps_per_s_single_system_nograph":
                           round(sides["plain_single_system_nograph"], 3),
                       "interactions_per_step": inter["plain"]},
        "mixed_over_plain_single_system": round(value / world / sides["plain_single_system_nograph"], 3),
        "reference_mode": reference_mode,
        "dropin": dropin,
        "momentum_drift_rel": float(np.abs(p1 - p0).max() / pscale),
        "tree": {"cells": stats["cells"], "nodes": stats["nodes"], "max_depth": stats["max_depth"]},
        "roofline": {"bound": "fp32", "kernel": "k_walk_acc", "achieved": round(achieved, 3),
                     "peak": round(fp32_peak, 2), "unit": "TFLOP/s",
                     "frac": round(achieved / fp32_peak, 4),
                     "flops_per_interaction": roofline.FLOPS_P2P,
                     "walk_ms": round(walk_ms, 4),
                     "rule": "achieved = 14 flops x interactions_per_step / walk_ms "
                             "(k_walk_acc alone, CUDA events on its stream)",
                     "achieved_with_multipole": round(achieved_mp, 3),
                     "frac_with_multipole": round(achieved_mp / fp32_peak, 4),
                     "peak_source": "measured in-process: max of FFMA and FFMA2 chain probes "
                                    "(bh_measure_fp32_peaks)",
                     "peak_probes": {k: round(v, 2) for k, v in peaks.items()},
                     "traffic": traffic, "phases": phases,
                     "hbm_peak_gbs": hbm_peak, "hbm_peak_source": hbm_kind},
        "e2e": e2e,
        "ensemble": ens,
        "gpu_launches": LAUNCHES_PER_STEP * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(x, y, vx, vy, m)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def ctypes_stream(stream):
    import ctypes

    return ctypes.c_void_p(stream.cuda_stream)


def recorded_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary (None until captured)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(WORKLOAD, {}).get(kernel)
    except Exception:
        return None


def run_e2e(bh, torch, stream, sp, n, x, y, vx, vy, m, params, local, args):
    pin = {k: torch.from_numpy(v.copy()).pin_memory() for k, v in
           (("x", x), ("y", y), ("vx", vx), ("vy", vy), ("m", m))}
    outx = torch.empty(n, dtype=torch.float32).pin_memory()
    outy = torch.empty(n, dtype=torch.float32).pin_memory()
    ptr = {k: v.data_ptr() for k, v in pin.items()}
    lib = bh.lib()
    with bh.BarnesHutSystem(n, device=local, mode=args.mode, use_graph=True,
                            theta=params.theta, eps2=params.eps2, gravity=params.gravity,
                            timestep=params.timestep, dampening=params.dampening,
                            leaf_bucket=params.leaf_bucket, block_size=params.block_size,
                            stack_depth=params.stack_depth, alpha=params.alpha,
                            bodies_per_lane=params.bodies_per_lane) as s:
        # the accelerations of the uploaded state: one step from it, then
        # bh_get_accel (the |a| that step computed at the uploaded positions)
        pin["ax"] = torch.empty(n, dtype=torch.float32).pin_memory()
        pin["ay"] = torch.empty(n, dtype=torch.float32).pin_memory()
        ptr["ax"], ptr["ay"] = pin["ax"].data_ptr(), pin["ay"].data_ptr()
        rc = lib.bh_set_state(s.handle, ptr["x"], ptr["y"], ptr["vx"], ptr["vy"], ptr["m"], sp)
        rc |= lib.bh_step(s.handle, 1, sp)
        rc |= lib.bh_get_accel(s.handle, ptr["ax"], ptr["ay"], sp)
        s.sync(sp)
        if rc:
            raise RuntimeError(f"e2e C-ABI call failed: {rc}")

        def one():
            rc = lib.bh_set_state(s.handle, ptr["x"], ptr["y"], ptr["vx"], ptr["vy"], ptr["m"], sp)
            rc |= lib.bh_set_accel(s.handle, ptr["ax"], ptr["ay"], sp)
            rc |= lib.bh_step(s.handle, 1, sp)
            rc |= lib.bh_get_state(s.handle, outx.data_ptr(), outy.data_ptr(), None, None, None, sp)
            if rc:
                raise RuntimeError(f"e2e C-ABI call failed: {rc}")

        for _ in range(args.warmup):
            one()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            one()
        b.record(stream)
        torch.cuda.synchronize()
        secs = a.elapsed_time(b) / 1e3
        s.sync(sp)
    return {"value": round(args.steps / secs, 3), "unit": "steps/s",
            "h2d_bytes_per_step": 28 * n, "d2h_bytes_per_step": 8 * n,
            "path": "bh_set_state + bh_set_accel (pinned host: the arrays of the reference's "
                    "reset()) + bh_step + bh_get_state(x, y -> pinned host)"}


def run_dropin(torch, stream, sp, flush, n, x, y, vx, vy, m, args):
    """steps/s of BarnesHutParticleSystem::update() (BarnesHutParticleSystem.cpp:308-315)
    through the drop-in wrappers: ResetArrays ... FillOutputArray on the compat stream,
    CUDA events per step, L2 flushed before each."""
    from stellarsolver_gb300 import dropin

    L = dropin.load()
    L.bh_compat_set_stream(sp)
    L.bh_compat_set_constants(THETA, EPS * EPS)
    L.bh_compat_clear_status()
    a = dropin.RefArrays(torch, x, y, vx, vy, m)
    for _ in range(args.warmup):
        dropin.update(L, a, DT, 1.0)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for e0, e1 in evs:
        flush.zero_()
        e0.record(stream)
        dropin.update(L, a, DT, 1.0)
        e1.record(stream)
    torch.cuda.synchronize()
    secs = sum(e0.elapsed_time(e1) for e0, e1 in evs) / 1e3
    status = L.bh_compat_status()
    L.bh_compat_set_stream(None)
    L.bh_compat_release()
    return {"steps_per_s": round(args.steps / secs, 3), "ms_per_step": round(1e3 * secs / args.steps, 4),
            "status": status,
            "path": "ResetArrays, ComputeBoundingBox, BuildQuadTree, ComputeCentreOfMass, "
                    "SortParticles, CalculateForces, IntegrateParticles, FillOutputArray "
                    "(BarnesHutParticleSystem.cpp:308-315), C linkage, arrays of 2n + 12000, "
                    "L2 flushed before every timed step"}


def run_ensemble(bh, torch, stream, sp, local, world, rank, args):
    """256 independent systems, N log-uniform in [2^10, 2^17], half disks and half
    Plummer spheres (eps = 0.01, dt = 1e-4, theta = 0.5).  The batched MIXED engine
    (one launch per phase, CUDA graph) against one handle per system in PLAIN FP32
    without a graph.  With several GPUs each rank steps its own systems."""
    from stellarsolver_gb300 import models, sharding

    sizes = models.ensemble_sizes(256)
    mine = sharding.shard_of(sizes, world, rank)
    systems = models.ensemble(sizes, indices=mine)
    my_sizes = [int(sizes[i]) for i in mine]
    cat = [np.concatenate([sy[k] for sy in systems]) for k in range(5)]
    common = dict(theta=THETA, eps2=EPS * EPS, gravity=1.0, timestep=DT, dampening=1.0)
    k = max(3, min(args.steps, 10))

    def timed(step_fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(k):
            step_fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / k

    with bh.BarnesHutSystem(sizes=my_sizes, device=local, mode="mixed", use_graph=True,
                            **common) as b:
        b.set_state(*cat)
        b.autotune(sp)
        for _ in range(2):
            b.step(1, sp)
        e0 = b.energy(sp)  # FP64 (kinetic, potential, px, py) per system
        t_batch = timed(lambda: b.step(1, sp))
        inter = b.stats(sp)["interactions"]
        e1 = b.energy(sp)
    # per-system diagnostics gathered once, after the timed steps, in system order
    gather = torch.distributed.all_gather_object if world > 1 else None
    diag = sharding.gather_by_system(len(sizes), mine, np.hstack([e0, e1]), gather)
    E0, E1 = diag[:, 0] + diag[:, 1], diag[:, 4] + diag[:, 5]
    drift = np.abs(E1 - E0) / np.abs(E0)
    handles = []
    try:
        for sy in systems:
            h = bh.BarnesHutSystem(len(sy[0]), device=local, mode="plain", use_graph=False,
                                   **common)
            h.set_state(*sy)
            handles.append(h)

        def one_each():
            for h in handles:
                h.step(1, sp)

        one_each()
        t_each = timed(one_each)
    finally:
        for h in handles:
            h.close()
    if world > 1:
        t = torch.tensor([t_batch, t_each], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_batch, t_each = float(t[0]), float(t[1])
    return {"workload": "ensemble of 256 systems, N log-uniform in [2^10, 2^17]",
            "bodies": int(np.sum(sizes)), "steps_timed": k,
            "batched_mixed_graph_steps_per_s": round(1.0 / t_batch, 3),
            "one_handle_per_system_plain_steps_per_s": round(1.0 / t_each, 3),
            "batched_over_per_system": round(t_each / t_batch, 2),
            "interactions_per_s": round(inter / t_batch, 1),
            "systems_diagnosed": int(np.sum(np.isfinite(drift))),
            "energy_drift_rel_max_over_systems": float(np.max(drift)),
            "diagnostics": "FP64 energy and momentum per system before and after the timed "
                           "steps, gathered by system over the ranks"}


CPU_BASELINE_STEPS = 5


def cpu_baseline(x, y, vx, vy, m):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    po.lib()
    state = (x, y, vx, vy)
    t0 = time.perf_counter()
    for _ in range(CPU_BASELINE_STEPS):
        state = po.step_ref(*state, m, THETA, EPS * EPS, DT, 1.0)[:4]
    secs = time.perf_counter() - t0
    return {"value": round(CPU_BASELINE_STEPS / secs, 4), "unit": "steps/s",
            "cores": po.num_threads(), "kind": "port",
            "sample": f"{CPU_BASELINE_STEPS} consecutive full reference-rule steps of the "
                      f"{WORKLOAD} workload (box, keys, sort, tree, centre of mass, warp-vote "
                      "walk, update), OpenMP over all host threads"}


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po

    from stellarsolver_gb300 import models

    po.lib()
    x, y, vx, vy, m = models.plummer(N_BODIES, models.SEED_BASE + 1)
    state = (x, y, vx, vy)
    for _ in range(args.warmup):
        state = po.step_ref(*state, m, THETA, EPS * EPS, DT, 1.0)[:4]
    t0 = time.perf_counter()
    inter = 0
    for _ in range(args.steps):
        out = po.step_ref(*state, m, THETA, EPS * EPS, DT, 1.0)
        state = out[:4]
        inter = out[6]
    secs = time.perf_counter() - t0
    value = args.steps / secs
    cores = po.num_threads()
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * secs / args.steps, 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded 2D Plummer, models.plummer)",
        "config": {"workload": WORKLOAD, "n_bodies": N_BODIES, "theta": THETA, "eps": EPS,
                   "dt": DT, "mode": "reference rule (monopole, warp vote)"},
        "interactions_per_step": inter,
        "interactions_per_s": round(inter * value, 1),
        "cpu_baseline": {"value": round(value, 4), "unit": "steps/s", "cores": cores,
                         "kind": "port",
                         "sample": "full steps of the workload: the reference's algorithm "
                                   "(kernels.cu) restated in C, OpenMP over all host threads; "
                                   "the reference has no CPU path and its CUDA kernels are not "
                                   "run on the shared GPUs (spin-waits that can hang)"},
        "e2e": {"value": round(value, 4), "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--mode", choices=["mixed", "plain", "reference"], default="mixed")
    ap.add_argument("--bucket", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "engine":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
