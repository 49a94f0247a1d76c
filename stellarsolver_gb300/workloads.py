"""Measured workloads beside the headline benchmark, one JSON line each.

  python -m stellarsolver_gb300.workloads colliding   # two colliding disks, N = 2^22
  python -m stellarsolver_gb300.workloads plummer24   # Plummer N = 2^24, theta sweep
  python -m stellarsolver_gb300.workloads disk4096    # the small disk, N = 4096

colliding: 2 x 2^21 bodies (disks of radius U[5,80], central masses 1e4,
  centres (+-150, 0), bulk velocities (-+2, +-0.5)), eps = 0.05, dt = 5e-4,
  theta = 0.5, 200 MIXED steps; FP64 energy and momentum every 10 steps,
  recorded on the device by a captured diagnostics graph (bh_set_energy_log),
  inside the timed steps.
plummer24: N = 2^24 2D Plummer, eps = 0.005, dt = 1e-4, 50 steps per run, theta
  in {0.3, 0.5, 0.8}, PLAIN and MIXED: steps/s, interactions/s, per-phase GB/s,
  walk FP32 fraction, force error against the FP64 direct sum on 4096 bodies.
disk4096: the reference's small case (central mass 1000, radius U[5,50]),
  eps = 0.1, dt = 1e-3, theta = 0.5, 50 steps in each mode.

Inputs are the seeded synthetic generators of models.py.  Steps are timed on
the host around graph replays with a device synchronisation on both sides.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import bh, models, roofline

SAMPLE = 4096


def _sample(n: int) -> np.ndarray:
    return np.sort(np.random.default_rng(7).choice(n, size=min(SAMPLE, n),
                                                   replace=False)).astype(np.int32)


def _error(ax, ay, idx, rx, ry) -> dict:
    rel = np.hypot(ax[idx] - rx, ay[idx] - ry) / np.hypot(rx, ry)
    return {"rms_rel": float(np.sqrt(np.mean(rel ** 2))), "max_rel": float(rel.max())}


def _timed_steps(s: bh.BarnesHutSystem, steps: int) -> float:
    s.sync()
    t0 = time.perf_counter()
    s.step(steps)
    s.sync()
    return time.perf_counter() - t0


def _drift(e0: np.ndarray, e: np.ndarray, pscale: float) -> dict:
    E0 = e0[0] + e0[1]
    E = e[0] + e[1]
    return {"energy_rel": float(abs(E - E0) / abs(E0)),
            "momentum_rel": float(np.hypot(e[2] - e0[2], e[3] - e0[3]) / pscale)}


def _pscale(st: dict) -> float:
    m = st["m"].astype(np.float64)
    return float(np.sum(m * np.hypot(st["vx"], st["vy"])))


def colliding(args) -> dict:
    n = 1 << 22
    x, y, vx, vy, m = models.colliding_disks(n, models.SEED_BASE + 2)
    eps, dt, theta, steps = 0.05, 5e-4, 0.5, args.steps or 200
    idx = _sample(n)
    with bh.BarnesHutSystem(n, mode="mixed", theta=theta, eps2=eps * eps, timestep=dt,
                            use_graph=True) as s:
        s.set_state(x, y, vx, vy, m)
        rx, ry = s.direct_sum_f64(idx)
        shape = s.autotune()
        s.set_state(x, y, vx, vy, m)
        pscale = _pscale(s.get_state())
        e0 = s.energy()[0]
        s.step(1)
        ax, ay = s.get_accel()
        err = _error(ax, ay, idx, rx, ry)
        # diagnostics on the device after every 10th step, captured as a graph
        s.set_energy_log(10, capacity=steps // 10 + 1)
        secs = _timed_steps(s, steps - 1)
        inter = s.stats()["interactions"]
        count, log = s.energy_log()
    series = [{"step": 1 + 10 * (r + 1), **_drift(e0, log[r, 0], pscale)} for r in range(count)]
    worst = {key: max(d[key] for d in series) for key in ("energy_rel", "momentum_rel")}
    return {"workload": "colliding disks 2 x 2^21", "n_bodies": n, "mode": "mixed",
            "theta": theta, "eps": eps, "dt": dt, "steps": steps, "walk_shape": shape,
            "steps_per_s_with_diagnostics_every_10": round((steps - 1) / secs, 2),
            "interactions_per_s": round(inter * (steps - 1) / secs, 1),
            "force_error_vs_fp64_step0": err, "max_drift_every_10_steps": worst,
            "drift_series": series}


def plummer24(args) -> dict:
    n = 1 << 24
    x, y, vx, vy, m = models.plummer(n, models.SEED_BASE + 4)
    eps, dt, steps = 0.005, 1e-4, args.steps or 50
    idx = _sample(n)
    hbm, hbm_kind = roofline.hbm_peak()
    fp32_peak = bh.measure_fp32_peak(0)
    rows = []
    rx = ry = None
    for theta in (0.3, 0.5, 0.8):
        for mode in ("plain", "mixed"):
            with bh.BarnesHutSystem(n, mode=mode, theta=theta, eps2=eps * eps, timestep=dt,
                                    use_graph=True) as s:
                s.set_state(x, y, vx, vy, m)
                if rx is None:
                    rx, ry = s.direct_sum_f64(idx)
                shape = s.autotune()
                s.set_state(x, y, vx, vy, m)
                pscale = _pscale(s.get_state())
                e0 = s.energy()[0]
                s.step(1)
                ax, ay = s.get_accel()
                err = _error(ax, ay, idx, rx, ry)
                s.step(2)
                secs = _timed_steps(s, steps)
                st = s.stats()
                drift = _drift(e0, s.energy()[0], pscale)
                phase_ms = np.zeros(bh.PHASES_N, np.float32)
                for _ in range(3):
                    s.step_profiled(phase_ms)
                phase_ms /= 3
                st = s.stats()
            pb = roofline.phase_bytes(n, mode == "mixed", passes=roofline.high_passes(n))
            phases = {}
            for i, name in enumerate(bh.PHASES):
                ms = float(phase_ms[i])
                e = {"ms": round(ms, 4)}
                if name in pb and ms > 0:
                    gbs = pb[name] / (ms * 1e-3) / 1e9
                    e.update({"GB/s": round(gbs, 1), "frac_hbm": round(gbs / hbm, 4)})
                phases[name] = e
            walk_ms = float(phase_ms[bh.PHASES.index("walk")])
            tflops = roofline.walk_flops(st) / (walk_ms * 1e-3) / 1e12
            tflops_mp = roofline.walk_flops_with_multipole(st) / (walk_ms * 1e-3) / 1e12
            rows.append({"theta": theta, "mode": mode, "walk_shape": shape,
                         "steps_per_s": round(steps / secs, 3),
                         "interactions_per_step": st["interactions"],
                         "interactions_per_s": round(st["interactions"] * steps / secs, 1),
                         "force_error_vs_fp64": err, "drift_after_steps": drift,
                         "walk_tflops": round(tflops, 3), "walk_frac_fp32": round(tflops / fp32_peak, 4),
                         "walk_tflops_with_multipole": round(tflops_mp, 3),
                         "phases": phases})
    return {"workload": "plummer2d_2^24 theta sweep", "n_bodies": n, "eps": eps, "dt": dt,
            "steps": steps, "fp32_peak_tflops": round(fp32_peak, 2), "hbm_peak_gbs": hbm,
            "hbm_peak_source": hbm_kind, "runs": rows}


def disk4096(args) -> dict:
    n = 4096
    x, y, vx, vy, m = models.disk(n, models.SEED_BASE)
    eps, dt, theta, steps = 0.1, 1e-3, 0.5, args.steps or 50
    idx = _sample(n)
    rows = []
    rx = ry = None
    for mode in ("reference", "plain", "mixed"):
        with bh.BarnesHutSystem(n, mode=mode, theta=theta, eps2=eps * eps, timestep=dt,
                                use_graph=True) as s:
            s.set_state(x, y, vx, vy, m)
            if rx is None:
                rx, ry = s.direct_sum_f64(idx)
            s.step(1)
            ax, ay = s.get_accel()
            err = _error(ax, ay, idx, rx, ry)
            s.step(3)
            secs = _timed_steps(s, steps)
            rows.append({"mode": mode, "steps_per_s": round(steps / secs, 1),
                         "interactions_per_step": s.stats()["interactions"],
                         "force_error_vs_fp64": err})
    return {"workload": "disk 4096", "n_bodies": n, "theta": theta, "eps": eps, "dt": dt,
            "steps": steps, "runs": rows}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("workload", choices=("colliding", "plummer24", "disk4096"))
    ap.add_argument("--steps", type=int, default=0, help="override the workload's step count")
    args = ap.parse_args(argv)
    out = {"colliding": colliding, "plummer24": plummer24, "disk4096": disk4096}[args.workload](args)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
