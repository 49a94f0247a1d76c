"""Small fixed workload for profiler captures (ncu launch lists and kernel captures).

    python -m stellarsolver_gb300.profile_step --n 1048576 --mode mixed --steps 3

Creates one system on the 2D Plummer input, runs `--warmup` steps, then
`--steps` steps, synchronising after each, and prints the per-step status.
Kernel order per step: k_bbox, k_keys, (k_radix_hist, k_radix_scan,
k_radix_scatter) x 8, k_gather, k_build, k_moments, k_records, then the walk
(REFERENCE: k_walk_vote; PLAIN/MIXED: the bootstrap k_walk_acc, which exits at
once unless the state was just set, and the main k_walk_acc).
"""
import argparse

import numpy as np

from . import bh, models


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--mode", default="mixed", choices=list(bh.MODES))
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--bucket", type=int, default=0)
    ap.add_argument("--bpl", type=int, default=0, help="bodies per lane of the accuracy walk")
    ap.add_argument("--block", type=int, default=0, help="walk threads per block")
    ap.add_argument("--phases", action="store_true", help="also print event-timed phase ms")
    ap.add_argument("--graph-ms", type=int, default=0, metavar="K",
                    help="also time K steps replayed as a CUDA graph (host clock, synchronised)")
    ap.add_argument("--error", action="store_true",
                    help="also print the force error against the FP64 direct sum (4096 bodies)")
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--model", default="plummer", choices=["plummer", "disk", "colliding"])
    a = ap.parse_args()
    if a.model == "plummer":
        x, y, vx, vy, m = models.plummer(a.n, models.SEED_BASE + 1)
    elif a.model == "disk":
        x, y, vx, vy, m = models.disk(a.n, models.SEED_BASE)
    else:
        x, y, vx, vy, m = models.colliding_disks(a.n, models.SEED_BASE + 2)
    with bh.BarnesHutSystem(a.n, mode=a.mode, theta=0.5, eps2=1e-4, timestep=1e-4,
                            leaf_bucket=a.bucket, use_graph=a.graph, bodies_per_lane=a.bpl,
                            block_size=a.block) as s:
        s.set_state(x, y, vx, vy, m)
        if a.error:
            idx = np.sort(np.random.default_rng(7).choice(a.n, size=min(4096, a.n),
                                                          replace=False)).astype(np.int32)
            rx, ry = s.direct_sum_f64(idx)
            s.step(1)
            ax, ay = s.get_accel()
            rel = np.hypot(ax[idx] - rx, ay[idx] - ry) / np.hypot(rx, ry)
            print(f"force error vs FP64: rms {np.sqrt(np.mean(rel ** 2)):.4e} max {rel.max():.4e}")
        for _ in range(a.warmup):
            s.step(1)
            s.sync()
        for k in range(a.steps):
            s.step(1)
            s.sync()
        st = s.stats()
        if a.graph_ms:
            import time
            s.set_params(mode=a.mode, theta=0.5, eps2=1e-4, timestep=1e-4, leaf_bucket=a.bucket,
                         use_graph=True, bodies_per_lane=a.bpl, block_size=a.block)
            s.step(3)
            s.sync()
            t0 = time.perf_counter()
            s.step(a.graph_ms)
            s.sync()
            print(f"graph step ms: {1e3 * (time.perf_counter() - t0) / a.graph_ms:.4f}")
        if a.phases:
            ms = np.zeros(bh.PHASES_N, np.float32)
            for _ in range(5):
                s.step_profiled(ms)
            print("phases ms:", {k: round(float(v) / 5, 4) for k, v in zip(bh.PHASES, ms)})
    print(f"profile_step n={a.n} mode={a.mode} steps={a.steps} interactions={st['interactions']} "
          f"status={st['status']} max_stack={st['max_stack']} nodes={st['nodes']} "
          f"rounds={st['walk_rounds']} tested={st['nodes_tested']}")


if __name__ == "__main__":
    main()
