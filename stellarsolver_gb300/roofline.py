"""Roofline bookkeeping shared by bench.py and workloads.py: the algorithmic
bytes of the HBM-bound phases, the walk's flop count and the HBM peak."""
from __future__ import annotations

import json
import os

# FP32 flops per interaction (an FMA counts 2, rsqrt 1), from the kernels' arithmetic:
#   body-body  (p2p): dx,dy 2; u 4; rsqrt 1; r^-3 2; m*r^-3 1; two FMAs 4           = 14
#   body-cell  (p2m): dx,dy 2; u 4; rsqrt 1; r^-2,r^-3 2; T.d 6; d.T.d 3; t 3;
#                     coef 2; fx,fy 6; two FMAs 4                                    = 33
FLOPS_P2P = 14
FLOPS_P2M = 33

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def walk_flops(stats: dict) -> int:
    """The walk's algorithmic FP32 flops by the project's measurement rule:
    14 per body-node interaction of either kind (the reference's force law,
    kernels.cu:403-411); the quadrupole terms are overhead, reported apart."""
    return FLOPS_P2P * stats["interactions"]


def walk_flops_with_multipole(stats: dict) -> int:
    """The walk's FP32 flops as the kernels execute them: 14 per body-body and
    33 per body-cell (quadrupole) interaction, from the exact counts."""
    cells = stats["cell_interactions"]
    return FLOPS_P2P * (stats["interactions"] - cells) + FLOPS_P2M * cells


def high_passes(largest_system: int) -> int:
    """Radix passes of the sort's fast path: 3 (top 24 key bits) for systems
    up to 2^21 bodies, 4 (top 32 bits) above."""
    return 3 if largest_system <= 1 << 21 else 4


def phase_bytes(n: int, mixed: bool, passes: int = 3, accuracy: bool = True) -> dict:
    """Algorithmic bytes per launch of each HBM-bound phase (each array once).
    The sort: `passes` radix passes over the key's high word and the run
    fixup, each one read and one write of (key, index).  The reorder moves
    x, y, vx, vy, m, id (and the hi/lo tails in MIXED mode, |a_old| and the
    walk-group cost in the accuracy modes) and reads the permutation."""
    lo = 16 * n if mixed else 0
    acc = 16 * n if accuracy else 0
    return {
        "bbox": 8 * n,
        "keys": 20 * n,
        "sort": 24 * n * (passes + 1),
        "reorder": 52 * n + lo + acc,
        "build": 36 * n + 16 * n,  # keys and node arrays, climb records
        "moments": 12 * n + 64 * n + 108 * n,  # bodies, node sums, then walk records
    }


def hbm_peak() -> tuple[float, str]:
    """Measured STREAM-style copy bandwidth (GB/s) of the GB300s, else
    the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"
