"""Seeded initial conditions for the benchmark workloads (numpy, host side).

Each generator returns float32 arrays (x, y, vx, vy, m).  Seeds are
0x5EED0000 + workload index (plus system index << 16 for ensembles), so the
engine, the oracle and the CPU baseline see identical bytes.  These are
synthetic stand-ins with the shapes and distributions of the workloads; the
reference's own generators (std::default_random_engine,
BarnesHutParticleSystem.cpp:390-560) are reproduced by the C++ host
(stellar_app -disk/-plummer/-colliding-disks).
"""
from __future__ import annotations

import numpy as np

SEED_BASE = 0x5EED0000


def disk(n: int, seed: int, r_lo: float = 5.0, r_hi: float = 50.0, m_c: float = 1000.0,
         G: float = 1.0, centre=(0.0, 0.0), bulk=(0.0, 0.0)):
    """Body 0: central mass m_c at rest; bodies 1..n-1: mass 1, angle U[0,2pi),
    radius U[r_lo, r_hi], counter-clockwise speed sqrt(G * M_enc(r) / r) with
    M_enc = m_c + #(bodies at smaller radius)."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    r = rng.uniform(r_lo, r_hi, n)
    x = np.zeros(n)
    y = np.zeros(n)
    vx = np.zeros(n)
    vy = np.zeros(n)
    m = np.ones(n)
    m[0] = m_c
    if n > 1:
        rr = r[1:]
        order = np.argsort(rr, kind="stable")
        menc = np.empty(n - 1)
        menc[order] = m_c + np.arange(n - 1)
        v = np.sqrt(G * menc / rr)
        x[1:] = rr * np.cos(th[1:])
        y[1:] = rr * np.sin(th[1:])
        vx[1:] = -v * np.sin(th[1:])
        vy[1:] = v * np.cos(th[1:])
    x += centre[0]
    y += centre[1]
    vx += bulk[0]
    vy += bulk[1]
    return tuple(a.astype(np.float32) for a in (x, y, vx, vy, m))


def plummer(n: int, seed: int, a: float = 1.0, M: float = 1.0, G: float = 1.0,
            rmax: float = 10.0):
    """Plummer sphere projected to 2D: r = a / sqrt(u^(-2/3) - 1), u ~ U(0,1),
    rejected unless r < rmax*a; uniform angle; per-component Gaussian
    velocities with sigma = sqrt(G M / (6 a)); equal masses M/n."""
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while len(r) < n:
        u = rng.uniform(0.0, 1.0, 2 * n + 16)
        u = u[u > 0.0]
        rr = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr < rmax * a]])
    r = r[:n]
    th = rng.uniform(0.0, 2.0 * np.pi, n)
    sig = np.sqrt(G * M / (6.0 * a))
    vx = rng.normal(0.0, sig, n)
    vy = rng.normal(0.0, sig, n)
    m = np.full(n, M / n)
    return tuple(v.astype(np.float32) for v in (r * np.cos(th), r * np.sin(th), vx, vy, m))


def colliding_disks(n: int, seed: int, G: float = 1.0):
    """Two disks of n/2 bodies (radius U[5,80], central mass 1e4) centred at
    (-150, 0) and (+150, 0) with bulk velocities (+2, -0.5) and (-2, +0.5)."""
    h = n // 2
    a = disk(h, seed, 5.0, 80.0, 1e4, G, (-150.0, 0.0), (2.0, -0.5))
    b = disk(n - h, seed + 1, 5.0, 80.0, 1e4, G, (150.0, 0.0), (-2.0, 0.5))
    return tuple(np.concatenate([u, v]) for u, v in zip(a, b))


def ensemble_sizes(count: int = 256, lo: int = 1 << 10, hi: int = 1 << 17, seed: int = SEED_BASE + 3):
    """Per-system body counts, log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64).clip(lo, hi)


def ensemble_system(i: int, n: int, seed_base: int = SEED_BASE + 3):
    """System i of an ensemble: a disk for even i, a Plummer sphere for odd i."""
    sd = seed_base + (i << 16)
    return disk(int(n), sd) if i % 2 == 0 else plummer(int(n), sd)


def ensemble(sizes, seed_base: int = SEED_BASE + 3, indices=None):
    """Alternating disk (even index) and Plummer (odd) systems, each with its own seed."""
    idx = range(len(sizes)) if indices is None else indices
    return [ensemble_system(i, sizes[i], seed_base) for i in idx]


# Benchmark workloads with their integration parameters.
WORKLOADS = {
    "disk4096": dict(gen=lambda: disk(4096, SEED_BASE + 0), eps=0.1, dt=1e-3, theta=0.5, steps=50),
    "plummer2d_2^20": dict(gen=lambda: plummer(1 << 20, SEED_BASE + 1), eps=0.01, dt=1e-4,
                           theta=0.5, steps=100),
    "colliding_disks_2^22": dict(gen=lambda: colliding_disks(1 << 22, SEED_BASE + 2), eps=0.05,
                                 dt=5e-4, theta=0.5, steps=200),
    "plummer2d_2^24": dict(gen=lambda: plummer(1 << 24, SEED_BASE + 4), eps=0.005, dt=1e-4,
                           theta=0.5, steps=50),
}
