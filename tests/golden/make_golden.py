"""Generate the golden fixtures in this folder from the reference itself.

The reference (pentilm/StellarSolver) has no CPU path, no tests and no golden
vectors.  This script compiles its own kernels.cu for the host
(oracle/Makefile target `ref`, sources read where they lie) and runs the
reference's update() sequence (BarnesHutParticleSystem.cpp:308-314) phase by
phase on seeded inputs, through the same launch wrappers
(Particle_cuda.cu:14-53) with one 64-thread block.  Each fixture stores the
inputs and every phase output in a canonical, cell-numbering-independent form.

Run where the reference sources are present:
    STELLARSOLVER_REF=<reference checkout> python tests/golden/make_golden.py
    (or --ref <reference checkout>)
The fixtures are committed; tests never need the reference at run time.

The reference's softening and opening angle are compile-time constants
(kernels.cu:8-9: eps2 = 0.025, theta = 0.5); fixtures record them.
"""
from __future__ import annotations

import argparse
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

REF_EPS2 = 0.025  # kernels.cu:8
REF_THETA = 0.5   # kernels.cu:9
BLOCK = 64        # one emulated block; grid-stride loops cover n


def load_ref(ref_dir: str) -> ctypes.CDLL:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref_dir}"],
                   check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_emu.so"))
    vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.refemu_ResetArrays.argtypes = [i32] + [vp] * 13 + [i32, i32]
    lib.refemu_ComputeBoundingBox.argtypes = [i32] + [vp] * 7 + [i32]
    lib.refemu_BuildQuadTree.argtypes = [i32] + [vp] * 11 + [i32, i32]
    lib.refemu_ComputeCentreOfMass.argtypes = [i32] + [vp] * 4 + [i32]
    lib.refemu_SortParticles.argtypes = [i32] + [vp] * 5 + [i32]
    lib.refemu_CalculateForces.argtypes = [i32] + [vp] * 11 + [i32, f32]
    lib.refemu_IntegrateParticles.argtypes = [i32] + [vp] * 6 + [i32, f32, f32]
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefSystem:
    """The reference's device arrays (length m = 2n+12000, BarnesHutParticleSystem.cpp:33)."""

    def __init__(self, lib, x, y, vx, vy, mass):
        self.lib = lib
        n = len(x)
        self.n, self.m = n, 2 * n + 12000
        z = lambda: np.zeros(self.m, np.float32)  # noqa: E731
        self.x, self.y, self.vx, self.vy, self.mass, self.ax, self.ay = (z() for _ in range(7))
        for dst, src in ((self.x, x), (self.y, y), (self.vx, vx), (self.vy, vy), (self.mass, mass)):
            dst[:n] = src
        self.count = np.zeros(self.m, np.int32)
        self.start = np.zeros(self.m, np.int32)
        self.sorted = np.zeros(self.m, np.int32)
        self.child = np.zeros(4 * self.m, np.int32)
        self.index = np.zeros(1, np.int32)
        self.mutex = np.zeros(1, np.int32)
        self.box = [np.zeros(1, np.float32) for _ in range(4)]

    def update(self, dt, damp, record=None):
        L, n, m, B = self.lib, self.n, self.m, BLOCK
        bx = [_p(b) for b in self.box]
        chk = lambda st: None if st == 0 else (_ for _ in ()).throw(RuntimeError(st))  # noqa
        chk(L.refemu_ResetArrays(B, _p(self.mutex), _p(self.x), _p(self.y), _p(self.mass),
                                 _p(self.count), _p(self.start), _p(self.sorted), _p(self.child),
                                 _p(self.index), *bx, n, m))
        chk(L.refemu_ComputeBoundingBox(B, _p(self.mutex), _p(self.x), _p(self.y), *bx, n))
        if record is not None:
            record["box"] = np.array([b[0] for b in self.box], np.float32)
        chk(L.refemu_BuildQuadTree(B, _p(self.x), _p(self.y), _p(self.mass), _p(self.count),
                                   _p(self.start), _p(self.child), _p(self.index), *bx, n, m))
        if record is not None:
            record["cells_before_com"] = (self.x.copy(), self.y.copy(), self.mass.copy())
        chk(L.refemu_ComputeCentreOfMass(B, _p(self.x), _p(self.y), _p(self.mass),
                                         _p(self.index), n))
        chk(L.refemu_SortParticles(B, _p(self.count), _p(self.start), _p(self.sorted),
                                   _p(self.child), _p(self.index), n))
        chk(L.refemu_CalculateForces(B, _p(self.x), _p(self.y), _p(self.vx), _p(self.vy),
                                     _p(self.ax), _p(self.ay), _p(self.mass), _p(self.sorted),
                                     _p(self.child), bx[0], bx[1], n, 1.0))
        if record is not None:
            record["child"] = self.child.copy()
            record["count"] = self.count.copy()
            record["index"] = int(self.index[0])
            record["com"] = (self.x.copy(), self.y.copy(), self.mass.copy())
            record["sorted"] = self.sorted[:n].copy()
            record["ax"] = self.ax[:n].copy()
            record["ay"] = self.ay[:n].copy()
        chk(L.refemu_IntegrateParticles(B, _p(self.x), _p(self.y), _p(self.vx), _p(self.vy),
                                        _p(self.ax), _p(self.ay), n, dt, damp))

    def state(self):
        n = self.n
        return self.x[:n].copy(), self.y[:n].copy(), self.vx[:n].copy(), self.vy[:n].copy()


# ------------------------------------------------------------------ inputs

def disk(n, seed, r_lo=5.0, r_hi=50.0, m_c=1000.0, G=1.0):
    """Config-0 style disk: body 0 a central mass at rest, the rest on circular orbits."""
    rng = np.random.default_rng(seed)
    th = rng.uniform(0.0, 2 * np.pi, n)
    r = rng.uniform(r_lo, r_hi, n)
    m = np.ones(n)
    order = np.argsort(r[1:])
    menc = np.empty(n - 1)
    menc[order] = m_c + np.arange(n - 1)
    v = np.sqrt(G * menc / r[1:])
    x = np.concatenate([[0.0], r[1:] * np.cos(th[1:])])
    y = np.concatenate([[0.0], r[1:] * np.sin(th[1:])])
    vx = np.concatenate([[0.0], -v * np.sin(th[1:])])
    vy = np.concatenate([[0.0], v * np.cos(th[1:])])
    m[0] = m_c
    return [a.astype(np.float32) for a in (x, y, vx, vy, m)]


def plummer(n, seed, a=1.0, G=1.0):
    """Config-1 style Plummer sphere projected to 2D, truncated at r < 10a, total mass 1."""
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while len(r) < n:
        u = rng.uniform(0.0, 1.0, 2 * n)
        rr = a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr < 10 * a]])
    r = r[:n]
    th = rng.uniform(0.0, 2 * np.pi, n)
    sig = np.sqrt(G * 1.0 / (6 * a))
    vx = rng.normal(0.0, sig, n)
    vy = rng.normal(0.0, sig, n)
    m = np.full(n, 1.0 / n)
    return [a_.astype(np.float32) for a_ in (r * np.cos(th), r * np.sin(th), vx, vy, m)]


def clustered(n, seed):
    """Two tight clumps and a distant pair: long single-child chains and a deep tree."""
    rng = np.random.default_rng(seed)
    h = n // 2 - 1
    c1 = rng.normal(0.0, 1e-3, (h, 2)) + [3.0, 3.0]
    c2 = rng.normal(0.0, 0.3, (n - h - 2, 2)) + [-2.0, 1.0]
    far = np.array([[-40.0, -25.0], [-39.5, -25.25]])
    pos = np.concatenate([c1, c2, far])
    v = rng.normal(0.0, 0.5, (n, 2))
    m = rng.uniform(0.5, 2.0, n)
    return [a.astype(np.float32) for a in (pos[:, 0], pos[:, 1], v[:, 0], v[:, 1], m)]


CASES = {
    "disk4096": (lambda: disk(4096, 0x5EED0000), 1e-3, 1.0),
    "plummer2048": (lambda: plummer(2048, 0x5EED0001), 1e-4, 1.0),
    "clustered512": (lambda: clustered(512, 0x5EED0002), 1e-3, 0.9),
}


def make_case(lib, name, gen, dt, damp, steps=3):
    x, y, vx, vy, m = gen()
    n = len(x)
    sysr = RefSystem(lib, x, y, vx, vy, m)
    rec = {}
    sysr.update(dt, damp, record=rec)
    x1, y1, vx1, vy1 = sysr.state()
    for _ in range(steps - 1):
        sysr.update(dt, damp)
    x3, y3, vx3, vy3 = sysr.state()

    bd, bp, cells, vals = po.canonical_from_child(rec["child"], rec["count"], n, rec["com"])
    _, _, _, sums = po.canonical_from_child(rec["child"], rec["count"], n,
                                            rec["cells_before_com"])
    out = dict(
        n=np.int32(n), eps2=np.float32(REF_EPS2), theta=np.float32(REF_THETA),
        dt=np.float32(dt), damp=np.float32(damp), steps=np.int32(steps),
        x=x, y=y, vx=vx, vy=vy, m=m,
        box=rec["box"], sorted=rec["sorted"], ncells=np.int32(rec["index"] - n),
        body_depth=bd, body_path=bp,
        cell_level=cells["level"], cell_prefix=cells["prefix"], cell_count=cells["count"],
        cell_cx=vals[0], cell_cy=vals[1], cell_m=vals[2],
        cell_mx=sums[0], cell_my=sums[1],
        ax=rec["ax"], ay=rec["ay"],
        x1=x1, y1=y1, vx1=vx1, vy1=vy1, x3=x3, y3=y3, vx3=vx3, vy3=vy3,
    )
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: n={n} cells={rec['index'] - n} -> {os.path.relpath(path, ROOT)} "
          f"({os.path.getsize(path) // 1024} KiB)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("STELLARSOLVER_REF"),
                    help="reference sources (default: $STELLARSOLVER_REF)")
    args = ap.parse_args()
    if not args.ref:
        sys.exit("give the reference sources with --ref or STELLARSOLVER_REF")
    lib = load_ref(args.ref)
    for name, (gen, dt, damp) in CASES.items():
        make_case(lib, name, gen, dt, damp)


if __name__ == "__main__":
    main()
