"""The drop-in wrappers from Python: their ctypes signatures, the reference's
device arrays, and its update() order.

The reference's host class calls nine launch wrappers (Particle_cuda.cuh:5-13)
on device arrays it allocates with m = 2n + 12000 entries
(BarnesHutParticleSystem.cpp:33, 54-83) in a fixed order
(BarnesHutParticleSystem.cpp:308-315).  This module binds the same nine
functions of libstellar_bh.so (C linkage, include/Particle_cuda.cuh) and
replays that order on arrays of that layout, held in torch tensors (PyTorch is
only the device allocator here).
"""
from __future__ import annotations

import ctypes

from . import bh

SIGNATURES = {
    "SetDrawArray": (["p", "p", "p", "i"]),
    "ResetArrays": (["p"] * 13 + ["i", "i"]),
    "ComputeBoundingBox": (["p"] * 7 + ["i"]),
    "BuildQuadTree": (["p"] * 11 + ["i", "i"]),
    "ComputeCentreOfMass": (["p"] * 4 + ["i"]),
    "SortParticles": (["p"] * 5 + ["i"]),
    "CalculateForces": (["p"] * 11 + ["i", "f"]),
    "IntegrateParticles": (["p"] * 6 + ["i", "f", "f"]),
    "FillOutputArray": (["p", "p", "p", "i"]),
    "bh_compat_set_constants": (["f", "f"]),
    "bh_compat_set_stream": (["p"]),
    "bh_compat_status": ([]),
    "bh_compat_clear_status": ([]),
    "bh_compat_release": ([]),
}
_CT = {"p": ctypes.c_void_p, "i": ctypes.c_int, "f": ctypes.c_float}


def load() -> ctypes.CDLL:
    """libstellar_bh.so with the drop-in wrappers' argument types set."""
    L = bh.lib()
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = [_CT[a] for a in args]
        fn.restype = ctypes.c_int if name == "bh_compat_status" else None
    return L


class RefArrays:
    """Device arrays laid out like BarnesHutParticleSystem.cpp:54-83 (m = 2n + 12000),
    with the first n entries of x, y, vx, vy, mass set from host arrays."""

    def __init__(self, torch, x, y, vx, vy, mass, device="cuda"):
        n = len(x)
        m = 2 * n + 12000
        self.n, self.m = n, m

        def f():
            return torch.zeros(m, dtype=torch.float32, device=device)

        self.x, self.y, self.vx, self.vy, self.mass, self.ax, self.ay = (f() for _ in range(7))
        for t, a in ((self.x, x), (self.y, y), (self.vx, vx), (self.vy, vy), (self.mass, mass)):
            t[:n] = torch.as_tensor(a, dtype=torch.float32)

        def i(k=1):
            return torch.zeros(k * m, dtype=torch.int32, device=device)

        self.count, self.start, self.sorted, self.child = i(), i(), i(), i(4)
        self.index = torch.zeros(1, dtype=torch.int32, device=device)
        self.mutex = torch.zeros(1, dtype=torch.int32, device=device)
        self.box = [torch.zeros(1, dtype=torch.float32, device=device) for _ in range(4)]
        self.out = torch.zeros(2 * m, dtype=torch.float32, device=device)


def update(L, a: RefArrays, dt: float, damp: float, gravity: float = 1.0) -> None:
    """One BarnesHutParticleSystem::update() (BarnesHutParticleSystem.cpp:308-315):
    the eight wrapper calls in the reference's order, on the compat stream."""
    n, m = a.n, a.m
    P = lambda t: t.data_ptr()  # noqa: E731
    bx = [P(b) for b in a.box]
    L.ResetArrays(P(a.mutex), P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.sorted),
                  P(a.child), P(a.index), *bx, n, m)
    L.ComputeBoundingBox(P(a.mutex), P(a.x), P(a.y), *bx, n)
    L.BuildQuadTree(P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.child), P(a.index),
                    *bx, n, m)
    L.ComputeCentreOfMass(P(a.x), P(a.y), P(a.mass), P(a.index), n)
    L.SortParticles(P(a.count), P(a.start), P(a.sorted), P(a.child), P(a.index), n)
    L.CalculateForces(P(a.x), P(a.y), P(a.vx), P(a.vy), P(a.ax), P(a.ay), P(a.mass), P(a.sorted),
                      P(a.child), bx[0], bx[1], n, gravity)
    L.IntegrateParticles(P(a.x), P(a.y), P(a.vx), P(a.vy), P(a.ax), P(a.ay), n, dt, damp)
    L.FillOutputArray(P(a.x), P(a.y), P(a.out), m)
