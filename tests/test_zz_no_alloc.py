"""BuildQuadTreeNoAlloc: the drop-in BuildQuadTree for callers that cannot
allocate device memory.

Examples are a host that owns the whole device-memory budget, a real-time loop
that cannot take an allocation stall, and code whose allocator the library
cannot call.  This variant takes its scratch from one static device array
(limit 65536 bodies) instead of a cudaMalloc'ed workspace.

Checked through the C ABI:
- on two calls in a row, with different inputs (the array keeps the previous
  call's contents), its output equals that of the existing BuildQuadTree on
  the same arrays.  Both build the same tree with the same float operations,
  so the tolerance is bit-exact, as in the other tree tests;
- the same at the limit, 65536 bodies of the reference's Plummer model;
- the wrappers that follow it in the reference's update() (centre of mass,
  sort, forces) give the same results as after BuildQuadTree;
- a call made once the other wrappers have their workspace leaves the
  device's free memory unchanged;
- sizes above the limit are rejected with BH_ERR_CAPACITY, also reported by
  bh_compat_status().

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BH_ERR_CAPACITY = 4


@pytest.fixture(scope="module")
def L():
    import compat_lib

    lib = compat_lib.load()
    vp, i32 = ctypes.c_void_p, ctypes.c_int
    lib.BuildQuadTreeNoAlloc.argtypes = [vp] * 11 + [i32, i32]
    lib.BuildQuadTreeNoAlloc.restype = ctypes.c_int
    return lib


def _arrays(g):
    n = int(g["n"])
    m = 2 * n + 12000
    f = lambda: torch.zeros(m, dtype=torch.float32, device="cuda")  # noqa: E731
    a = {k: f() for k in ("x", "y", "mass", "vx", "vy", "ax", "ay")}
    for k, src in (("x", "x"), ("y", "y"), ("mass", "m")):
        a[k][:n] = torch.from_numpy(g[src])
    a["count"] = torch.zeros(m, dtype=torch.int32, device="cuda")
    a["start"] = torch.zeros(m, dtype=torch.int32, device="cuda")
    a["sorted"] = torch.zeros(m, dtype=torch.int32, device="cuda")
    a["child"] = torch.zeros(4 * m, dtype=torch.int32, device="cuda")
    a["index"] = torch.zeros(1, dtype=torch.int32, device="cuda")
    a["mutex"] = torch.zeros(1, dtype=torch.int32, device="cuda")
    a["box"] = [torch.zeros(1, dtype=torch.float32, device="cuda") for _ in range(4)]
    return a, n, m


def _prepare(L, a, n, m):
    P = lambda t: t.data_ptr()  # noqa: E731
    bx = [P(b) for b in a["box"]]
    L.ResetArrays(P(a["mutex"]), P(a["x"]), P(a["y"]), P(a["mass"]), P(a["count"]),
                  P(a["start"]), P(a["sorted"]), P(a["child"]), P(a["index"]), *bx, n, m)
    L.ComputeBoundingBox(P(a["mutex"]), P(a["x"]), P(a["y"]), *bx, n)
    return P, bx


def _build_args(a, P, bx, n, m):
    return (P(a["x"]), P(a["y"]), P(a["mass"]), P(a["count"]), P(a["start"]), P(a["child"]),
            P(a["index"]), *bx, n, m)


def _snapshot(a):
    torch.cuda.synchronize()
    return {k: a[k].cpu().numpy() for k in ("x", "y", "mass", "count", "start", "child", "index")}


def _bit_equal(a, b, what):
    for k in a:
        if a[k].dtype == np.float32:
            assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (what, k)
        else:
            assert np.array_equal(a[k], b[k]), (what, k)


def _plummer(n):
    from stellarsolver_gb300 import bh

    x, y, vx, vy, m = bh.reference_initial_conditions("plummer", n)
    return {"n": np.int64(n), "x": x, "y": y, "m": m}


def _rest_of_update(L, a, P, bx, n):
    """The wrappers after the tree build in the reference's update()
    (BarnesHutParticleSystem.cpp:311-314): centre of mass, sort, forces."""
    L.ComputeCentreOfMass(P(a["x"]), P(a["y"]), P(a["mass"]), P(a["index"]), n)
    L.SortParticles(P(a["count"]), P(a["start"]), P(a["sorted"]), P(a["child"]), P(a["index"]), n)
    L.CalculateForces(P(a["x"]), P(a["y"]), P(a["vx"]), P(a["vy"]), P(a["ax"]), P(a["ay"]),
                      P(a["mass"]), P(a["sorted"]), P(a["child"]), bx[0], bx[1], n, 1.0)
    torch.cuda.synchronize()
    return {k: a[k].cpu().numpy() for k in ("x", "y", "start", "sorted", "ax", "ay")}


def test_no_alloc_matches_build_quad_tree_two_calls_in_a_row(L):
    L.bh_compat_set_stream(None)
    L.bh_compat_clear_status()
    for name in ("disk4096", "clustered512"):  # two calls in a row, different inputs
        g = gc.load(name)
        ref, n, m = _arrays(g)
        new, _, _ = _arrays(g)
        P, bx = _prepare(L, ref, n, m)
        L.BuildQuadTree(*_build_args(ref, P, bx, n, m))
        P2, bx2 = _prepare(L, new, n, m)
        rc = L.BuildQuadTreeNoAlloc(*_build_args(new, P2, bx2, n, m))
        assert rc == 0, rc
        b = _snapshot(new)
        _bit_equal(_snapshot(ref), b, name)
        assert int(b["index"][0]) - n == int(g["ncells"]), name
    assert L.bh_compat_status() == 0


def test_no_alloc_at_its_limit(L):
    """65536 bodies fill the whole static array.  The child array first holds a
    smaller tree built by BuildQuadTree (n = 4096, m = 20192): the wrappers
    after the no-alloc build must bound child[] by its own m, not the old one."""
    g = _plummer(1 << 16)
    ref, n, m = _arrays(g)
    new, _, _ = _arrays(g)
    P, bx = _prepare(L, ref, n, m)
    L.BuildQuadTree(*_build_args(ref, P, bx, n, m))
    tree_ref = _snapshot(ref)
    a = _rest_of_update(L, ref, P, bx, n)
    n1 = 4096
    m1 = 2 * n1 + 12000
    P2, bx2 = _prepare(L, new, n1, m1)
    L.BuildQuadTree(*_build_args(new, P2, bx2, n1, m1))
    # that tree's cells (slots 4096 on) overwrote bodies: load them again
    for k, src in (("x", "x"), ("y", "y"), ("mass", "m")):
        new[k][:n] = torch.from_numpy(g[src])
    L.bh_compat_clear_status()
    P2, bx2 = _prepare(L, new, n, m)
    rc = L.BuildQuadTreeNoAlloc(*_build_args(new, P2, bx2, n, m))
    assert rc == 0, rc
    _bit_equal(tree_ref, _snapshot(new), "plummer65536 tree")
    b = _rest_of_update(L, new, P2, bx2, n)
    assert L.bh_compat_status() == 0
    _bit_equal(a, b, "plummer65536 forces")


def test_wrappers_after_no_alloc_build(L):
    """Centre of mass, sort and forces after the no-alloc build equal those
    after BuildQuadTree, bit for bit: both builds leave the same layout."""
    for name in ("disk4096", "plummer2048"):
        g = gc.load(name)
        ref, n, m = _arrays(g)
        new, _, _ = _arrays(g)
        P, bx = _prepare(L, ref, n, m)
        L.BuildQuadTree(*_build_args(ref, P, bx, n, m))
        a = _rest_of_update(L, ref, P, bx, n)
        P2, bx2 = _prepare(L, new, n, m)
        assert L.BuildQuadTreeNoAlloc(*_build_args(new, P2, bx2, n, m)) == 0
        b = _rest_of_update(L, new, P2, bx2, n)
        _bit_equal(a, b, name)
    assert L.bh_compat_status() == 0


def test_no_alloc_allocates_nothing(L):
    """With the other wrappers' workspace in place (ResetArrays and
    ComputeBoundingBox ran), a call leaves the device's free memory as it was."""
    g = gc.load("disk4096")
    a, n, m = _arrays(g)
    P, bx = _prepare(L, a, n, m)
    assert L.BuildQuadTreeNoAlloc(*_build_args(a, P, bx, n, m)) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    P, bx = _prepare(L, a, n, m)
    rc = L.BuildQuadTreeNoAlloc(*_build_args(a, P, bx, n, m))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0, rc
    assert free1 == free0, (free0, free1)


def test_no_alloc_rejects_sizes_above_its_limit(L):
    n = (1 << 16) + 1
    m = 2 * n + 12000
    z = torch.zeros(4 * m, dtype=torch.float32, device="cuda")
    zi = torch.zeros(4 * m, dtype=torch.int32, device="cuda")
    p, pi = z.data_ptr(), zi.data_ptr()
    L.bh_compat_clear_status()
    rc = L.BuildQuadTreeNoAlloc(p, p, p, pi, pi, pi, pi, p, p, p, p, n, m)
    assert rc == BH_ERR_CAPACITY
    assert L.bh_compat_status() == BH_ERR_CAPACITY  # the failure is recorded too
    L.bh_compat_clear_status()
