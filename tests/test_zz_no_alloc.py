"""BuildQuadTreeNoAlloc: the drop-in BuildQuadTree for callers that cannot
allocate device memory.

Examples are a host that owns the whole device-memory budget, a real-time loop
that cannot take an allocation stall, and code whose allocator the library
cannot call.  This variant takes its scratch from one static device array
(limit 65536 bodies) instead of a cudaMalloc'ed workspace.

Checked through the C ABI: on two calls in a row, with different inputs (the
array keeps the previous call's contents), its output equals that of the
existing BuildQuadTree on the same arrays.  Both build the same tree with the
same float operations, so the tolerance is bit-exact, as in the other tree
tests.  Sizes above the limit are rejected with BH_ERR_CAPACITY.

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
    a = {k: f() for k in ("x", "y", "mass")}
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


def test_no_alloc_matches_build_quad_tree_two_calls_in_a_row(L):
    L.bh_compat_set_stream(None)
    for name in ("disk4096", "clustered512"):  # two calls in a row, different inputs
        g = gc.load(name)
        ref, n, m = _arrays(g)
        new, _, _ = _arrays(g)
        P, bx = _prepare(L, ref, n, m)
        L.BuildQuadTree(*_build_args(ref, P, bx, n, m))
        P2, bx2 = _prepare(L, new, n, m)
        rc = L.BuildQuadTreeNoAlloc(*_build_args(new, P2, bx2, n, m))
        assert rc == 0, rc
        a, b = _snapshot(ref), _snapshot(new)
        for k in a:
            if a[k].dtype == np.float32:
                assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (name, k)
            else:
                assert np.array_equal(a[k], b[k]), (name, k)
        assert int(b["index"][0]) - n == int(g["ncells"]), name


def test_no_alloc_rejects_sizes_above_its_limit(L):
    n = (1 << 16) + 1
    m = 2 * n + 12000
    z = torch.zeros(4 * m, dtype=torch.float32, device="cuda")
    zi = torch.zeros(4 * m, dtype=torch.int32, device="cuda")
    p, pi = z.data_ptr(), zi.data_ptr()
    rc = L.BuildQuadTreeNoAlloc(p, p, p, pi, pi, pi, pi, p, p, p, p, n, m)
    assert rc == BH_ERR_CAPACITY
