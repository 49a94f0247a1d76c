"""Test infrastructure (oracle), never shipped.

ctypes wrapper over lib/liboracle.so, the CPU restatement of the reference's
Barnes-Hut step (pentilm/StellarSolver kernels.cu), plus the canonical tree
form used to compare trees whose cell numbering differs (the reference numbers
cells in atomic-allocation order, kernels.cu:199).  Imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liboracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, f32, f64, i64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_double, ctypes.c_int64)
        L.orc_bbox.argtypes = [i32, vp, vp, vp]
        L.orc_keys.argtypes = [i32, vp, vp, vp, vp]
        L.orc_keys.restype = None
        L.orc_sort_keys.argtypes = [i32, vp, vp]
        L.orc_build_tree.argtypes = [i32, vp] + [vp] * 8
        L.orc_node_sums.argtypes = [i32] + [vp] * 10
        L.orc_node_sums.restype = None
        L.orc_quad_children.argtypes = [i32] + [vp] * 5
        L.orc_quad_children.restype = None
        L.orc_walk_ref.argtypes = [i32] + [vp] * 9 + [f32, f32, vp, vp]
        L.orc_walk_ref.restype = i64
        L.orc_step_ref.argtypes = [i32] + [vp] * 7 + [f32, f32, f32, f32, vp]
        L.orc_direct_f64.argtypes = [i32, vp, vp, vp, i32, vp, f64, f64, vp, vp]
        L.orc_direct_f64.restype = None
        L.orc_direct_f64_hilo.argtypes = [i32, vp, vp, vp, vp, vp, i32, vp, f64, f64, vp, vp]
        L.orc_direct_f64_hilo.restype = None
        L.orc_energy_f64.argtypes = [i32] + [vp] * 5 + [f64, f64, vp]
        L.orc_energy_f64.restype = None
        L.orc_walk_acc.argtypes = [i32] + [vp] * 11 + [f32, f32, f32, i32, f32, vp, i32, i32, vp,
                                                        vp]
        L.orc_walk_acc.restype = i64
        L.orc_check_tree.argtypes = [i32] + [vp] * 11
        L.orc_check_tree.restype = ctypes.c_uint
        L.orc_render.argtypes = [i32, vp, vp, i32, i32, f32, f32, f32, f32, vp]
        L.orc_render.restype = None
        L.orc_frontier_check.argtypes = [i32] + [vp] * 11 + [f32, f32, i32, f32, vp, i32, i32, vp]
        L.orc_frontier_check.restype = None
        L.orc_num_threads.restype = i32
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def bbox(x, y):
    x, y = _f32(x), _f32(y)
    box = np.zeros(4, np.float32)
    st = lib().orc_bbox(len(x), _p(x), _p(y), _p(box))
    if st:
        raise ValueError(f"orc_bbox status {st}")
    return box


def keys(x, y, box):
    x, y = _f32(x), _f32(y)
    box = _f32(box)
    k = np.zeros(len(x), np.uint64)
    lib().orc_keys(len(x), _p(x), _p(y), _p(box), _p(k))
    return k


def sort_keys(k):
    k = np.ascontiguousarray(k, dtype=np.uint64)
    perm = np.zeros(len(k), np.uint32)
    dups = lib().orc_sort_keys(len(k), _p(k), _p(perm))
    return perm, int(dups)


class Tree:
    """Binary radix tree (Karras numbering) with the quadtree digit merge."""

    def __init__(self, skeys):
        n = len(skeys)
        self.n = n
        nn = n - 1
        self.left = np.zeros(nn, np.int32)
        self.right = np.zeros(nn, np.int32)
        self.split = np.zeros(nn, np.int32)
        self.first = np.zeros(nn, np.int32)
        self.last = np.zeros(nn, np.int32)
        self.parent = np.zeros(nn, np.int32)
        self.leaf_parent = np.zeros(n, np.int32)
        self.qmerged = np.zeros(nn, np.uint8)
        skeys = np.ascontiguousarray(skeys, dtype=np.uint64)
        st = lib().orc_build_tree(n, _p(skeys), _p(self.left), _p(self.right), _p(self.split),
                                  _p(self.first), _p(self.last), _p(self.parent),
                                  _p(self.leaf_parent), _p(self.qmerged))
        if st:
            raise ValueError(f"orc_build_tree status {st}")
        self.qchild = np.zeros(4 * nn, np.int32)
        lib().orc_quad_children(n, _p(self.left), _p(self.right), _p(self.split),
                                _p(self.qmerged), _p(self.qchild))

    def sums(self, sx, sy, sm):
        nn = self.n - 1
        out = [np.zeros(nn, np.float32) for _ in range(5)]
        sx, sy, sm = _f32(sx), _f32(sy), _f32(sm)
        lib().orc_node_sums(self.n, _p(sx), _p(sy), _p(sm), _p(self.left), _p(self.right),
                            *[_p(o) for o in out])
        return out  # m, mx, my, cx, cy


def walk_ref(sx, sy, sm, tree: Tree, node_m, node_cx, node_cy, box, theta, eps2):
    n = len(sx)
    sax = np.zeros(n, np.float32)
    say = np.zeros(n, np.float32)
    sx, sy, sm = _f32(sx), _f32(sy), _f32(sm)
    box = _f32(box)
    inter = lib().orc_walk_ref(n, _p(sx), _p(sy), _p(sm), _p(tree.split), _p(tree.qchild),
                               _p(_f32(node_m)), _p(_f32(node_cx)), _p(_f32(node_cy)), _p(box),
                               theta, eps2, _p(sax), _p(say))
    return sax, say, int(inter)


def walk_acc(sx, sy, sm, skeys, tree: Tree, box, theta, eps2, G=1.0, bucket=8, alpha=0.0,
             aold=None, quadrupole=True, group=32):
    """The engine's PLAIN-mode walk restated on the CPU; returns (sax, say, interactions).

    aold: |a| of the previous step per sorted body (None = geometric rule only).
    quadrupole=False: accepted cells as monopoles (the engine's bootstrap pass).
    group: bodies per walk group (32, or 64 for two bodies per lane)."""
    n = len(sx)
    sax = np.zeros(n, np.float32)
    say = np.zeros(n, np.float32)
    sx, sy, sm = _f32(sx), _f32(sy), _f32(sm)
    skeys = np.ascontiguousarray(skeys, dtype=np.uint64)
    inter = lib().orc_walk_acc(n, _p(sx), _p(sy), _p(sm), _p(skeys), _p(tree.left),
                               _p(tree.right), _p(tree.split), _p(tree.first), _p(tree.last),
                               _p(tree.qchild), _p(_f32(box)), theta, eps2, G, bucket, alpha,
                               _p(_f32(aold)) if aold is not None else None,
                               1 if quadrupole else 0, int(group), _p(sax), _p(say))
    return sax, say, int(inter)


def frontier_check(sx, sy, sm, skeys, tree: Tree, box, theta, G=1.0, bucket=8, alpha=0.0,
                   aold=None, group=32, super_=512) -> dict:
    """The engine's shared walk frontiers checked on the CPU (orc_frontier_check):
    groups whose accepted cells or direct bodies differ between the root start
    and the frontier start (0 expected), frontier sizes and node tests."""
    n = len(sx)
    sx, sy, sm = _f32(sx), _f32(sy), _f32(sm)
    out = np.zeros(5, np.int64)
    lib().orc_frontier_check(n, _p(sx), _p(sy), _p(sm),
                             _p(np.ascontiguousarray(skeys, dtype=np.uint64)), _p(tree.left),
                             _p(tree.right), _p(tree.split), _p(tree.first), _p(tree.last),
                             _p(tree.qchild), _p(_f32(box)), theta, G, bucket, alpha,
                             _p(_f32(aold)) if aold is not None else None, int(group),
                             int(super_), _p(out))
    return dict(differing_groups=int(out[0]), frontier_nodes=int(out[1]),
                accepted_cells=int(out[2]), tests_from_root=int(out[3]),
                tests_from_frontier=int(out[4]))


def check_tree(skeys, tree: Tree, sm, node_m, ids, box, left=None, right=None, parent=None,
               leaf_parent=None, first=None, last=None) -> int:
    """Tree invariants of one system (the engine's bh_check restated): the mask
    of failing checks.  Any tree array may be overridden (tests plant errors)."""
    n = len(skeys)
    arr = lambda a, d: np.ascontiguousarray(d if a is None else a, dtype=np.int32)
    return int(lib().orc_check_tree(
        n, _p(np.ascontiguousarray(skeys, dtype=np.uint64)), _p(arr(left, tree.left)),
        _p(arr(right, tree.right)), _p(arr(parent, tree.parent)),
        _p(arr(leaf_parent, tree.leaf_parent)), _p(arr(first, tree.first)),
        _p(arr(last, tree.last)), _p(_f32(sm)), _p(_f32(node_m)),
        _p(np.ascontiguousarray(ids, dtype=np.int32)), _p(_f32(box))))


def render(x, y, width=1000, height=1000, extent=(-25.0, 25.0, -25.0, 25.0)):
    """Headless point rendering (the engine's bh_render restated): uint8 (height, width, 4)."""
    x, y = _f32(x), _f32(y)
    out = np.zeros((height, width, 4), np.uint8)
    lib().orc_render(len(x), _p(x), _p(y), width, height, *[float(e) for e in extent], _p(out))
    return out


def step_ref(x, y, vx, vy, m, theta=0.5, eps2=0.025, dt=1e-3, damp=1.0):
    """One reference step in place on float32 copies; returns (x, y, vx, vy, ax, ay, inter)."""
    x, y, vx, vy, m = [np.array(a, dtype=np.float32) for a in (x, y, vx, vy, m)]
    n = len(x)
    ax = np.zeros(n, np.float32)
    ay = np.zeros(n, np.float32)
    inter = ctypes.c_int64(0)
    st = lib().orc_step_ref(n, _p(x), _p(y), _p(vx), _p(vy), _p(m), _p(ax), _p(ay), theta, eps2,
                            dt, damp, ctypes.byref(inter))
    if st:
        raise ValueError(f"orc_step_ref status {st}")
    return x, y, vx, vy, ax, ay, int(inter.value)


def direct_f64(x, y, m, idx, eps2, G=1.0, xlo=None, ylo=None):
    x, y, m = _f32(x), _f32(y), _f32(m)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    ax = np.zeros(len(idx), np.float64)
    ay = np.zeros(len(idx), np.float64)
    if xlo is None and ylo is None:
        lib().orc_direct_f64(len(x), _p(x), _p(y), _p(m), len(idx), _p(idx), eps2, G, _p(ax),
                             _p(ay))
    else:
        xlo = _f32(xlo) if xlo is not None else None
        ylo = _f32(ylo) if ylo is not None else None
        lib().orc_direct_f64_hilo(len(x), _p(x), _p(xlo), _p(y), _p(ylo), _p(m), len(idx),
                                  _p(idx), eps2, G, _p(ax), _p(ay))
    return ax, ay


def energy_f64(x, y, vx, vy, m, eps2, G=1.0):
    out = np.zeros(4, np.float64)
    arrs = [_f32(a) for a in (x, y, vx, vy, m)]
    lib().orc_energy_f64(len(arrs[0]), *[_p(a) for a in arrs], eps2, G, _p(out))
    return out  # kinetic, potential, px, py


# ---------------------------------------------------------------- canonical form

def lcp_levels(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Number of equal leading 2-bit digits of two uint64 key arrays (32 if equal)."""
    x = np.bitwise_xor(a.astype(np.uint64), b.astype(np.uint64))
    out = np.full(x.shape, 32, np.int32)
    nz = x != 0
    # highest set bit position via float64 log2 is exact enough after a shift guard
    hb = np.zeros(x.shape, np.int32)
    xv = x[nz]
    hb_nz = np.zeros(xv.shape, np.int32)
    for s in (32, 16, 8, 4, 2, 1):
        m = (xv >> np.uint64(s)) != 0
        hb_nz[m] += s
        xv = np.where(m, xv >> np.uint64(s), xv)
    hb[nz] = hb_nz
    out[nz] = (63 - hb[nz]) // 2
    return out


def canonical_from_keys(skeys: np.ndarray):
    """Canonical uncompressed quadtree of sorted distinct keys.

    Returns (depth, cells): depth[j] = leaf depth of the j-th sorted body (root
    children at depth 1); cells = sorted structured array of (level, prefix,
    first, count) for every key prefix shared by >= 2 bodies (level >= 1).
    """
    skeys = np.ascontiguousarray(skeys, dtype=np.uint64)
    n = len(skeys)
    d = lcp_levels(skeys[:-1], skeys[1:]) if n > 1 else np.zeros(0, np.int32)
    prev = np.concatenate([[0], d])
    nxt = np.concatenate([d, [0]])
    depth = (np.maximum(prev, nxt) + 1).astype(np.int32)
    maxd = int(depth.max()) if n else 0
    levels, prefixes, firsts, counts = [], [], [], []
    for lev in range(1, maxd):
        pre = skeys >> np.uint64(64 - 2 * lev)
        brk = np.concatenate([[True], pre[1:] != pre[:-1]])
        starts = np.flatnonzero(brk)
        lens = np.diff(np.concatenate([starts, [n]]))
        sel = lens >= 2
        levels.append(np.full(sel.sum(), lev, np.int32))
        prefixes.append(pre[starts[sel]])
        firsts.append(starts[sel].astype(np.int32))
        counts.append(lens[sel].astype(np.int32))
    cells = _cells_array(levels, prefixes, firsts, counts)
    return depth, cells


def _cells_array(levels, prefixes, firsts, counts):
    dt = np.dtype([("level", np.int32), ("prefix", np.uint64), ("first", np.int32),
                   ("count", np.int32)])
    if not levels:
        return np.zeros(0, dt)
    out = np.zeros(sum(len(a) for a in levels), dt)
    out["level"] = np.concatenate(levels)
    out["prefix"] = np.concatenate(prefixes)
    out["first"] = np.concatenate(firsts)
    out["count"] = np.concatenate(counts)
    out.sort(order=["level", "prefix"])
    return out


def canonical_from_child(child: np.ndarray, count: np.ndarray, n: int, cell_vals=None):
    """Canonical form of a reference-layout tree (kernels.cu child[4*node+slot]).

    Returns (body_depth[n], body_path[n], cells, vals) where body_path is the
    digit path of each body's leaf (depth digits, right aligned) and cells has
    (level, prefix, first=-1, count).  If cell_vals is a tuple of per-node
    arrays, vals holds their values per canonical cell, in the same order.
    """
    body_depth = np.full(n, -1, np.int32)
    body_path = np.zeros(n, np.uint64)
    lv, pf, ct, ids = [], [], [], []
    stack = [(0, 0, 0)]  # node, level, prefix ; node 0 = root slots child[0..3]
    while stack:
        node, level, prefix = stack.pop()
        for s in range(4):
            c = int(child[4 * node + s])
            if c < 0:
                continue
            p = (prefix << 2) | s
            if c >= n:
                lv.append(level + 1)
                pf.append(p)
                ct.append(int(count[c]))
                ids.append(c)
                stack.append((c, level + 1, p))
            else:
                if body_depth[c] != -1:
                    raise ValueError(f"body {c} appears twice")
                body_depth[c] = level + 1
                body_path[c] = p
    cells = _cells_array([np.array(lv, np.int32)], [np.array(pf, np.uint64)],
                         [np.full(len(lv), -1, np.int32)], [np.array(ct, np.int32)])
    vals = None
    if cell_vals is not None:
        order = np.lexsort((np.array(pf, np.uint64), np.array(lv, np.int32)))
        ids = np.array(ids, np.int64)[order]
        vals = tuple(np.asarray(v)[ids] for v in cell_vals)
    return body_depth, body_path, cells, vals


def body_paths_from_keys(keys: np.ndarray, depth_by_body: np.ndarray) -> np.ndarray:
    keys = keys.astype(np.uint64)
    return keys >> (np.uint64(64) - 2 * depth_by_body.astype(np.uint64))
