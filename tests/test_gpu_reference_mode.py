"""REFERENCE mode on the GPU, through the C ABI, against the reference.

Two anchors:
  * golden fixtures from the reference's own kernels (tests/golden/);
  * the oracle (oracle/oracle.c) on the same inputs, at sizes up to 2^20.
Tolerances:
  box, keys, sort permutation, tree topology, node sums and centres of mass
  vs the oracle: bit-exact (same float operations in the same order);
  forces vs the oracle: identical interaction sets, the GPU's rsqrtf differs
  from the oracle's 1/sqrtf by a few ulp: max |da| <= 1e-5 * RMS|a|;
  vs golden: the tolerances of test_oracle_golden.py (the reference sums
  centres of mass in atomic arrival order).
"""
import numpy as np
import pytest

import golden_cases as gc
from test_oracle_golden import FORCE_TOL, TRAJ_TOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def make(bh, n, eps2=0.025, theta=0.5, dt=1e-3, damp=1.0, **kw):
    return bh.BarnesHutSystem(n, mode="reference", theta=theta, eps2=eps2, timestep=dt,
                              dampening=damp, **kw)


def rms(ax, ay):
    return float(np.sqrt(np.mean(ax.astype(np.float64) ** 2 + ay.astype(np.float64) ** 2)))


@pytest.fixture(scope="module", params=gc.CASES)
def golden_run(request, bh):
    g = gc.load(request.param)
    g["name"] = request.param
    n = int(g["n"])
    with make(bh, n, float(g["eps2"]), float(g["theta"]), float(g["dt"]), float(g["damp"])) as s:
        s.set_state(g["x"], g["y"], g["vx"], g["vy"], g["m"])
        s.step(1)
        s.sync()
        out = dict(box=s.debug("box"), keys=s.debug("keys"), perm=s.debug("perm"),
                   first=s.debug("node_first"), last=s.debug("node_last"),
                   cx=s.debug("node_cx"), cy=s.debug("node_cy"), m=s.debug("node_m"),
                   accel=s.get_accel(), state1=s.get_state(), stats=s.stats())
        s.step(int(g["steps"]) - 1)
        s.sync()
        out["state3"] = s.get_state()
    return g, out


def test_golden_box_bit_exact(golden_run):
    g, o = golden_run
    assert np.array_equal(o["box"].view(np.uint32), g["box"].view(np.uint32))


def test_golden_sort_permutation_bit_exact(golden_run):
    g, o = golden_run
    assert np.array_equal(o["perm"], g["sorted"])


def test_golden_topology_bit_exact(golden_run, oracle):
    g, o = golden_run
    n = int(g["n"])
    depth, cells = oracle.canonical_from_keys(o["keys"])
    dby = np.zeros(n, np.int32)
    dby[o["perm"]] = depth
    assert np.array_equal(dby, g["body_depth"])
    keys_by_body = np.zeros(n, np.uint64)
    keys_by_body[o["perm"]] = o["keys"]
    assert np.array_equal(oracle.body_paths_from_keys(keys_by_body, dby), g["body_path"])
    assert np.array_equal(cells["level"], g["cell_level"])
    assert np.array_equal(cells["prefix"], g["cell_prefix"])
    assert np.array_equal(cells["count"], g["cell_count"])
    assert o["stats"]["cells"] == int(g["ncells"])


def test_golden_centre_of_mass(golden_run, oracle):
    g, o = golden_run
    _, cells = oracle.canonical_from_keys(o["keys"])
    rng = {(int(f), int(l)): i for i, (f, l) in enumerate(zip(o["first"], o["last"]))}
    idx = np.array([rng[(int(c["first"]), int(c["first"] + c["count"] - 1))] for c in cells])
    box = g["box"]
    ext = float(max(box[1] - box[0], box[3] - box[2]))
    assert np.allclose(o["m"][idx], g["cell_m"], rtol=2e-6, atol=0)
    tol = 64 * np.finfo(np.float32).eps * ext
    assert np.max(np.abs(o["cx"][idx] - g["cell_cx"])) <= tol
    assert np.max(np.abs(o["cy"][idx] - g["cell_cy"])) <= tol


def test_golden_forces(golden_run):
    g, o = golden_run
    ax, ay = o["accel"]
    err = np.hypot(ax - g["ax"], ay - g["ay"]).max() / rms(g["ax"], g["ay"])
    assert err <= FORCE_TOL[g["name"]], err


def test_golden_trajectory(golden_run):
    g, o = golden_run
    tol = TRAJ_TOL[g["name"]]
    for k, ref in (("x", "x1"), ("y", "y1"), ("vx", "vx1"), ("vy", "vy1")):
        a, b = o["state1"][k], g[ref]
        assert np.max(np.abs(a - b)) <= tol * np.abs(b).max(), k
    for k, ref in (("x", "x3"), ("y", "y3"), ("vx", "vx3"), ("vy", "vy3")):
        a, b = o["state3"][k], g[ref]
        assert np.max(np.abs(a - b)) <= 3 * tol * np.abs(b).max(), k


# ------------------------------------------------------------------ vs oracle

def _inputs(kind, n, seed):
    from stellarsolver_gb300 import models

    if kind == "plummer":
        return models.plummer(n, seed)
    return models.disk(n, seed)


@pytest.mark.parametrize("kind,n", [("plummer", 1 << 16), ("disk", 1 << 16), ("plummer", 1 << 20)])
def test_oracle_bit_exact_tree_and_forces(bh, oracle, kind, n):
    x, y, vx, vy, m = _inputs(kind, n, 0x5EED1000 + n)
    eps2 = 1e-4 if kind == "plummer" else 0.01
    with make(bh, n, eps2=eps2, dt=1e-4) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(1)
        s.sync()
        box = s.debug("box")
        keys = s.debug("keys")
        perm = s.debug("perm")
        nodes = {k: s.debug("node_" + k) for k in ("left", "right", "split", "first", "last",
                                                    "m", "mx", "my", "cx", "cy")}
        ax, ay = s.get_accel()
        st = s.get_state()
        stats = s.stats()
    obox = oracle.bbox(x, y)
    assert np.array_equal(box.view(np.uint32), obox.view(np.uint32))
    okeys = oracle.keys(x, y, obox)
    operm, dups = oracle.sort_keys(okeys)
    assert dups == 0
    assert np.array_equal(perm, operm.astype(np.int32))
    assert np.array_equal(keys, okeys[operm])
    t = oracle.Tree(okeys[operm])
    for k in ("left", "right", "split", "first", "last"):
        assert np.array_equal(nodes[k][: n - 1], getattr(t, k)), k
    sx, sy, sm = x[operm], y[operm], m[operm]
    om, omx, omy, ocx, ocy = t.sums(sx, sy, sm)
    for k, ref in (("m", om), ("mx", omx), ("my", omy), ("cx", ocx), ("cy", ocy)):
        assert np.array_equal(nodes[k][: n - 1].view(np.uint32), ref.view(np.uint32)), k
    sax, say, inter = oracle.walk_ref(sx, sy, sm, t, om, ocx, ocy, obox, 0.5, eps2)
    oax = np.zeros(n, np.float32)
    oay = np.zeros(n, np.float32)
    oax[operm] = sax
    oay[operm] = say
    err = np.hypot(ax - oax, ay - oay).max() / rms(oax, oay)
    assert err <= 1e-5, err
    assert stats["interactions"] == inter
    # integration: v += dt*a, x += d*dt*v with the GPU's own a (bit-exact op order)
    vx1 = (vx + np.float32(1e-4) * ax).astype(np.float32)
    x1 = (x + np.float32(1e-4) * vx1).astype(np.float32)
    assert np.array_equal(st["vx"], vx1)
    assert np.array_equal(st["x"], x1)


# ------------------------------------------------------------------ edge cases

def test_single_body_and_pair(bh):
    with make(bh, 1) as s:
        s.set_state([1.0], [2.0], [0.5], [0.0], [3.0])
        s.step(2)
        s.sync()
        st = s.get_state()
        assert st["vx"][0] == np.float32(0.5)
        ax, ay = s.get_accel()
        assert ax[0] == 0 and ay[0] == 0
    with make(bh, 2) as s:
        s.set_state([-1.0, 1.0], [0.0, 0.0], [0, 0], [0, 0], [1.0, 1.0])
        s.step(1)
        s.sync()
        ax, _ = s.get_accel()
        expect = 2.0 / (4.0 + 0.025) ** 1.5
        assert np.allclose(ax, [expect, -expect], rtol=1e-6)


@pytest.mark.parametrize("n", [3, 33, 95, 1000])
def test_partial_warps_match_oracle(bh, oracle, n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-10, 10, n).astype(np.float32)
    y = rng.uniform(-3, 12, n).astype(np.float32)
    v = np.zeros(n, np.float32)
    m = rng.uniform(0.5, 1.5, n).astype(np.float32)
    with make(bh, n) as s:
        s.set_state(x, y, v, v, m)
        s.step(1)
        s.sync()
        ax, ay = s.get_accel()
        perm = s.debug("perm")
    _, _, _, _, oax, oay, _ = oracle.step_ref(x, y, v, v, m)
    operm, _ = oracle.sort_keys(oracle.keys(x, y, oracle.bbox(x, y)))
    assert np.array_equal(perm, operm.astype(np.int32))
    assert np.hypot(ax - oax, ay - oay).max() <= 1e-5 * rms(oax, oay)


def test_duplicate_bodies_are_reported(bh):
    x = np.array([0.0, 1.0, 1.0, -2.0], np.float32)
    y = np.array([0.0, 1.0, 1.0, 3.0], np.float32)
    z = np.zeros(4, np.float32)
    with make(bh, 4) as s:
        s.set_state(x, y, z, z, np.ones(4, np.float32))
        s.step(1)
        with pytest.raises(bh.BHError) as e:
            s.sync()
        assert e.value.code == 2  # BH_ERR_DUPLICATE_KEYS


def test_nonfinite_is_reported(bh):
    x = np.array([0.0, np.nan, 1.0], np.float32)
    z = np.zeros(3, np.float32)
    with make(bh, 3) as s:
        s.set_state(x, np.array([0, 1, 2], np.float32), z, z, np.ones(3, np.float32))
        s.step(1)
        with pytest.raises(bh.BHError) as e:
            s.sync()
        assert e.value.code == 3  # BH_ERR_NONFINITE


def test_graph_replay_is_bitwise_identical(bh):
    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.plummer(1 << 14, 99)
    outs = []
    for graph in (False, True):
        with make(bh, len(x), eps2=1e-4, dt=1e-4, use_graph=graph) as s:
            s.set_state(x, y, vx, vy, m)
            s.step(5)
            s.sync()
            outs.append(s.get_state())
    for k in ("x", "y", "vx", "vy"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
