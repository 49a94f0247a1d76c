"""Pin the CPU oracle against golden vectors from the reference's own kernels.

The fixtures (tests/golden/*.npz) hold one reference update() per case, run
from the reference's kernels.cu (pentilm/StellarSolver) on the host; see
tests/golden/make_golden.py.  Tolerances:
  box, sort permutation, tree topology (leaf depths, leaf paths, cell set and
  cell counts): bit-exact;
  centre of mass: the reference sums with float atomics in arrival order
  (kernels.cu:180-183), the oracle sums left+right in a binary tree, so they
  agree to a few float ulps of the box extent;
  forces: same interaction set, different summation order and rsqrt.  The
  error is normalised by the RMS acceleration of the case.  FORCE_TOL holds
  the bound per case.  clustered512 has a 1e-3-wide clump of 255 bodies at
  distance 3.  Its float centre of mass carries an order-dependent rounding of
  about 1e-5, and the reference leaves that order to atomic arrival, so its
  bound is looser.
"""
import numpy as np
import pytest

import golden_cases as gc

FORCE_TOL = {"disk4096": 5e-6, "plummer2048": 5e-6, "clustered512": 1e-3}
# state after 1 and 3 steps, error / max|value|: dt * (force error) on top of ulps
TRAJ_TOL = {"disk4096": 1e-6, "plummer2048": 1e-6, "clustered512": 2e-4}


@pytest.fixture(scope="module", params=gc.CASES)
def case(request):
    g = gc.load(request.param)
    g["name"] = request.param
    return g


def _oracle_tree(oracle, g):
    box = oracle.bbox(g["x"], g["y"])
    keys = oracle.keys(g["x"], g["y"], box)
    perm, dups = oracle.sort_keys(keys)
    return box, keys, perm, dups


def test_box_bit_exact(oracle, case):
    box = oracle.bbox(case["x"], case["y"])
    assert np.array_equal(box.view(np.uint32), case["box"].view(np.uint32))


def test_sort_permutation_bit_exact(oracle, case):
    _, _, perm, dups = _oracle_tree(oracle, case)
    assert dups == 0
    assert np.array_equal(perm.astype(np.int32), case["sorted"])


def test_topology_bit_exact(oracle, case):
    _, keys, perm, _ = _oracle_tree(oracle, case)
    depth, cells = oracle.canonical_from_keys(keys[perm])
    n = int(case["n"])
    dby = np.zeros(n, np.int32)
    dby[perm] = depth
    assert np.array_equal(dby, case["body_depth"])
    assert np.array_equal(oracle.body_paths_from_keys(keys, dby), case["body_path"])
    assert len(cells) == int(case["ncells"])
    assert np.array_equal(cells["level"], case["cell_level"])
    assert np.array_equal(cells["prefix"], case["cell_prefix"])
    assert np.array_equal(cells["count"], case["cell_count"])


def test_debug_invariants_of_golden(case):
    """debug.cpp:23-174 invariants hold on the reference's own output."""
    n = int(case["n"])
    s = case["sorted"]
    assert int(s.astype(np.int64).sum()) == n * (n - 1) // 2
    assert np.array_equal(np.sort(s), np.arange(n))
    b = case["box"]
    assert b[0] <= b[1] and b[2] <= b[3]
    assert b[0] <= 0 <= b[1] and b[2] <= 0 <= b[3]


def _cell_com_from_oracle(oracle, g, keys, perm):
    """Per canonical cell: the oracle's COM of the quadtree node owning it."""
    sk = keys[perm]
    t = oracle.Tree(sk)
    sx, sy, sm = g["x"][perm], g["y"][perm], g["m"][perm]
    nm, nmx, nmy, ncx, ncy = t.sums(sx, sy, sm)
    # every canonical cell (level, prefix, count) maps to the deepest binary node
    # whose body range is exactly the cell's range
    depth, cells = oracle.canonical_from_keys(sk)
    rng = {(int(f), int(l)): i for i, (f, l) in enumerate(zip(t.first, t.last))}
    idx = np.array([rng[(int(c["first"]), int(c["first"] + c["count"] - 1))] for c in cells])
    return cells, nm[idx], ncx[idx], ncy[idx], nmx[idx], nmy[idx]


def test_centre_of_mass(oracle, case):
    box, keys, perm, _ = _oracle_tree(oracle, case)
    cells, m, cx, cy, mx, my = _cell_com_from_oracle(oracle, case, keys, perm)
    ext = float(max(box[1] - box[0], box[3] - box[2]))
    assert np.allclose(m, case["cell_m"], rtol=2e-6, atol=0)
    assert np.max(np.abs(cx - case["cell_cx"])) <= 64 * np.finfo(np.float32).eps * ext
    assert np.max(np.abs(cy - case["cell_cy"])) <= 64 * np.finfo(np.float32).eps * ext


def test_forces(oracle, case):
    box, keys, perm, _ = _oracle_tree(oracle, case)
    g = case
    sk = keys[perm]
    t = oracle.Tree(sk)
    sx, sy, sm = g["x"][perm], g["y"][perm], g["m"][perm]
    nm, _, _, ncx, ncy = t.sums(sx, sy, sm)
    sax, say, inter = oracle.walk_ref(sx, sy, sm, t, nm, ncx, ncy, box, float(g["theta"]),
                                      float(g["eps2"]))
    n = int(g["n"])
    ax = np.zeros(n, np.float32)
    ay = np.zeros(n, np.float32)
    ax[perm] = sax
    ay[perm] = say
    err = np.hypot(ax - g["ax"], ay - g["ay"])
    rms = np.sqrt(np.mean(g["ax"].astype(np.float64) ** 2 + g["ay"].astype(np.float64) ** 2))
    assert err.max() / rms <= FORCE_TOL[g["name"]], err.max() / rms
    rel = err / np.hypot(g["ax"], g["ay"])
    assert np.median(rel) < 1e-5
    assert inter > n


def test_step_and_trajectory(oracle, case):
    g = case
    args = dict(theta=float(g["theta"]), eps2=float(g["eps2"]), dt=float(g["dt"]),
                damp=float(g["damp"]))
    x, y, vx, vy = g["x"], g["y"], g["vx"], g["vy"]
    for step in range(int(g["steps"])):
        x, y, vx, vy, ax, ay, _ = oracle.step_ref(x, y, vx, vy, g["m"], **args)
        if step == 0:
            for a, b in ((x, g["x1"]), (y, g["y1"]), (vx, g["vx1"]), (vy, g["vy1"])):
                scale = np.abs(b).max()
                assert np.max(np.abs(a - b)) <= TRAJ_TOL[g["name"]] * scale
    for a, b in ((x, g["x3"]), (y, g["y3"]), (vx, g["vx3"]), (vy, g["vy3"])):
        scale = np.abs(b).max()
        assert np.max(np.abs(a - b)) <= 3 * TRAJ_TOL[g["name"]] * scale
