"""The drop-in wrappers (include/Particle_cuda.cuh) on the reference's layout.

Runs the reference's update() sequence (BarnesHutParticleSystem.cpp:308-315)
through the nine wrappers on device arrays of length m = 2n+12000, phase by
phase, and compares every phase with the golden fixtures made by the
reference's own kernels: box, tree (canonical form), counts, sorted[] and
start[] bit-exact; centres of mass, forces and the integrated state within the
tolerances of test_oracle_golden.py.  debug.cpp's invariants must hold too.
"""
import numpy as np
import pytest

import golden_cases as gc
from test_oracle_golden import FORCE_TOL, TRAJ_TOL

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def L():
    import compat_lib

    lib = compat_lib.load()
    lib.bh_compat_set_constants(0.5, 0.025)
    return lib


def P(t):
    return t.data_ptr()


class RefArrays:
    """Device arrays laid out like BarnesHutParticleSystem.cpp:54-83."""

    def __init__(self, g):
        n = int(g["n"])
        m = 2 * n + 12000
        self.n, self.m = n, m
        dev = "cuda"
        f = lambda: torch.zeros(m, dtype=torch.float32, device=dev)  # noqa: E731
        self.x, self.y, self.vx, self.vy, self.mass, self.ax, self.ay = (f() for _ in range(7))
        for t, k in ((self.x, "x"), (self.y, "y"), (self.vx, "vx"), (self.vy, "vy"),
                     (self.mass, "m")):
            t[:n] = torch.from_numpy(g[k])
        i = lambda k=1: torch.zeros(k * m, dtype=torch.int32, device=dev)  # noqa: E731
        self.count, self.start, self.sorted, self.child = i(), i(), i(), i(4)
        self.index = torch.zeros(1, dtype=torch.int32, device=dev)
        self.mutex = torch.zeros(1, dtype=torch.int32, device=dev)
        self.box = [torch.zeros(1, dtype=torch.float32, device=dev) for _ in range(4)]
        self.out = torch.zeros(2 * m, dtype=torch.float32, device=dev)


def update(L, a, dt, damp, rec):
    n, m = a.n, a.m
    bx = [P(b) for b in a.box]
    L.ResetArrays(P(a.mutex), P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.sorted),
                  P(a.child), P(a.index), *bx, n, m)
    L.ComputeBoundingBox(P(a.mutex), P(a.x), P(a.y), *bx, n)
    torch.cuda.synchronize()
    rec["box"] = np.array([float(b.item()) for b in a.box], np.float32)
    L.BuildQuadTree(P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.child), P(a.index),
                    *bx, n, m)
    torch.cuda.synchronize()
    rec["sums"] = (a.x.cpu().numpy(), a.y.cpu().numpy(), a.mass.cpu().numpy())
    L.ComputeCentreOfMass(P(a.x), P(a.y), P(a.mass), P(a.index), n)
    L.SortParticles(P(a.count), P(a.start), P(a.sorted), P(a.child), P(a.index), n)
    L.CalculateForces(P(a.x), P(a.y), P(a.vx), P(a.vy), P(a.ax), P(a.ay), P(a.mass), P(a.sorted),
                      P(a.child), bx[0], bx[1], n, 1.0)
    torch.cuda.synchronize()
    rec["child"] = a.child.cpu().numpy()
    rec["count"] = a.count.cpu().numpy()
    rec["start"] = a.start.cpu().numpy()
    rec["index"] = int(a.index.item())
    rec["com"] = (a.x.cpu().numpy(), a.y.cpu().numpy(), a.mass.cpu().numpy())
    rec["sorted"] = a.sorted.cpu().numpy()
    rec["ax"] = a.ax[:n].cpu().numpy()
    rec["ay"] = a.ay[:n].cpu().numpy()
    L.IntegrateParticles(P(a.x), P(a.y), P(a.vx), P(a.vy), P(a.ax), P(a.ay), n, dt, damp)
    L.FillOutputArray(P(a.x), P(a.y), P(a.out), m)
    torch.cuda.synchronize()
    rec["out"] = a.out.cpu().numpy()
    rec["state"] = tuple(t[:n].cpu().numpy() for t in (a.x, a.y, a.vx, a.vy))


@pytest.fixture(scope="module", params=gc.CASES)
def run(request, L):
    g = gc.load(request.param)
    g["name"] = request.param
    a = RefArrays(g)
    L.bh_compat_clear_status()
    rec = {}
    update(L, a, float(g["dt"]), float(g["damp"]), rec)
    rec["status1"] = L.bh_compat_status()
    for _ in range(int(g["steps"]) - 1):
        update(L, a, float(g["dt"]), float(g["damp"]), {})
    rec["state3"] = tuple(t[: a.n].cpu().numpy() for t in (a.x, a.y, a.vx, a.vy))
    rec["status3"] = L.bh_compat_status()
    return g, rec


def test_status_ok(run):
    _, rec = run
    assert rec["status1"] == 0 and rec["status3"] == 0


def test_box_bit_exact(run):
    g, rec = run
    assert np.array_equal(rec["box"].view(np.uint32), g["box"].view(np.uint32))


def test_tree_bit_exact(run, oracle):
    g, rec = run
    n = int(g["n"])
    bd, bp, cells, vals = oracle.canonical_from_child(rec["child"], rec["count"], n, rec["com"])
    assert np.array_equal(bd, g["body_depth"])
    assert np.array_equal(bp, g["body_path"])
    assert np.array_equal(cells["level"], g["cell_level"])
    assert np.array_equal(cells["prefix"], g["cell_prefix"])
    assert np.array_equal(cells["count"], g["cell_count"])
    assert rec["index"] - n == int(g["ncells"])
    box = g["box"]
    ext = float(max(box[1] - box[0], box[3] - box[2]))
    tol = 64 * np.finfo(np.float32).eps * ext
    assert np.max(np.abs(vals[0] - g["cell_cx"])) <= tol
    assert np.max(np.abs(vals[1] - g["cell_cy"])) <= tol
    assert np.allclose(vals[2], g["cell_m"], rtol=2e-6, atol=0)


def test_sorted_bit_exact(run):
    g, rec = run
    n = int(g["n"])
    assert np.array_equal(rec["sorted"][:n], g["sorted"])


def test_forces_and_integration(run):
    g, rec = run
    rms = np.sqrt(np.mean(g["ax"].astype(np.float64) ** 2 + g["ay"].astype(np.float64) ** 2))
    err = np.hypot(rec["ax"] - g["ax"], rec["ay"] - g["ay"]).max() / rms
    assert err <= FORCE_TOL[g["name"]], err
    tol = TRAJ_TOL[g["name"]]
    for a, ref in zip(rec["state"], ("x1", "y1", "vx1", "vy1")):
        assert np.max(np.abs(a - g[ref])) <= tol * np.abs(g[ref]).max(), ref
    for a, ref in zip(rec["state3"], ("x3", "y3", "vx3", "vy3")):
        assert np.max(np.abs(a - g[ref])) <= 3 * tol * np.abs(g[ref]).max(), ref


def test_output_buffer(run):
    _, rec = run
    x, y = rec["state"][0], rec["state"][1]
    n = len(x)
    assert np.array_equal(rec["out"][0:2 * n:2], x)
    assert np.array_equal(rec["out"][1:2 * n:2], y)


def test_debug_invariants(run):
    """debug.cpp:23-174 on the wrappers' own output."""
    g, rec = run
    n = int(g["n"])
    m = 2 * n + 12000
    child = rec["child"].astype(np.int64)
    count = rec["count"]
    ch = child.reshape(m, 4)
    kids = np.where(ch[n:] >= 0, count[np.clip(ch[n:], 0, m - 1)], 0).sum(1)
    assert np.array_equal(kids, count[n:])                                  # COUNT 1
    assert child[(child >= 0) & (child < n)].sum() == n * (n - 1) // 2     # CHILD 1
    assert (child < m).all()                                                # CHILD 2
    assert (child >= -1).all()                                              # CHILD 3
    s = rec["sorted"][:n]
    assert np.array_equal(np.sort(s), np.arange(n))                          # SORTED 1, 2
    assert rec["box"][0] <= rec["box"][1] and rec["box"][2] <= rec["box"][3]  # BOX 1
    # start[] of every cell is the first sorted position of its bodies
    st = rec["start"]
    cells = np.arange(n, rec["index"])
    assert (st[cells] >= 0).all()


def test_two_systems_alternating(L):
    """Two systems of different sizes (disk 4096, clustered 512) stepped in
    turn through the nine wrappers on one device: each build replaces the
    device's workspace layout record, and every step must still match the
    golden outputs of its own system."""
    cases = [gc.load("disk4096"), gc.load("clustered512")]
    names = ["disk4096", "clustered512"]
    arrs = [RefArrays(g) for g in cases]
    L.bh_compat_clear_status()
    first = [{}, {}]
    steps = int(cases[0]["steps"])
    assert steps == int(cases[1]["steps"])
    for k in range(steps):
        for i, (g, a) in enumerate(zip(cases, arrs)):
            update(L, a, float(g["dt"]), float(g["damp"]), first[i] if k == 0 else {})
    assert L.bh_compat_status() == 0
    for g, a, rec, name in zip(cases, arrs, first, names):
        n = int(g["n"])
        assert np.array_equal(rec["box"].view(np.uint32), g["box"].view(np.uint32)), name
        assert np.array_equal(rec["sorted"][:n], g["sorted"]), name
        rms = np.sqrt(np.mean(g["ax"].astype(np.float64) ** 2 + g["ay"].astype(np.float64) ** 2))
        err = np.hypot(rec["ax"] - g["ax"], rec["ay"] - g["ay"]).max() / rms
        assert err <= FORCE_TOL[name], (name, err)
        tol = TRAJ_TOL[name]
        final = tuple(t[:n].cpu().numpy() for t in (a.x, a.y, a.vx, a.vy))
        for v, ref in zip(final, ("x3", "y3", "vx3", "vy3")):
            assert np.max(np.abs(v - g[ref])) <= 3 * tol * np.abs(g[ref]).max(), (name, ref)


def test_unaligned_child_array(L):
    """child[] 4 bytes off a 16-byte boundary (a caller's sub-array): the whole
    update() gives exactly the results of an aligned child[] (CalculateForces,
    and a SortParticles without the build's workspace, read its slots one by
    one there)."""
    g = gc.load("plummer2048")
    n = int(g["n"])
    outs = []
    for offset in (0, 1):
        a = RefArrays(g)
        big = torch.zeros(4 * a.m + 4, dtype=torch.int32, device="cuda")
        a.child = big[offset:offset + 4 * a.m]
        L.bh_compat_clear_status()
        rec = {}
        update(L, a, float(g["dt"]), float(g["damp"]), rec)
        assert L.bh_compat_status() == 0
        outs.append(rec)
    for k in ("sorted", "start", "count"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
    assert np.array_equal(outs[0]["ax"].view(np.uint32), outs[1]["ax"].view(np.uint32))
    assert np.array_equal(outs[0]["sorted"][:n], g["sorted"])


@pytest.mark.parametrize("n", [1 << 17, (1 << 18) + 333])
def test_dropin_update_matches_reference_mode(L, n):
    """The drop-in update() (the reference layout, with SortParticles and
    CalculateForces taken from BuildQuadTree's workspace) against the engine's
    REFERENCE mode on the same Plummer state (its own step, box, tree and
    graph): sorted[] equals the engine's permutation (both are the bodies in
    key order), the forces agree to 1e-5 of their RMS (the same interaction
    set, summed in another order), and the integrated positions to 1e-5 of
    their extent."""
    from stellarsolver_gb300 import bh, dropin, models

    x, y, vx, vy, m = models.plummer(n, 0x5EEDC0DE)
    eps2, dt = 1e-4, 1e-4
    L.bh_compat_set_constants(0.5, eps2)
    L.bh_compat_clear_status()
    a = dropin.RefArrays(torch, x, y, vx, vy, m)
    dropin.update(L, a, dt, 1.0)
    torch.cuda.synchronize()
    assert L.bh_compat_status() == 0
    L.bh_compat_set_constants(0.5, 0.025)  # the fixtures' constants, for the other tests
    sorted_ = a.sorted[:n].cpu().numpy()
    dax, day = a.ax[:n].cpu().numpy(), a.ay[:n].cpu().numpy()
    dx1, dy1 = a.x[:n].cpu().numpy(), a.y[:n].cpu().numpy()
    with bh.BarnesHutSystem(n, mode="reference", theta=0.5, eps2=eps2, timestep=dt) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(1)
        s.sync()
        perm = s.debug("perm")
        eax, eay = s.get_accel()
        st = s.get_state()
    assert np.array_equal(sorted_, perm)
    r = np.sqrt(np.mean(eax.astype(np.float64) ** 2 + eay.astype(np.float64) ** 2))
    assert np.hypot(dax - eax, day - eay).max() <= 1e-5 * r
    ext = max(np.ptp(x), np.ptp(y))
    assert max(np.abs(dx1 - st["x"]).max(), np.abs(dy1 - st["y"]).max()) <= 1e-5 * ext


@pytest.mark.parametrize("case", ["plummer2048", "plummer2e17"])
def test_sort_and_forces_from_build_equal_the_layout_walks(L, case):
    """SortParticles and CalculateForces right after BuildQuadTree on the same
    arrays work from the build: sorted[] and start[] (depth-first order is key
    order), and the vote walk on its compressed tree.  On a copy of the built
    count[] and child[] at other addresses they walk the reference's layout:
    the cells level by level (kernels.cu:299-335), the vote over child[]
    (kernels.cu:340-435).  The arrays are identical and the forces agree to
    1e-5 of their RMS (the same interaction set, summed in another order)."""
    from stellarsolver_gb300 import dropin, models

    if case == "plummer2048":
        g = gc.load(case)
        arrays = [g[k] for k in ("x", "y", "vx", "vy", "m")]
    else:
        arrays = models.plummer(1 << 17, 0x5EEDC0DF)
    a = dropin.RefArrays(torch, *arrays)
    n, m = a.n, a.m
    bx = [P(b) for b in a.box]
    L.bh_compat_clear_status()
    L.ResetArrays(P(a.mutex), P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.sorted),
                  P(a.child), P(a.index), *bx, n, m)
    L.ComputeBoundingBox(P(a.mutex), P(a.x), P(a.y), *bx, n)
    L.BuildQuadTree(P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.child), P(a.index),
                    *bx, n, m)
    L.ComputeCentreOfMass(P(a.x), P(a.y), P(a.mass), P(a.index), n)
    torch.cuda.synchronize()
    count2, start2, child2 = a.count.clone(), a.start.clone(), a.child.clone()
    sorted2 = a.sorted.clone()
    L.SortParticles(P(a.count), P(a.start), P(a.sorted), P(a.child), P(a.index), n)
    L.SortParticles(P(count2), P(start2), P(sorted2), P(child2), P(a.index), n)
    ax2, ay2 = a.ax.clone(), a.ay.clone()
    L.CalculateForces(P(a.x), P(a.y), P(a.vx), P(a.vy), P(a.ax), P(a.ay), P(a.mass), P(a.sorted),
                      P(a.child), bx[0], bx[1], n, 1.0)
    L.CalculateForces(P(a.x), P(a.y), P(a.vx), P(a.vy), P(ax2), P(ay2), P(a.mass), P(sorted2),
                      P(child2), bx[0], bx[1], n, 1.0)
    torch.cuda.synchronize()
    assert L.bh_compat_status() == 0
    f1 = np.stack([a.ax[:n].cpu().numpy(), a.ay[:n].cpu().numpy()]).astype(np.float64)
    f2 = np.stack([ax2[:n].cpu().numpy(), ay2[:n].cpu().numpy()]).astype(np.float64)
    rms = np.sqrt(np.mean(np.sum(f2 ** 2, axis=0)))
    assert np.abs(f1 - f2).max() <= 1e-5 * rms
    cells = int(a.index.item())
    assert cells > n
    assert np.array_equal(a.sorted.cpu().numpy(), sorted2.cpu().numpy())
    assert np.array_equal(a.start.cpu().numpy(), start2.cpu().numpy())
    st = a.start[n:cells].cpu().numpy()
    assert (st >= 0).all() and (st < n).all()
    assert np.array_equal(np.sort(a.sorted[:n].cpu().numpy()), np.arange(n))


@pytest.mark.parametrize("packed", [0, 600])
def test_build_with_the_full_sort(L, oracle, packed):
    """600 bodies 1e-8 apart in one 2^-12 cell of the box make a run of equal
    high key words longer than the fixup orders, so BuildQuadTree takes the
    full 8-pass sort (one cooperative kernel; with `packed` 0 it returns at
    once).  sorted[] equals the oracle's stable sort of the keys either way."""
    from stellarsolver_gb300 import dropin

    n = 8192
    rng = np.random.default_rng(31 + packed)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    i = np.arange(packed)
    x[:packed] = np.float32(1e-3) + (i * 1e-8).astype(np.float32)
    y[:packed] = np.float32(2e-3) + ((i % 7) * 1e-8).astype(np.float32)
    perm = rng.permutation(n)
    x, y = x[perm], y[perm]
    m = np.full(n, 1.0 / n, np.float32)
    z = np.zeros(n, np.float32)
    box = oracle.bbox(x, y)
    k = oracle.keys(x, y, box)
    _, runs = np.unique(k >> np.uint64(40), return_counts=True)
    assert (runs.max() > 256) == (packed > 0)
    want, _ = oracle.sort_keys(k)
    a = dropin.RefArrays(torch, x, y, z, z, m)
    bx = [P(b) for b in a.box]
    L.bh_compat_clear_status()
    L.ResetArrays(P(a.mutex), P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.sorted),
                  P(a.child), P(a.index), *bx, n, a.m)
    L.ComputeBoundingBox(P(a.mutex), P(a.x), P(a.y), *bx, n)
    L.BuildQuadTree(P(a.x), P(a.y), P(a.mass), P(a.count), P(a.start), P(a.child), P(a.index),
                    *bx, n, a.m)
    L.ComputeCentreOfMass(P(a.x), P(a.y), P(a.mass), P(a.index), n)
    L.SortParticles(P(a.count), P(a.start), P(a.sorted), P(a.child), P(a.index), n)
    torch.cuda.synchronize()
    assert L.bh_compat_status() == 0
    assert np.array_equal(a.sorted[:n].cpu().numpy(), want.astype(np.int32))
