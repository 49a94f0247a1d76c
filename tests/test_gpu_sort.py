"""The engine's sort on the GPU: stable passes over the key's top 24 bits (the
high word; top 32 bits for systems over 2^21 bodies), then each run of equal
high words ordered by the whole key; a run longer than 256 bodies (bodies
packed into one 2^-12 cell of the box) sends the step to
the full 8-pass sort, behind a conditional node in a graph replay and as
kernels gated by a device flag in stream order.

Every case compares the sort permutation and the sorted keys with the oracle's
stable sort, bit for bit, in stream order and as a graph replay, and the tree
built from them with bh_check."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def clustered(n, packed, seed):
    """n - packed bodies spread over a few units, plus `packed` bodies 1e-8
    apart near (1e-3, 2e-3): one 2^-12 cell of the box, distinct keys at 32
    levels."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    i = np.arange(packed)
    x[:packed] = np.float32(1e-3) + (i * 1e-8).astype(np.float32)
    y[:packed] = np.float32(2e-3) + ((i % 7) * 1e-8).astype(np.float32)
    perm = rng.permutation(n)
    x, y = x[perm], y[perm]
    vx = np.zeros(n, np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    return x, y, vx, vx.copy(), m


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("packed", [0, 200, 600])
def test_permutation_bit_exact(bh, oracle, graph, packed):
    n = 8192
    x, y, vx, vy, m = clustered(n, packed, 11 + packed)
    box = oracle.bbox(x, y)
    k = oracle.keys(x, y, box)
    hi = k >> np.uint64(40)  # the high word: the top 24 bits
    _, runs = np.unique(hi, return_counts=True)
    if packed == 600:
        assert runs.max() > 256  # the case that needs the full sort
    else:
        assert runs.max() <= 256
    operm, _ = oracle.sort_keys(k)
    with bh.BarnesHutSystem(n, mode="plain", eps2=1e-4, timestep=0.0, use_graph=graph) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(1)
        s.sync()
        assert s.stats()["status"] == 0
        assert np.array_equal(s.debug("perm"), operm.astype(np.int32))
        assert np.array_equal(s.debug("keys"), k[operm])
        assert s.check() == 0
        # a second step: with timestep 0 the bodies stay put, now in key order,
        # so the sort of the sorted keys is the identity and the caller index
        # of every position ("perm", composed over the steps) is unchanged
        s.step(1)
        s.sync()
        assert np.array_equal(s.debug("perm"), operm.astype(np.int32))
        assert np.array_equal(s.debug("keys"), k[operm])
        assert s.check() == 0


@pytest.mark.parametrize("graph", [False, True])
def test_full_sort_then_hybrid_again(bh, oracle, graph):
    """A packed run in one step, none in the next: the flag and the
    conditional node are reset by every step."""
    n = 4096
    x1, y1, vx, vy, m = clustered(n, 600, 5)
    x2, y2, _, _, _ = clustered(n, 0, 6)
    with bh.BarnesHutSystem(n, mode="mixed", eps2=1e-4, timestep=0.0, use_graph=graph) as s:
        for x, y in ((x1, y1), (x2, y2), (x1, y1)):
            s.set_state(x, y, vx, vy, m)
            s.step(1)
            s.sync()
            box = oracle.bbox(x, y)
            operm, _ = oracle.sort_keys(oracle.keys(x, y, box))
            assert np.array_equal(s.debug("perm"), operm.astype(np.int32))
            assert s.check() == 0


@pytest.mark.parametrize("graph", [False, True])
def test_batch_with_a_packed_system_equals_systems_alone(bh, graph):
    """A batch where one system packs 600 bodies into one cell takes the full
    sort for the whole batch; every system still gets exactly the results it
    gets alone."""
    sizes = [3000, 4096, 1500]
    systems = [clustered(sizes[0], 0, 21), clustered(sizes[1], 600, 22), clustered(sizes[2], 0, 23)]
    kw = dict(mode="mixed", theta=0.5, eps2=1e-4, timestep=1e-4, use_graph=graph)
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    with bh.BarnesHutSystem(sizes=sizes, **kw) as b:
        off = b.offsets()
        b.set_state(*cat)
        b.step(3)
        b.sync()
        assert b.stats()["status"] == 0
        got = b.get_state()
    for k, (x, y, vx, vy, m) in enumerate(systems):
        with bh.BarnesHutSystem(len(x), **kw) as s:
            s.set_state(x, y, vx, vy, m)
            s.step(3)
            s.sync()
            ref = s.get_state()
        sl = slice(off[k], off[k + 1])
        for key in ("x", "y", "vx", "vy"):
            assert np.array_equal(got[key][sl].view(np.uint32), ref[key].view(np.uint32)), (k, key)


@pytest.mark.parametrize("graph", [False, True])
def test_four_pass_sort_above_2e21_bodies(bh, oracle, graph):
    """Systems over 2^21 bodies sort the top 32 key bits (4 passes) before the
    fixup; 200 bodies in one 2^-16 cell stay within the fixup's runs."""
    n = (1 << 21) + 1
    x, y, vx, vy, m = clustered(n, 200, 41)
    box = oracle.bbox(x, y)
    k = oracle.keys(x, y, box)
    _, runs = np.unique(k >> np.uint64(32), return_counts=True)
    assert 200 <= runs.max() <= 256
    operm, _ = oracle.sort_keys(k)
    with bh.BarnesHutSystem(n, mode="plain", eps2=1e-4, timestep=0.0, use_graph=graph) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(1)
        s.sync()
        assert s.stats()["status"] == 0
        assert np.array_equal(s.debug("perm"), operm.astype(np.int32))
        assert np.array_equal(s.debug("keys"), k[operm])


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("mode", ["reference", "mixed"])
def test_sort_over_consecutive_steps(bh, oracle, graph, mode):
    """A stepped system enters each sort in the previous step's key order (the
    first step after bh_set_state in the caller's order).  Over eight steps,
    every step's permutation (caller index of each sorted position) and sorted
    keys equal the oracle's stable sort of that step's positions, bit for
    bit."""
    from stellarsolver_gb300 import models

    n = 1 << 17
    x, y, vx, vy, m = models.plummer(n, 0x5EED8000)
    kw = dict(mode=mode, theta=0.5, eps2=1e-4, timestep=1e-4, use_graph=graph)
    if mode == "reference":
        kw["eps2"] = 0.025
    with bh.BarnesHutSystem(n, **kw) as s:
        s.set_state(x, y, vx, vy, m)
        for step in range(8):
            st = s.get_state() if step else dict(x=x, y=y)
            s.step(1)
            s.sync()
            assert s.stats()["status"] == 0
            box = oracle.bbox(st["x"], st["y"])  # from step 1 on: the box the last walk folded
            assert np.array_equal(s.debug("box").view(np.uint32), box.view(np.uint32)), step
            k = oracle.keys(st["x"], st["y"], box)
            ok, _ = oracle.sort_keys(k)
            assert np.array_equal(s.debug("perm"), ok.astype(np.int32)), step
            assert np.array_equal(s.debug("keys"), k[ok]), step
