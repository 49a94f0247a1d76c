"""Tree-invariant checker (the engine's bh_check) restated in the oracle, with
planted mistakes.  The checks follow debug.cpp:23-174 of the reference,
stated for a binary radix tree; bits as BH_CHECK_* in include/stellar_bh.h.
Mistakes are planted here, in host copies of an oracle-built tree."""
import numpy as np
import pytest

COUNT, CHILD_SUM, CHILD_RANGE, PARENT, KEYS, PERM, BOX, MASS = (1, 2, 4, 8, 16, 32, 64, 128)


@pytest.fixture(scope="module")
def case(oracle):
    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.plummer(1 << 12, 0x5EED4000)
    m = m * np.linspace(0.5, 1.5, len(m), dtype=np.float32)  # unequal masses
    box = oracle.bbox(x, y)
    k = oracle.keys(x, y, box)
    perm, _ = oracle.sort_keys(k)
    sk = k[perm]
    t = oracle.Tree(sk)
    sm = m[perm]
    node_m = t.sums(x[perm], y[perm], sm)[0]
    return dict(sk=sk, t=t, sm=sm, node_m=node_m, ids=perm.astype(np.int32), box=box)


def run(oracle, c, **over):
    kw = dict(sk=c["sk"], sm=c["sm"], node_m=c["node_m"], ids=c["ids"], box=c["box"])
    tree_over = {k: over.pop(k) for k in list(over) if k in ("left", "right", "parent",
                                                             "leaf_parent", "first", "last")}
    kw.update(over)
    return oracle.check_tree(kw["sk"], c["t"], kw["sm"], kw["node_m"], kw["ids"], kw["box"],
                             **tree_over)


def test_valid_tree_passes(oracle, case):
    assert run(oracle, case) == 0


def test_single_body(oracle):
    from types import SimpleNamespace

    e = np.zeros(0, np.int32)
    t = SimpleNamespace(left=e, right=e, parent=e, leaf_parent=np.full(1, -1, np.int32), first=e,
                        last=e)
    assert oracle.check_tree(np.array([5], np.uint64), t, np.ones(1, np.float32),
                             np.zeros(0, np.float32), np.zeros(1, np.int32),
                             np.array([0, 1, 0, 1], np.float32)) == 0


def test_planted_mistakes(oracle, case):
    t = case["t"]
    # a body child replaced by another body: that body twice, one body never
    left = t.left.copy()
    i = int(np.flatnonzero(left < 0)[0])
    left[i] = ~((~left[i] + 7) % len(case["sk"]))
    f = run(oracle, case, left=left)
    assert f & CHILD_SUM and f & PARENT
    # a child index out of range
    right = t.right.copy()
    right[0] = len(case["sk"]) + 3
    assert run(oracle, case, right=right) & CHILD_RANGE
    # a node range that does not match its children
    last = t.last.copy()
    j = int(np.flatnonzero(t.first != np.arange(len(t.first)))[0])  # a node whose range ends at j
    last[j] = last[j] + 1
    assert run(oracle, case, last=last) & COUNT
    # a wrong parent link
    parent = t.parent.copy()
    c = int(np.flatnonzero(t.left >= 0)[0])
    parent[t.left[c]] = (c + 1) % len(parent)
    assert run(oracle, case, parent=parent) & PARENT
    # keys out of order
    sk = case["sk"].copy()
    sk[[10, 11]] = sk[[11, 10]]
    assert run(oracle, case, sk=sk) & KEYS
    # a caller index twice
    ids = case["ids"].copy()
    ids[5] = ids[6]
    assert run(oracle, case, ids=ids) == PERM
    # an inverted box
    box = np.array(case["box"], np.float32)[[1, 0, 2, 3]]
    assert run(oracle, case, box=box) == BOX
    # a node mass off by one ulp
    node_m = case["node_m"].copy()
    node_m[3] = np.nextafter(node_m[3], np.float32(np.inf))
    assert run(oracle, case, node_m=node_m) & MASS
