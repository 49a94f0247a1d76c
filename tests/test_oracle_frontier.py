"""The walk's shared frontiers, checked on the CPU restatement.

The engine's main accuracy walk starts each group from its super-group's
frontier (k_frontier, bh_walk.cuh): the nodes every group of the super-group
opens are opened once, and the frontier cells every group accepts go to the
groups untested.  The claim is that a group then accepts exactly the cells,
and interacts exactly the bodies, that it would from the root.  The oracle
restates the frontier and compares every group's two sets."""
import numpy as np
import pytest


def tree_of(oracle, x, y, m):
    box = oracle.bbox(x, y)
    k = oracle.keys(x, y, box)
    perm, _ = oracle.sort_keys(k)
    sk = k[perm]
    return box, sk, oracle.Tree(sk), x[perm], y[perm], m[perm]


@pytest.mark.parametrize("model", ["plummer", "colliding", "disk"])
@pytest.mark.parametrize("group,bucket", [(32, 16), (64, 8)])
def test_frontier_start_gives_the_root_start_sets(oracle, model, group, bucket):
    from stellarsolver_gb300 import models

    n = 1 << 15
    if model == "plummer":
        x, y, vx, vy, m = models.plummer(n, 301)
        eps2 = 1e-4
    elif model == "colliding":
        x, y, vx, vy, m = models.colliding_disks(n, 302)
        eps2 = 0.05 ** 2
    else:
        x, y, vx, vy, m = models.disk(n, 303)
        eps2 = 0.01
    box, sk, t, sx, sy, sm = tree_of(oracle, x, y, m)
    # |a| of the bootstrap pass as the relative rule's scale, as in the engine
    a0x, a0y, _ = oracle.walk_acc(sx, sy, sm, sk, t, box, 1.25, eps2, quadrupole=False, group=64)
    aold = np.hypot(a0x, a0y)
    r = oracle.frontier_check(sx, sy, sm, sk, t, box, 0.5, bucket=bucket, alpha=0.01,
                              aold=aold, group=group)
    assert r["differing_groups"] == 0, r
    assert r["frontier_nodes"] > 0 and r["accepted_cells"] > 0, r
    assert r["tests_from_frontier"] < r["tests_from_root"], r


def test_geometric_rule_only(oracle):
    """Without the relative rule (alpha = 0): frontier cells are accepted on
    the geometric rule alone."""
    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.plummer(1 << 14, 304)
    box, sk, t, sx, sy, sm = tree_of(oracle, x, y, m)
    r = oracle.frontier_check(sx, sy, sm, sk, t, box, 0.5, bucket=8)
    assert r["differing_groups"] == 0, r
