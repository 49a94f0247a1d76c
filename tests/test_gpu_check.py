"""bh_check: the tree invariants of debug.cpp:23-174, run on the device, hold
after real steps in every mode and for an ensemble, and agree with the
oracle's restatement of the checker on the same (downloaded) tree.  The
checker's response to broken trees is tested on the oracle
(tests/test_oracle_check.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


@pytest.mark.parametrize("mode", ["reference", "plain", "mixed"])
def test_check_after_steps(bh, oracle, mode):
    from types import SimpleNamespace

    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.plummer(1 << 16, 0x5EED5000)
    m = m * np.linspace(0.5, 1.5, len(m), dtype=np.float32)
    with bh.BarnesHutSystem(len(x), mode=mode, eps2=1e-4, timestep=1e-4) as s:
        s.set_state(x, y, vx, vy, m)
        with pytest.raises(RuntimeError):
            s.check()  # no tree before the first step
        s.step(2)
        assert s.check() == 0
        n = len(x)
        arr = {k: s.debug(k) for k in ("node_left", "node_right", "node_parent", "node_first",
                                       "node_last", "keys", "perm", "box", "node_m")}
    left, right = arr["node_left"][: n - 1], arr["node_right"][: n - 1]
    leaf_parent = np.full(n, -1, np.int32)
    for side in (left, right):
        body = side < 0
        leaf_parent[~side[body]] = np.flatnonzero(body)
    t = SimpleNamespace(left=left, right=right, parent=arr["node_parent"][: n - 1],
                        leaf_parent=leaf_parent, first=arr["node_first"][: n - 1],
                        last=arr["node_last"][: n - 1])
    perm = arr["perm"]
    assert oracle.check_tree(arr["keys"], t, m[perm], arr["node_m"][: n - 1], perm,
                             arr["box"]) == 0


def test_check_ensemble(bh):
    from stellarsolver_gb300 import models

    sizes = [1, 2, 33, 1000, 4096, 3]
    systems = [models.plummer(k, 0x5EED5100 + i) if k > 1 else
               tuple(np.ones(1, np.float32) for _ in range(5)) for i, k in enumerate(sizes)]
    cat = [np.concatenate([sy[k] for sy in systems]) for k in range(5)]
    with bh.BarnesHutSystem(sizes=sizes, mode="mixed", eps2=1e-4, timestep=1e-4,
                            use_graph=True) as s:
        s.set_state(*cat)
        s.step(3)
        assert s.check() == 0
