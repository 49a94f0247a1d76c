"""Batches of independent systems (bh_ensemble_create) on the GPU.

A batch steps every system with one launch per phase.  Each system's box,
keys, tree and walk only see its own bodies, so a batch must give exactly the
results of stepping each system alone (same float operations in the same
order): bit-exact, in REFERENCE and in MIXED mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def _systems(sizes):
    from stellarsolver_gb300 import models

    return models.ensemble(sizes)


@pytest.mark.parametrize("mode,bpl", [("reference", 0), ("mixed", 1), ("mixed", 2)])
def test_batch_equals_systems_alone(bh, mode, bpl):
    sizes = [1000, 33, 4096, 1, 2, 777, 20000, 64, 65, 95]
    systems = _systems(sizes)
    kw = dict(mode=mode, theta=0.5, eps2=0.01 if mode == "reference" else 1e-3, timestep=1e-3,
              bodies_per_lane=bpl)
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    with bh.BarnesHutSystem(sizes=sizes, **kw) as b:
        assert b.num_systems == len(sizes)
        off = b.offsets()
        assert list(np.diff(off)) == sizes
        b.set_state(*cat)
        b.step(3)
        b.sync()
        got = b.get_state()
        ax, ay = b.get_accel()
    for k, (x, y, vx, vy, m) in enumerate(systems):
        with bh.BarnesHutSystem(len(x), **kw) as s:
            s.set_state(x, y, vx, vy, m)
            s.step(3)
            s.sync()
            ref = s.get_state()
            rax, ray = s.get_accel()
        sl = slice(off[k], off[k + 1])
        for key in ("x", "y", "vx", "vy"):
            assert np.array_equal(got[key][sl].view(np.uint32), ref[key].view(np.uint32)), (k, key)
        assert np.array_equal(ax[sl].view(np.uint32), rax.view(np.uint32)), k


def test_batch_of_256_uneven_systems_runs_as_graph(bh):
    from stellarsolver_gb300 import models

    sizes = models.ensemble_sizes(256, 1 << 8, 1 << 12)
    systems = _systems(sizes)
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    with bh.BarnesHutSystem(sizes=sizes, mode="mixed", eps2=1e-3, timestep=1e-4,
                            use_graph=True) as b:
        b.set_state(*cat)
        b.step(4)
        b.sync()
        st = b.stats()
    assert st["status"] == 0 and st["interactions"] > 0
