"""The bounding box carried from one step to the next.

The walk writes the next step's positions, so it also folds their box
(min / max from the origin, kernels.cu:54-57 and 62-114) into a second box
that the next step takes instead of running the box kernel.  Min and max are
exact: every step's box must equal the oracle's box of that step's positions,
bit for bit, whatever came between the steps (a diagnostics pass, an energy
log, new positions, the autotuner's trial steps), for every system of a batch,
in stream order and as graph replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def _boxes(oracle, st, off):
    return np.concatenate([oracle.bbox(st["x"][a:b], st["y"][a:b])
                           for a, b in zip(off[:-1], off[1:])])


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("mode", ["reference", "mixed"])
def test_every_step_box_in_a_batch(bh, oracle, graph, mode):
    from stellarsolver_gb300 import models

    sizes = [5000, 1, 33, 20000, 777]
    systems = models.ensemble(sizes)
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    kw = dict(mode=mode, theta=0.5, eps2=0.01 if mode == "reference" else 1e-3,
              timestep=1e-3, use_graph=graph)
    with bh.BarnesHutSystem(sizes=sizes, **kw) as s:
        off = s.offsets()
        s.set_state(*cat)
        for step in range(5):
            st = s.get_state() if step else dict(x=cat[0], y=cat[1])
            s.step(1)
            s.sync()
            assert s.stats()["status"] == 0
            want = _boxes(oracle, st, off)
            assert np.array_equal(s.debug("boxes").view(np.uint32), want.view(np.uint32)), step


@pytest.mark.parametrize("graph", [False, True])
def test_box_after_diagnostics_new_state_and_autotune(bh, oracle, graph):
    from stellarsolver_gb300 import models

    n = 1 << 15
    x, y, vx, vy, m = models.plummer(n, 0x5EEDB0C5)
    x2, y2, vx2, vy2, m2 = models.colliding_disks(n, 0x5EEDB0C6)
    kw = dict(mode="mixed", theta=0.5, eps2=1e-4, timestep=1e-3, use_graph=graph)

    def step_and_check(s, prev, diagnosed=False):
        s.step(1)
        s.sync()
        assert s.stats()["status"] == 0
        # an energy-log pass after the step builds the tree of the new
        # positions: the box it leaves is theirs
        at = s.get_state() if diagnosed else prev
        want = oracle.bbox(at["x"], at["y"])
        assert np.array_equal(s.debug("box").view(np.uint32), want.view(np.uint32))

    with bh.BarnesHutSystem(n, **kw) as s:
        s.set_state(x, y, vx, vy, m)
        step_and_check(s, dict(x=x, y=y))
        step_and_check(s, s.get_state())
        s.energy()  # a diagnostics pass between two steps
        step_and_check(s, s.get_state())
        s.set_energy_log(2, 8)  # diagnostics after every second step
        for k in range(1, 5):
            step_and_check(s, s.get_state(), diagnosed=k % 2 == 0)
        s.set_energy_log(0, 0)
        s.set_state(x2, y2, vx2, vy2, m2)  # new positions
        step_and_check(s, dict(x=x2, y=y2))
        step_and_check(s, s.get_state())
        st = s.get_state()
        s.autotune()  # trial steps, then the state put back
        step_and_check(s, st)
        step_and_check(s, s.get_state())
