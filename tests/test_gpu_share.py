"""Shared walk groups.  The heavy groups (and, on request, the last groups
handed out) are walked by one warp while warps between groups evaluate their
interactions in slices; the owner adds the slices' batch sums in its own
order.  Results must not depend on the sharing at all: every state, every
acceleration and the interaction count are bit for bit the same with sharing
off, with the default sharing (on: 2^16 bodies are fewer walk groups than the
GPU's resident warps) and with every group shared.  Sharing every
group also runs the batch pool out, so that groups are walked again unshared
(the counter of reserved batches passes the pool's size).  Both accuracy
modes, one and two bodies per lane, graph replays and stream order, with and
without softening, single systems and a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALL = 1 << 30  # share_tail beyond the group count: every group shared


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def run(bh, arrays, steps, sizes=None, **kw):
    x = arrays[0]
    args = dict(sizes=sizes) if sizes else dict(n=len(x))
    with bh.BarnesHutSystem(**args, **kw) as s:
        s.set_state(*arrays)
        s.step(steps)
        s.sync()
        stats = s.stats()
        ax, ay = s.get_accel()
        return dict(s.get_state(), ax=ax, ay=ay), stats, s.debug("share")


def assert_same(a, b):
    for k in ("x", "y", "vx", "vy", "ax", "ay"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("bpl", [1, 2])
@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_results_do_not_depend_on_sharing(bh, mode, bpl, graph):
    from stellarsolver_gb300 import models

    n = 1 << 16
    arrays = models.plummer(n, 0x5EED5A1E)
    kw = dict(mode=mode, theta=0.5, eps2=1e-4, timestep=1e-4, bodies_per_lane=bpl,
              use_graph=graph)
    ref, rst, rsh = run(bh, arrays, 4, share_tail=-1, **kw)
    assert rst["status"] == 0
    assert rsh[1] == 0  # nothing shared
    for tail in (0, ALL):
        got, gst, gsh = run(bh, arrays, 4, share_tail=tail, **kw)
        assert gst["status"] == 0, tail
        assert gsh[1] > 0, tail  # slices were published
        assert gst["interactions"] == rst["interactions"], tail
        assert gst["cell_interactions"] == rst["cell_interactions"], tail
        assert_same(got, ref)
        if tail == ALL:
            # the pool (n / 4 batches of sums for one body per lane) ran out
            assert gsh[2] > n // 4 // bpl


def test_unsoftened_bodies(bh):
    """eps2 = 0: body-body terms take the guarded scalar path."""
    from stellarsolver_gb300 import models

    arrays = models.plummer(1 << 13, 0x5EED5A1F)
    kw = dict(mode="plain", theta=0.5, eps2=0.0, timestep=1e-5)
    ref, rst, _ = run(bh, arrays, 2, share_tail=-1, **kw)
    got, gst, gsh = run(bh, arrays, 2, share_tail=ALL, **kw)
    assert rst["status"] == 0 and gst["status"] == 0
    assert gsh[1] > 0
    assert_same(got, ref)


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_batch_of_ragged_systems(bh, mode):
    """Groups at the end of a system have lanes past its last body."""
    from stellarsolver_gb300 import models

    sizes = [5000, 1, 33, 20000, 777]
    systems = models.ensemble(sizes)
    arrays = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    kw = dict(mode=mode, theta=0.5, eps2=1e-3, timestep=1e-3, use_graph=True)
    ref, rst, _ = run(bh, arrays, 3, sizes=sizes, share_tail=-1, **kw)
    got, gst, gsh = run(bh, arrays, 3, sizes=sizes, share_tail=ALL, **kw)
    assert rst["status"] == 0 and gst["status"] == 0
    assert gsh[1] > 0
    assert_same(got, ref)
