"""bh_set_state copies vx, vy and mass, and bh_set_accel the accelerations, on
the handle's copy stream, overlapped with the next step's box, keys and sort;
bh_step joins them before the reorder, and every other call before its own
work.

Each case uploads a sequence of different states from pinned host memory and
steps right away (the overlapped path), then compares every result bit for bit
with the same sequence where the stream is synchronised after each upload (the
copies done before the step starts)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def states(n, count):
    from stellarsolver_gb300 import models

    return [models.plummer(n, 900 + k) for k in range(count)]


def accels(bh, seq, mode):
    out = []
    for x, y, vx, vy, m in seq:
        with bh.BarnesHutSystem(len(x), mode=mode, eps2=1e-4, timestep=1e-4) as s:
            s.set_state(x, y, vx, vy, m)
            s.step(1)
            s.sync()
            out.append(s.get_accel())
    return out


def run(bh, torch, seq, acc, mode, graph, steps, synchronise):
    n = len(seq[0][0])
    pin = [torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(7)]
    ptr = [p.data_ptr() for p in pin]
    lib = bh.lib()
    results = []
    with bh.BarnesHutSystem(n, mode=mode, eps2=1e-4, timestep=1e-4, use_graph=graph) as s:
        for k, st in enumerate(seq):
            for p, a in zip(pin, st):
                p.numpy()[:] = a
            s.set_state_ptrs(*ptr[:5])
            if acc is not None:
                pin[5].numpy()[:] = acc[k][0]
                pin[6].numpy()[:] = acc[k][1]
                assert lib.bh_set_accel(s.handle, ptr[5], ptr[6], None) == 0
            if synchronise:
                s.sync()
            s.step(steps)
            out = s.get_state()  # synchronises: the pinned buffers are free again
            out["ax"], out["ay"] = s.get_accel()
            assert s.stats()["status"] == 0
            results.append(out)
    return results


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("mode,with_accel,steps", [
    ("plain", False, 1), ("plain", True, 1), ("mixed", False, 2), ("mixed", True, 1),
    ("reference", False, 1)])
def test_overlapped_uploads_equal_synchronised(bh, graph, mode, with_accel, steps):
    torch = pytest.importorskip("torch")
    seq = states(1 << 18, 3)
    acc = accels(bh, seq, mode) if with_accel else None
    a = run(bh, torch, seq, acc, mode, graph, steps, synchronise=False)
    b = run(bh, torch, seq, acc, mode, graph, steps, synchronise=True)
    for k in range(len(seq)):
        for key in ("x", "y", "vx", "vy", "m", "ax", "ay"):
            assert np.array_equal(a[k][key].view(np.uint32), b[k][key].view(np.uint32)), (k, key)


def test_upload_then_read_back(bh):
    """A read right after the upload (no step) returns the uploaded arrays."""
    torch = pytest.importorskip("torch")
    x, y, vx, vy, m = states(1 << 16, 1)[0]
    pin = [torch.from_numpy(a.copy()).pin_memory() for a in (x, y, vx, vy, m)]
    with bh.BarnesHutSystem(len(x), mode="mixed") as s:
        s.set_state_ptrs(*[p.data_ptr() for p in pin])
        got = s.get_state()
    for key, a in zip(("x", "y", "vx", "vy", "m"), (x, y, vx, vy, m)):
        assert np.array_equal(got[key], a), key


@pytest.mark.parametrize("graph", [False, True])
def test_overlapped_uploads_ensemble(bh, graph):
    """The same for a batch of systems: the batched step after an overlapped
    upload equals the one after a synchronised upload."""
    torch = pytest.importorskip("torch")
    from stellarsolver_gb300 import models

    sizes = [3000, 40000, 1500]
    systems = [models.plummer(n, 950 + k) for k, n in enumerate(sizes)]
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    pin = [torch.from_numpy(a.copy()).pin_memory() for a in cat]
    outs = []
    for synchronise in (False, True):
        with bh.BarnesHutSystem(sizes=sizes, mode="mixed", eps2=1e-4, timestep=1e-4,
                                use_graph=graph) as b:
            for _ in range(2):
                b.set_state_ptrs(*[p.data_ptr() for p in pin])
                if synchronise:
                    b.sync()
                b.step(2)
                outs.append(b.get_state())
                assert b.stats()["status"] == 0
    half = len(outs) // 2
    for a, c in zip(outs[:half], outs[half:]):
        for key in ("x", "y", "vx", "vy"):
            assert np.array_equal(a[key].view(np.uint32), c[key].view(np.uint32)), key
