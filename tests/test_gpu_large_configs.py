"""Parity and accuracy at the two large workloads, plus the FP64 diagnostics
the accuracy reports rest on.

Workloads (models.py, seeded):
- two colliding disks, 2 x 2^21 bodies (radius U[5,80], central masses 1e4,
  centres (+-150, 0), bulk velocities (-+2, +-0.5)), eps = 0.05, dt = 5e-4,
  theta = 0.5;
- a 2D Plummer sphere of 2^24 bodies, eps = 0.005, dt = 1e-4, theta in
  {0.3, 0.5, 0.8}.
At these sizes the sort takes its 4-pass fast path (the key's top 32 bits)
and the run fixup (runs of up to ~86 bodies at 2^24), and leaves reach depth
24-26.  One step in PLAIN and in MIXED mode must give
- the box, the sorted keys and the sort permutation bit-exact against the
  oracle: the reference's float-midpoint quadrant digits (kernels.cu:144-157)
  and its depth-first leaf order (kernels.cu:299-335);
- RMS relative force error <= 1e-3 against the FP64 direct sum on a seeded
  sample of 1024 bodies (the error definition of test_gpu_accuracy.py).

bh_direct_sum_f64, the truth of bench.py's force error, is checked against
the oracle's FP64 direct sum (same float inputs and the same float
softening, FP64 sums in another order: rounding differences only).  The
device energy log of the colliding-disks recipe at 2^16 bodies is checked
over 20 steps against the oracle's exact FP64 O(N^2) energy and momentum.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SAMPLE = 1024


@pytest.fixture(scope="module")
def bh():
    from stellarsolver_gb300 import bh as _bh

    _bh.lib()
    return _bh


def _configs():
    from stellarsolver_gb300 import models

    return {
        "colliding_disks_2^22": dict(gen=lambda: models.colliding_disks(1 << 22, models.SEED_BASE + 2),
                                     eps=0.05, dt=5e-4),
        "plummer2d_2^24": dict(gen=lambda: models.plummer(1 << 24, models.SEED_BASE + 4),
                               eps=0.005, dt=1e-4),
    }


_CACHE = {}


def _data(name, oracle):
    """Inputs, oracle box / sorted keys / permutation, and the FP64 direct sum on
    the sample, once per workload."""
    if name not in _CACHE:
        _CACHE.clear()  # one workload's arrays at a time
        cfg = _configs()[name]
        x, y, vx, vy, m = cfg["gen"]()
        box = oracle.bbox(x, y)
        k = oracle.keys(x, y, box)
        perm, dups = oracle.sort_keys(k)
        assert dups == 0
        n = len(x)
        idx = np.sort(np.random.default_rng(7).choice(n, size=SAMPLE, replace=False))
        eps2 = float(np.float32(cfg["eps"] ** 2))  # the engine holds the softening in float
        rx, ry = oracle.direct_f64(x, y, m, idx, eps2)
        _CACHE[name] = dict(state=(x, y, vx, vy, m), box=box, skeys=k[perm],
                            perm=perm.astype(np.int32), idx=idx, rx=rx, ry=ry, eps2=eps2,
                            dt=cfg["dt"])
    return _CACHE[name]


CASES = [("colliding_disks_2^22", 0.5, "plain"), ("colliding_disks_2^22", 0.5, "mixed")] + [
    ("plummer2d_2^24", th, mode) for th in (0.3, 0.5, 0.8) for mode in ("plain", "mixed")]


@pytest.mark.parametrize("name,theta,mode", CASES)
def test_large_workload_step(bh, oracle, name, theta, mode):
    d = _data(name, oracle)
    x, y, vx, vy, m = d["state"]
    n = len(x)
    with bh.BarnesHutSystem(n, mode=mode, theta=theta, eps2=d["eps2"], timestep=d["dt"],
                            use_graph=True) as s:
        s.set_state(x, y, vx, vy, m)
        s.step(1)
        s.sync()
        st = s.stats()
        box = s.debug("box")
        skeys = s.debug("keys")
        perm = s.debug("perm")
        ax, ay = s.get_accel()
    assert st["status"] == 0
    assert np.array_equal(box.view(np.uint32), d["box"].view(np.uint32))
    assert np.array_equal(skeys, d["skeys"])
    assert np.array_equal(perm, d["perm"])
    idx = d["idx"]
    rel = np.hypot(ax[idx] - d["rx"], ay[idx] - d["ry"]) / np.hypot(d["rx"], d["ry"])
    rms = float(np.sqrt(np.mean(rel ** 2)))
    assert rms <= 1e-3, (name, theta, mode, rms, float(rel.max()))


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_direct_sum_f64_matches_oracle(bh, oracle, mode):
    """2D Plummer 2^20 (eps 0.01), 4096 sampled targets.  In MIXED mode after
    three steps, so that the positions' lo words are not zero and the sum
    takes hi + lo."""
    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.plummer(1 << 20, models.SEED_BASE + 1)
    n = len(x)
    eps2 = float(np.float32(1e-4))  # the engine holds the softening in float
    idx = np.sort(np.random.default_rng(11).choice(n, size=4096, replace=False)).astype(np.int32)
    with bh.BarnesHutSystem(n, mode=mode, theta=0.5, eps2=eps2, timestep=1e-4) as s:
        s.set_state(x, y, vx, vy, m)
        if mode == "mixed":
            s.step(3)
            s.sync()
        gx, gy = s.direct_sum_f64(idx)
        st = s.get_state()
        if mode == "mixed":
            xh, xl, yh, yl = s.get_positions_hilo()
    if mode == "mixed":
        assert np.any(xl != 0.0) and np.any(yl != 0.0)
        rx, ry = oracle.direct_f64(xh, yh, st["m"], idx, eps2, xlo=xl, ylo=yl)
    else:
        rx, ry = oracle.direct_f64(st["x"], st["y"], st["m"], idx, eps2)
    rel = np.hypot(gx - rx, gy - ry) / np.hypot(rx, ry)
    assert float(np.sqrt(np.mean(rel ** 2))) <= 1e-12, float(np.sqrt(np.mean(rel ** 2)))
    assert float(rel.max()) <= 1e-10, float(rel.max())


def test_colliding_disks_energy_log_matches_fp64(bh, oracle):
    """The colliding-disks recipe at 2^16 bodies, MIXED, diagnostics logged on
    the device every 10 steps for 20 steps (graph replay).  Each record against
    the oracle's exact FP64 sums at the same state: kinetic energy and momentum
    to 1e-12 (the same float inputs summed in FP64), potential energy to 1e-3
    (tree walk with quadrupole cells and the geometric rule)."""
    from stellarsolver_gb300 import models

    x, y, vx, vy, m = models.colliding_disks(1 << 16, models.SEED_BASE + 2)
    n = len(x)
    eps2 = float(np.float32(0.05 ** 2))  # the engine holds the softening in float
    states = []
    with bh.BarnesHutSystem(n, mode="mixed", theta=0.5, eps2=eps2, timestep=5e-4,
                            use_graph=True) as s:
        s.set_state(x, y, vx, vy, m)
        s.set_energy_log(10, capacity=2)
        for _ in range(2):
            s.step(10)
            s.sync()
            states.append(s.get_state())
        count, log = s.energy_log()
    assert count == 2 and log.shape == (2, 1, 4)
    for rec, st in zip(log[:, 0, :], states):
        ke, pe, px, py = oracle.energy_f64(st["x"], st["y"], st["vx"], st["vy"], st["m"], eps2)
        pscale = float(np.sum(st["m"].astype(np.float64) * np.hypot(st["vx"], st["vy"])))
        assert abs(rec[0] - ke) <= 1e-12 * abs(ke), (rec[0], ke)
        assert abs(rec[2] - px) <= 1e-12 * pscale and abs(rec[3] - py) <= 1e-12 * pscale
        assert abs(rec[1] - pe) <= 1e-3 * abs(pe), (rec[1], pe)
