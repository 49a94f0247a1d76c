"""ctypes binding of the C ABI in include/stellar_bh.h.

`BarnesHutSystem` mirrors the reference's host class
(BarnesHutParticleSystem.h:62-71): construct for n bodies, load a state
(reset()), advance (update()), read positions back (getOutputBuffer()).
Arrays are numpy float32 in the caller's body order.  All compute runs on the
GPU through the library; a missing library or a failing call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

MODES = {"reference": 0, "plain": 1, "mixed": 2}
CHECK_BITS = {"count": 1, "child_sum": 2, "child_range": 4, "parent": 8, "keys_sorted": 16,
              "permutation": 32, "box": 64, "mass": 128}
PHASES = ("bbox", "keys", "sort", "reorder", "build", "moments", "bootstrap", "frontier",
          "walk")
PHASES_N = len(PHASES)

BH_OK = 0
STATUS_NAMES = {
    0: "BH_OK", 1: "BH_ERR_ARG", 2: "BH_ERR_DUPLICATE_KEYS", 3: "BH_ERR_NONFINITE",
    4: "BH_ERR_CAPACITY", 5: "BH_ERR_STACK", 6: "BH_ERR_CUDA", 7: "BH_ERR_NOMEM",
    8: "BH_ERR_STATE", 9: "BH_ERR_NO_DEVICE", 10: "BH_ERR_TREE",
}


class BHError(RuntimeError):
    def __init__(self, code: int, what: str):
        self.code = code
        super().__init__(f"{what}: {STATUS_NAMES.get(code, code)} ({_status_string(code)})"
                         + (f" [{last_error()}]" if code == 6 else ""))


class Params(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("theta", ctypes.c_float), ("eps2", ctypes.c_float),
                ("gravity", ctypes.c_float), ("timestep", ctypes.c_float),
                ("dampening", ctypes.c_float), ("leaf_bucket", ctypes.c_int),
                ("block_size", ctypes.c_int), ("stack_depth", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("alpha", ctypes.c_float),
                ("bodies_per_lane", ctypes.c_int), ("share_tail", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("interactions", ctypes.c_int64), ("cells", ctypes.c_int32),
                ("nodes", ctypes.c_int32), ("max_depth", ctypes.c_int32),
                ("status", ctypes.c_int32), ("box", ctypes.c_float * 4),
                ("max_stack", ctypes.c_int32), ("walk_rounds", ctypes.c_int32),
                ("nodes_tested", ctypes.c_int32), ("cell_interactions", ctypes.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB


def lib() -> ctypes.CDLL:
    """Load lib/libstellar_bh.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    vp, i32, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    P = ctypes.POINTER
    L.bh_default_params.argtypes = [P(Params)]
    L.bh_default_params.restype = None
    L.bh_create.argtypes = [P(Params), i32, i32, P(vp)]
    L.bh_ensemble_create.argtypes = [P(Params), i32, vp, i32, P(vp)]
    L.bh_num_systems.argtypes = [vp]
    L.bh_system_offset.argtypes = [vp, i32]
    L.bh_destroy.argtypes = [vp]
    L.bh_set_params.argtypes = [vp, P(Params)]
    L.bh_get_params.argtypes = [vp, P(Params)]
    L.bh_num_bodies.argtypes = [vp]
    L.bh_set_state.argtypes = [vp] + [vp] * 5 + [vp]
    L.bh_get_state.argtypes = [vp] + [vp] * 5 + [vp]
    L.bh_set_accel.argtypes = [vp, vp, vp, vp]
    L.bh_get_accel.argtypes = [vp, vp, vp, vp]
    L.bh_get_positions_hilo.argtypes = [vp, vp, vp, vp, vp, vp]
    L.bh_step.argtypes = [vp, i32, vp]
    L.bh_sync.argtypes = [vp, vp]
    L.bh_get_stats.argtypes = [vp, P(Stats), vp]
    L.bh_get_debug.argtypes = [vp, ctypes.c_char_p, vp, sz, vp]
    L.bh_check.argtypes = [vp, vp, P(ctypes.c_uint)]
    L.bh_set_energy_log.argtypes = [vp, i32, i32]
    L.bh_get_energy_log.argtypes = [vp, vp, i32, P(ctypes.c_int), vp]
    f32 = ctypes.c_float
    L.bh_render.argtypes = [vp, i32, i32, f32, f32, f32, f32, vp, vp]
    L.bh_step_profiled.argtypes = [vp, vp, vp]
    L.bh_direct_sum_f64.argtypes = [vp, i32, vp, vp, vp]
    L.bh_measure_fp32_peak.argtypes = [i32, P(ctypes.c_double)]
    L.bh_measure_fp32_peaks.argtypes = [i32, P(ctypes.c_double), P(ctypes.c_double)]
    L.bh_autotune.argtypes = [vp, vp, P(Params)]
    L.bh_energy.argtypes = [vp, vp, vp]
    L.bh_initial_conditions.argtypes = [i32, i32, ctypes.c_float] + [vp] * 5
    L.bh_status_string.argtypes = [i32]
    L.bh_status_string.restype = ctypes.c_char_p
    L.bh_last_error.restype = ctypes.c_char_p
    L.bh_version.restype = ctypes.c_char_p
    _lib = L
    return L


def _status_string(code: int) -> str:
    try:
        return lib().bh_status_string(code).decode()
    except Exception:  # pragma: no cover - only while the library is absent
        return "?"


def last_error() -> str:
    return lib().bh_last_error().decode()


def _check(code: int, what: str):
    if code != BH_OK:
        raise BHError(code, what)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


REFERENCE_MODELS = {"disk": 0, "colliding-disks": 1, "plummer": 2}


def reference_initial_conditions(model: str, n: int, gravity: float = 1.0):
    """The reference's -disk/-plummer/-colliding-disks initial conditions
    (host arrays x, y, vx, vy, m), generated by the library."""
    out = [np.empty(n, np.float32) for _ in range(5)]  # m, x, y, vx, vy
    _check(lib().bh_initial_conditions(REFERENCE_MODELS[model], n, gravity, *[_p(a) for a in out]),
           "bh_initial_conditions")
    m, x, y, vx, vy = out
    return x, y, vx, vy, m


def measure_fp32_peak(device: int = -1) -> float:
    """Measured FP32 FMA throughput of the device in TFLOP/s (the larger of
    the scalar FFMA and packed FFMA2 probes)."""
    v = ctypes.c_double(0.0)
    _check(lib().bh_measure_fp32_peak(device, ctypes.byref(v)), "bh_measure_fp32_peak")
    return float(v.value)


def measure_fp32_peaks(device: int = -1) -> dict:
    """Both FP32 FMA probes in TFLOP/s: scalar FFMA chains and packed FFMA2 chains."""
    a, b = ctypes.c_double(0.0), ctypes.c_double(0.0)
    _check(lib().bh_measure_fp32_peaks(device, ctypes.byref(a), ctypes.byref(b)),
           "bh_measure_fp32_peaks")
    return {"ffma": float(a.value), "ffma2": float(b.value)}


def make_params(mode="reference", theta=0.5, eps2=0.025, gravity=1.0, timestep=1e-3,
                dampening=1.0, leaf_bucket=0, use_graph=False, stack_depth=0,
                block_size=0, alpha=0.01, bodies_per_lane=0, share_tail=0) -> Params:
    p = Params()
    lib().bh_default_params(ctypes.byref(p))
    p.mode = MODES[mode] if isinstance(mode, str) else int(mode)
    p.theta, p.eps2, p.gravity = theta, eps2, gravity
    p.timestep, p.dampening = timestep, dampening
    p.leaf_bucket, p.use_graph = int(leaf_bucket), int(bool(use_graph))
    p.stack_depth, p.block_size = int(stack_depth), int(block_size)
    p.alpha = alpha
    p.bodies_per_lane = int(bodies_per_lane)
    p.share_tail = int(share_tail)
    return p


class BarnesHutSystem:
    """One system of n bodies on one GPU (BarnesHutParticleSystem.cpp:28-84), or,
    with `sizes`, a batch of independent systems stepped together
    (bh_ensemble_create); body arrays then hold the systems back to back."""

    def __init__(self, n: int = 0, device: int = 0, sizes=None, **params):
        self.params = make_params(**params)
        h = ctypes.c_void_p()
        if sizes is None:
            self.n = int(n)
            _check(lib().bh_create(ctypes.byref(self.params), self.n, device, ctypes.byref(h)),
                   "bh_create")
        else:
            sz = np.ascontiguousarray(sizes, dtype=np.int32)
            self.n = int(sz.sum())
            _check(lib().bh_ensemble_create(ctypes.byref(self.params), len(sz), _p(sz), device,
                                            ctypes.byref(h)), "bh_ensemble_create")
        self._h = h

    # lifecycle -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().bh_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def num_systems(self) -> int:
        return int(lib().bh_num_systems(self._h))

    def offsets(self) -> np.ndarray:
        k = self.num_systems
        return np.array([lib().bh_system_offset(self._h, i) for i in range(k + 1)], np.int64)

    # state ----------------------------------------------------------------
    def set_params(self, **params):
        p = make_params(**params)
        _check(lib().bh_set_params(self._h, ctypes.byref(p)), "bh_set_params")
        self.params = p

    def set_state(self, x, y, vx, vy, m, stream=None):
        arrs = [_f32(a) for a in (x, y, vx, vy, m)]
        for a in arrs:
            if a.shape != (self.n,):
                raise ValueError(f"expected arrays of shape ({self.n},), got {a.shape}")
        _check(lib().bh_set_state(self._h, *[_p(a) for a in arrs], stream), "bh_set_state")
        self.sync(stream)

    def set_accel(self, ax, ay, stream=None):
        """Accelerations of the state just set (skips the bootstrap pass)."""
        ax, ay = _f32(ax), _f32(ay)
        _check(lib().bh_set_accel(self._h, _p(ax), _p(ay), stream), "bh_set_accel")
        self.sync(stream)

    def set_state_ptrs(self, x, y, vx, vy, m, stream=None):
        """Raw pointers (host or device), no copy of the arrays on the Python side."""
        _check(lib().bh_set_state(self._h, x, y, vx, vy, m, stream), "bh_set_state")

    def get_state(self, stream=None):
        out = {k: np.empty(self.n, np.float32) for k in ("x", "y", "vx", "vy", "m")}
        _check(lib().bh_get_state(self._h, *[_p(out[k]) for k in ("x", "y", "vx", "vy", "m")],
                                  stream), "bh_get_state")
        self.sync(stream)
        return out

    def get_positions_hilo(self, stream=None):
        out = [np.empty(self.n, np.float32) for _ in range(4)]
        _check(lib().bh_get_positions_hilo(self._h, *[_p(a) for a in out], stream),
               "bh_get_positions_hilo")
        self.sync(stream)
        return out  # xhi, xlo, yhi, ylo

    def get_accel(self, stream=None):
        ax = np.empty(self.n, np.float32)
        ay = np.empty(self.n, np.float32)
        _check(lib().bh_get_accel(self._h, _p(ax), _p(ay), stream), "bh_get_accel")
        self.sync(stream)
        return ax, ay

    # stepping ---------------------------------------------------------------
    def step(self, steps: int = 1, stream=None):
        _check(lib().bh_step(self._h, int(steps), stream), "bh_step")

    def energy(self, stream=None) -> np.ndarray:
        """FP64 (kinetic, potential, px, py) per system, shape (systems, 4)."""
        out = np.zeros(4 * self.num_systems, np.float64)
        _check(lib().bh_energy(self._h, stream, _p(out)), "bh_energy")
        return out.reshape(-1, 4)

    def set_energy_log(self, every: int, capacity: int = 64):
        """Record FP64 energy/momentum on the device after every `every`-th step."""
        _check(lib().bh_set_energy_log(self._h, every, capacity), "bh_set_energy_log")
        self._elog_cap = capacity

    def energy_log(self, stream=None):
        """(records written, array (kept, systems, 4)) of the energy log, oldest first."""
        cap = getattr(self, "_elog_cap", 0)
        out = np.zeros(max(cap, 1) * 4 * self.num_systems, np.float64)
        rec = ctypes.c_int(0)
        _check(lib().bh_get_energy_log(self._h, _p(out), cap, ctypes.byref(rec), stream),
               "bh_get_energy_log")
        kept = min(rec.value, cap)
        return rec.value, out[: kept * 4 * self.num_systems].reshape(kept, self.num_systems, 4)

    def autotune(self, stream=None) -> dict:
        """Pick the walk's block size, leaf bucket and stack depth (bh_autotune)."""
        p = Params()
        _check(lib().bh_autotune(self._h, stream, ctypes.byref(p)), "bh_autotune")
        self.params = p
        return {"block_size": p.block_size, "leaf_bucket": p.leaf_bucket,
                "stack_depth": p.stack_depth, "bodies_per_lane": p.bodies_per_lane}

    def step_profiled(self, phase_ms: np.ndarray, stream=None):
        """One non-graph step with events at the phase boundaries; adds each
        phase's milliseconds to phase_ms (float32[9]: bbox, keys, sort,
        reorder, build, moments with the walk records, bootstrap, frontier,
        walk)."""
        assert phase_ms.dtype == np.float32 and phase_ms.shape == (PHASES_N,)
        _check(lib().bh_step_profiled(self._h, stream, _p(phase_ms)), "bh_step_profiled")

    def direct_sum_f64(self, idx):
        """FP64 direct-sum accelerations (times G) at caller indices idx."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        ax = np.empty(len(idx), np.float64)
        ay = np.empty(len(idx), np.float64)
        _check(lib().bh_direct_sum_f64(self._h, len(idx), _p(idx), _p(ax), _p(ay)),
               "bh_direct_sum_f64")
        return ax, ay

    def sync(self, stream=None):
        _check(lib().bh_sync(self._h, stream), "bh_sync")

    def stats(self, stream=None) -> dict:
        s = Stats()
        _check(lib().bh_get_stats(self._h, ctypes.byref(s), stream), "bh_get_stats")
        return dict(interactions=int(s.interactions), cells=int(s.cells), nodes=int(s.nodes),
                    max_depth=int(s.max_depth), status=int(s.status), box=np.array(s.box[:]),
                    max_stack=int(s.max_stack), walk_rounds=int(s.walk_rounds),
                    nodes_tested=int(s.nodes_tested),
                    cell_interactions=int(s.cell_interactions))

    def render(self, width: int = 1000, height: int = 1000,
               extent=(-25.0, 25.0, -25.0, 25.0), stream=None) -> np.ndarray:
        """The current positions as one-pixel points (bh_render): uint8 array
        (height, width, 4), RGBA, top row first.  The default view is the
        reference viewer's: 1000 x 1000 pixels over [-25, 25]^2."""
        out = np.empty((height, width, 4), np.uint8)
        _check(lib().bh_render(self._h, width, height, *[float(e) for e in extent], _p(out),
                               stream), "bh_render")
        self.sync(stream)
        return out

    def check(self, stream=None) -> int:
        """Tree invariants of the last step checked on the device (bh_check):
        the mask of BH_CHECK_* bits that fail, 0 when all hold."""
        f = ctypes.c_uint(0)
        _check(lib().bh_check(self._h, stream, ctypes.byref(f)), "bh_check")
        return int(f.value)

    def debug(self, name: str):
        n = self.n
        spec = {"box": (np.float32, 4), "boxes": (np.float32, 4 * self.num_systems),
                "keys": (np.uint64, n), "perm": (np.int32, n),
                "accel_sorted": (np.float32, 2 * n), "share": (np.int32, 4)}
        dt, cnt = spec.get(name, (np.float32 if name in ("node_m", "node_mx", "node_my",
                                                          "node_cx", "node_cy") else np.int32, n))
        out = np.empty(cnt, dt)
        _check(lib().bh_get_debug(self._h, name.encode(), _p(out), out.nbytes, None),
               f"bh_get_debug({name})")
        return out
