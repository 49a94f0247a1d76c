"""ctypes signatures of the drop-in wrappers (include/Particle_cuda.cuh)."""
import ctypes


def load():
    from stellarsolver_gb300 import bh

    L = bh.lib()
    vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    sig = {
        "SetDrawArray": [vp, vp, vp, i32],
        "ResetArrays": [vp] * 13 + [i32, i32],
        "ComputeBoundingBox": [vp] * 7 + [i32],
        "BuildQuadTree": [vp] * 11 + [i32, i32],
        "ComputeCentreOfMass": [vp] * 4 + [i32],
        "SortParticles": [vp] * 5 + [i32],
        "CalculateForces": [vp] * 11 + [i32, f32],
        "IntegrateParticles": [vp] * 6 + [i32, f32, f32],
        "FillOutputArray": [vp, vp, vp, i32],
        "bh_compat_set_constants": [f32, f32],
        "bh_compat_set_stream": [vp],
        "bh_compat_status": [],
        "bh_compat_clear_status": [],
        "bh_compat_release": [],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int if name == "bh_compat_status" else None
    return L
