"""The C-ABI library loads and exports every function include/*.h declares.

CPU only: no compute call is made (this host may have no GPU)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h")) +
                    glob.glob(os.path.join(ROOT, "include", "*.cuh"))):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        # every function declared at file scope: "<type> [*]name(" at a line start
        for m in re.finditer(r"^(?:const\s+)?(?:void|int|char|float|double)\s*\**\s*([A-Za-z_]\w*)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from stellarsolver_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("bh_create", "bh_destroy", "bh_set_state", "bh_get_state", "bh_step",
                     "bh_sync", "bh_get_accel", "bh_default_params", "ResetArrays",
                     "ComputeBoundingBox", "BuildQuadTree", "ComputeCentreOfMass",
                     "SortParticles", "CalculateForces", "IntegrateParticles", "FillOutputArray",
                     "SetDrawArray"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_pure_host_entry_points(lib):
    lib.bh_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.bh_version()
    lib.bh_status_string.restype = ctypes.c_char_p
    assert lib.bh_status_string(0) == b"ok"
    from stellarsolver_gb300 import bh

    p = bh.make_params()
    assert p.mode == 0 and abs(p.theta - 0.5) < 1e-7 and abs(p.eps2 - 0.025) < 1e-9
    assert lib.bh_destroy(None) == 1  # BH_ERR_ARG, no device touched
