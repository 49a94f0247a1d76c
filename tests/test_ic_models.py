"""The reference's initial conditions (-disk, -plummer, -colliding-disks),
bit for bit.

bh_initial_conditions (library) against the reference's own private model
functions (BarnesHutParticleSystem.cpp:390-560):
- always, against the SHA-256 of the reference's arrays committed in
  tests/golden/ic_models.json (made by tests/golden/make_ic_golden.py from the
  reference sources);
- and, when the STELLARSOLVER_REF environment variable names the reference
  sources, against the reference's functions compiled into a small host
  program here (no GPU needed: the models are host code).
CPU only."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
REF = os.environ.get("STELLARSOLVER_REF", "")

with open(os.path.join(GOLDEN, "ic_models.json")) as _f:
    TABLE = json.load(_f)

NAMES = {0: "disk", 1: "colliding-disks", 2: "plummer"}


def _ours(name, n, g):
    from stellarsolver_gb300 import bh

    x, y, vx, vy, m = bh.reference_initial_conditions(name, n, g)
    return m, x, y, vx, vy


@pytest.mark.parametrize("key", sorted(TABLE))
def test_initial_conditions_match_reference_hashes(key):
    import make_ic_golden as mk

    c = TABLE[key]
    arrays = _ours(NAMES[c["model"]], c["n"], c["gravity"])
    assert mk.digest(arrays) == c["sha256_m_x_y_vx_vy"], key


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not REF or not os.path.isfile(os.path.join(REF, "BarnesHutParticleSystem.cpp")):
        pytest.skip("STELLARSOLVER_REF does not name the reference sources")
    import make_ic_golden as mk

    d = tmp_path_factory.mktemp("ic")
    return mk.build_harness(REF, str(d)), str(d)


@pytest.mark.parametrize("model,name,n,g", [(0, "disk", 4096, 1.0), (0, "disk", 1000, 2.5),
                                            (1, "colliding-disks", 4096, 1.0),
                                            (2, "plummer", 4096, 1.0)])
def test_initial_conditions_bit_exact_live(harness, model, name, n, g):
    import make_ic_golden as mk

    exe, d = harness
    ref = mk.run_case(exe, d, model, n, g)  # m, x, y, vx, vy
    for a, b, k in zip(_ours(name, n, g), ref, ("m", "x", "y", "vx", "vy")):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k
