"""The C++ host surface: stellar_app with the reference's flags, on the GPU.

-benchmark prints one "Timestep: k    Elapsed time: ms" line per step
(BarnesHutParticleSystem.cpp:323-325); -debug prints the debug.cpp test lines,
which must all PASS."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def app():
    from stellarsolver_gb300 import build

    assert os.path.exists(build.APP), "stellar_app not built"
    return build.APP


@pytest.mark.parametrize("model", ["-disk", "-plummer", "-colliding-disks"])
def test_benchmark_lines(model):
    r = subprocess.run([app(), model, "-benchmark", "-iterations=5", "-n=4096"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    steps = re.findall(r"^Timestep: (\d+)\s+Elapsed time: ([0-9.e+-]+)$", r.stdout, re.M)
    assert [int(s) for s, _ in steps] == list(range(5))


@pytest.mark.parametrize("mode", ["reference", "mixed"])
def test_debug_invariants_pass(mode):
    r = subprocess.run([app(), "-plummer", "-debug", "-iterations=2", "-n=8192", f"-mode={mode}",
                        "-eps2=0.0001", "-timestep=0.0001"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    results = re.findall(r"RESULT = (PASS|FAIL)", r.stdout)
    assert len(results) == 16 and set(results) == {"PASS"}, r.stdout


def test_opengl_is_headless_and_fills_the_output_buffer():
    r = subprocess.run([app(), "-disk", "-opengl", "-iterations=2", "-n=2048", "-graph"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "headless" in r.stdout and "body 0 at" in r.stdout


def test_image_flag_writes_the_viewer_frame(tmp_path):
    import numpy as np

    path = tmp_path / "frame.ppm"
    r = subprocess.run([app(), "-disk", "-iterations=3", "-n=20000", f"-image={path}"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    data = path.read_bytes()
    header = b"P6\n1000 1000\n255\n"
    assert data.startswith(header) and len(data) == len(header) + 1000 * 1000 * 3
    rgb = np.frombuffer(data[len(header):], np.uint8).reshape(1000, 1000, 3)
    assert (rgb[..., 0] > 0).sum() > 1000 and np.array_equal(rgb[..., 0], rgb[..., 2])
