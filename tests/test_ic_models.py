"""The reference's initial conditions (-disk, -plummer, -colliding-disks),
bit for bit.

bh_initial_conditions (library) against the reference's own private model
functions (BarnesHutParticleSystem.cpp:390-560), compiled from the reference
sources into a small host program (no GPU needed: the models are host code).
CPU only; skipped where the reference sources are not present."""
import os
import subprocess

import numpy as np
import pytest

REF = "/root/reference"
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r'''
#include <cstdio>
#include <cstdlib>
#include <new>
#define private public
#include "BarnesHutParticleSystem.h"
#undef private
int main(int argc, char** argv) {
    int model = atoi(argv[1]), n = atoi(argv[2]);
    float g = (float)atof(argv[3]);
    // the model functions read only `parameters`; no device memory is touched
    void* raw = ::operator new(sizeof(BarnesHutParticleSystem));
    BarnesHutParticleSystem* s = static_cast<BarnesHutParticleSystem*>(raw);
    s->parameters.gravity = g;
    float *m = new float[n], *x = new float[n], *y = new float[n], *vx = new float[n],
          *vy = new float[n], *ax = new float[n], *ay = new float[n];
    if (model == 0) s->diskModel(m, x, y, vx, vy, ax, ay, n);
    else if (model == 1) s->collidingDiskModel(m, x, y, vx, vy, ax, ay, n);
    else s->plummerModel(m, x, y, vx, vy, ax, ay, n);
    FILE* f = fopen(argv[4], "wb");
    float* arrs[5] = {m, x, y, vx, vy};
    for (float* a : arrs) fwrite(a, sizeof(float), n, f);
    fclose(f);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not os.path.isfile(os.path.join(REF, "BarnesHutParticleSystem.cpp")):
        pytest.skip("reference sources not present")
    from stellarsolver_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    d = tmp_path_factory.mktemp("ic")
    (d / "h.cpp").write_text(HARNESS)
    nvcc = build.nvcc()
    inc = ["-I" + REF]
    for src, obj in ((os.path.join(REF, "BarnesHutParticleSystem.cpp"), d / "b.o"),
                     (os.path.join(REF, "debug.cpp"), d / "d.o"), (str(d / "h.cpp"), d / "h.o")):
        subprocess.run([nvcc, "-std=c++11", "-x", "cu", "-w"] + inc + ["-c", src, "-o", str(obj)],
                       check=True, capture_output=True)
    exe = d / "ic"
    subprocess.run([nvcc, "-o", str(exe), str(d / "b.o"), str(d / "d.o"), str(d / "h.o"),
                    "-L" + build.LIB_DIR, "-lstellar_bh", "-Xlinker", "-rpath=" + build.LIB_DIR],
                   check=True, capture_output=True)
    return exe, d


@pytest.mark.parametrize("model,name,n,g", [(0, "disk", 4096, 1.0), (0, "disk", 1000, 2.5),
                                            (1, "colliding-disks", 4096, 1.0),
                                            (2, "plummer", 4096, 1.0)])
def test_initial_conditions_bit_exact(harness, model, name, n, g):
    from stellarsolver_gb300 import bh

    exe, d = harness
    out = d / f"{name}_{n}.bin"
    subprocess.run([str(exe), str(model), str(n), str(g), str(out)], check=True)
    ref = np.fromfile(out, np.float32).reshape(5, n)  # m, x, y, vx, vy
    x, y, vx, vy, m = bh.reference_initial_conditions(name, n, g)
    for a, b, k in ((m, ref[0], "m"), (x, ref[1], "x"), (y, ref[2], "y"), (vx, ref[3], "vx"),
                    (vy, ref[4], "vy")):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k
