"""Golden hashes of the reference's initial conditions (-disk, -plummer,
-colliding-disks), for tests/test_ic_models.py.

Compiles the reference's own private model functions
(BarnesHutParticleSystem.cpp:390-560) with a small host harness, runs each
case and stores the SHA-256 of the five float32 arrays (m, x, y, vx, vy, in
that order, native byte order) in ic_models.json.  The reference sources are
read from the directory named by --ref or by the STELLARSOLVER_REF environment
variable; nothing is copied from them.

    STELLARSOLVER_REF=<reference checkout> python tests/golden/make_ic_golden.py
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (model, name, n, gravity): the Model enum of SimulationParameters.h:8-13
CASES = [(0, "disk", 4096, 1.0), (0, "disk", 1000, 2.5), (1, "colliding-disks", 4096, 1.0),
         (2, "plummer", 4096, 1.0), (2, "plummer", 65536, 1.0)]

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


def case_key(name: str, n: int, g: float) -> str:
    return f"{name}_{n}_g{g}"


def digest(arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype=np.float32).tobytes())
    return h.hexdigest()


def build_harness(ref: str, workdir: str) -> str:
    """The reference's model functions linked into a host program (the
    reference's class also references the nine wrappers: this library
    resolves them)."""
    sys.path.insert(0, ROOT)
    from stellarsolver_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    src = os.path.join(workdir, "h.cpp")
    with open(src, "w") as f:
        f.write(HARNESS)
    nvcc = build.nvcc()
    objs = []
    for s, o in ((os.path.join(ref, "BarnesHutParticleSystem.cpp"), "b.o"),
                 (os.path.join(ref, "debug.cpp"), "d.o"), (src, "h.o")):
        obj = os.path.join(workdir, o)
        subprocess.run([nvcc, "-std=c++11", "-x", "cu", "-w", "-I" + ref, "-c", s, "-o", obj],
                       check=True, capture_output=True)
        objs.append(obj)
    exe = os.path.join(workdir, "ic")
    subprocess.run([nvcc, "-o", exe] + objs + ["-L" + build.LIB_DIR, "-lstellar_bh",
                                               "-Xlinker", "-rpath=" + build.LIB_DIR],
                   check=True, capture_output=True)
    return exe


def run_case(exe: str, workdir: str, model: int, n: int, g: float):
    out = os.path.join(workdir, f"ic_{model}_{n}_{g}.bin")
    subprocess.run([exe, str(model), str(n), str(g), out], check=True)
    return np.fromfile(out, np.float32).reshape(5, n)  # m, x, y, vx, vy


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("STELLARSOLVER_REF"))
    args = ap.parse_args()
    if not args.ref or not os.path.isfile(os.path.join(args.ref, "BarnesHutParticleSystem.cpp")):
        sys.exit("give the reference sources with --ref or STELLARSOLVER_REF")
    table = {}
    with tempfile.TemporaryDirectory() as d:
        exe = build_harness(args.ref, d)
        for model, name, n, g in CASES:
            arr = run_case(exe, d, model, n, g)
            table[case_key(name, n, g)] = {"model": model, "n": n, "gravity": g,
                                           "sha256_m_x_y_vx_vy": digest(arr)}
    path = os.path.join(HERE, "ic_models.json")
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")
    print(f"wrote {os.path.relpath(path, ROOT)}: {len(table)} cases")


if __name__ == "__main__":
    main()
