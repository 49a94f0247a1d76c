"""The reference's update() sequence through the C++-linkage drop-in exports,
on the GPU.

The reference's host class binds the nine wrappers with C++ linkage
(Particle_cuda.cuh:5-13).  A small C++ program of this test (not the
reference's code: its sources are not available where this runs) declares
them the same way, allocates the reference's device arrays of length
m = 2n + 12000 (BarnesHutParticleSystem.cpp:54-83), uploads a state as reset()
does (:364-371), and steps three times calling exactly what update() calls,
in its order (:308-315): ResetArrays, ComputeBoundingBox, BuildQuadTree,
ComputeCentreOfMass, SortParticles, CalculateForces, IntegrateParticles,
FillOutputArray.  The outputs are compared with the golden fixtures made by
the reference's own kernels: sorted[] bit-exact, forces and trajectories
within the tolerances of test_oracle_golden.py; the output buffer holds the
positions; bh_compat_status() reports no error.
"""
import os
import subprocess

import numpy as np
import pytest

import golden_cases as gc
from test_oracle_golden import FORCE_TOL, TRAJ_TOL

pytestmark = pytest.mark.gpu

HARNESS = r'''
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <vector>

// the nine wrappers, C++ linkage, as the reference's host code declares them
void SetDrawArray(float* ptr, float* x, float* y, int n);
void ResetArrays(int* mutex, float* x, float* y, float* mass, int* count, int* start, int* sorted,
                 int* child, int* index, float* left, float* right, float* bottom, float* top, int n,
                 int m);
void ComputeBoundingBox(int* mutex, float* x, float* y, float* left, float* right, float* bottom,
                        float* top, int n);
void BuildQuadTree(float* x, float* y, float* mass, int* count, int* start, int* child, int* index,
                   float* left, float* right, float* bottom, float* top, int n, int m);
void ComputeCentreOfMass(float* x, float* y, float* mass, int* index, int n);
void SortParticles(int* count, int* start, int* sorted, int* child, int* index, int n);
void CalculateForces(float* x, float* y, float* vx, float* vy, float* ax, float* ay, float* mass,
                     int* sorted, int* child, float* left, float* right, int n, float g);
void IntegrateParticles(float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n,
                        float dt, float d);
void FillOutputArray(float* x, float* y, float* out, int n);
extern "C" int bh_compat_status(void);
extern "C" void bh_compat_set_constants(float theta, float eps2);

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { \
    fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e)); return 2; } } while (0)

int main(int argc, char** argv) {
    // in: n, steps, dt, d, eps2, then x, y, vx, vy, mass (n floats each)
    FILE* f = fopen(argv[1], "rb");
    int n = 0, steps = 0;
    float dt = 0, d = 0, eps2 = 0;
    if (fread(&n, 4, 1, f) != 1 || fread(&steps, 4, 1, f) != 1 || fread(&dt, 4, 1, f) != 1 ||
        fread(&d, 4, 1, f) != 1 || fread(&eps2, 4, 1, f) != 1) return 3;
    std::vector<float> h(5 * (size_t)n);
    if (fread(h.data(), 4, h.size(), f) != h.size()) return 3;
    fclose(f);
    const int m = 2 * n + 12000;  // BarnesHutParticleSystem.cpp:33
    float *x, *y, *vx, *vy, *ax, *ay, *mass, *left, *right, *bottom, *top, *out;
    int *count, *start, *sorted, *child, *index, *mutex;
    float** fl[] = {&x, &y, &vx, &vy, &ax, &ay, &mass};
    for (float** p : fl) { CK(cudaMalloc(p, sizeof(float) * m)); CK(cudaMemset(*p, 0, sizeof(float) * m)); }
    float** bx[] = {&left, &right, &bottom, &top};
    for (float** p : bx) CK(cudaMalloc(p, sizeof(float)));
    CK(cudaMalloc(&out, 2 * sizeof(float) * m));
    int** in[] = {&count, &start, &sorted, &index, &mutex};
    for (int** p : in) CK(cudaMalloc(p, sizeof(int) * m));
    CK(cudaMalloc(&child, 4 * sizeof(int) * m));
    float* dst[] = {x, y, vx, vy, mass};
    for (int k = 0; k < 5; ++k)  // reset(): the state to the device
        CK(cudaMemcpy(dst[k], h.data() + (size_t)k * n, sizeof(float) * n, cudaMemcpyHostToDevice));
    bh_compat_set_constants(0.5f, eps2);
    FILE* o = fopen(argv[2], "wb");
    std::vector<float> bf((size_t)n), ob(2 * (size_t)n);
    std::vector<int> bi((size_t)n);
    for (int s = 0; s < steps; ++s) {
        // update(), BarnesHutParticleSystem.cpp:308-315
        ResetArrays(mutex, x, y, mass, count, start, sorted, child, index, left, right, bottom, top, n, m);
        ComputeBoundingBox(mutex, x, y, left, right, bottom, top, n);
        BuildQuadTree(x, y, mass, count, start, child, index, left, right, bottom, top, n, m);
        ComputeCentreOfMass(x, y, mass, index, n);
        SortParticles(count, start, sorted, child, index, n);
        CalculateForces(x, y, vx, vy, ax, ay, mass, sorted, child, left, right, n, 1.0f);
        IntegrateParticles(x, y, vx, vy, ax, ay, n, dt, d);
        FillOutputArray(x, y, out, m);
        CK(cudaDeviceSynchronize());
        // per step: sorted, ax, ay, x, y, vx, vy, then the first 2n output floats
        CK(cudaMemcpy(bi.data(), sorted, sizeof(int) * n, cudaMemcpyDeviceToHost));
        fwrite(bi.data(), 4, n, o);
        float* srcs[] = {ax, ay, x, y, vx, vy};
        for (float* p : srcs) {
            CK(cudaMemcpy(bf.data(), p, sizeof(float) * n, cudaMemcpyDeviceToHost));
            fwrite(bf.data(), 4, n, o);
        }
        CK(cudaMemcpy(ob.data(), out, 2 * sizeof(float) * n, cudaMemcpyDeviceToHost));
        fwrite(ob.data(), 4, 2 * n, o);
    }
    fclose(o);
    return bh_compat_status();
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from stellarsolver_gb300 import build

    assert os.path.exists(build.LIB), "libstellar_bh.so not built"
    d = tmp_path_factory.mktemp("cxx")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    r = subprocess.run([build.nvcc(), "-std=c++17", "-O2", "-x", "cu", str(src), "-o", str(exe),
                        "-L" + build.LIB_DIR, "-lstellar_bh", "-Xlinker", "-rpath=" + build.LIB_DIR],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


@pytest.mark.parametrize("name", gc.CASES)
def test_update_sequence_through_cxx_linkage(harness, name):
    exe, d = harness
    g = gc.load(name)
    n, steps = int(g["n"]), int(g["steps"])
    inp = d / f"{name}.in"
    with open(inp, "wb") as f:
        np.array([n, steps], np.int32).tofile(f)
        np.array([g["dt"], g["damp"], g["eps2"]], np.float32).tofile(f)
        for k in ("x", "y", "vx", "vy", "m"):
            g[k].astype(np.float32).tofile(f)
    outp = d / f"{name}.out"
    r = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True, timeout=120,
                       stdin=subprocess.DEVNULL)
    assert r.returncode == 0, (r.returncode, r.stderr)  # bh_compat_status() == BH_OK
    raw = np.fromfile(outp, np.uint8)
    per = 4 * n * 9
    assert raw.size == steps * per
    recs = []
    for s in range(steps):
        b = raw[s * per:(s + 1) * per]
        recs.append({"sorted": b[:4 * n].view(np.int32),
                     **{k: b[4 * n * (1 + i):4 * n * (2 + i)].view(np.float32)
                        for i, k in enumerate(("ax", "ay", "x", "y", "vx", "vy"))},
                     "out": b[4 * n * 7:].view(np.float32)})
    first, last = recs[0], recs[-1]
    assert np.array_equal(first["sorted"], g["sorted"])
    rms = np.sqrt(np.mean(g["ax"].astype(np.float64) ** 2 + g["ay"].astype(np.float64) ** 2))
    err = np.hypot(first["ax"] - g["ax"], first["ay"] - g["ay"]).max() / rms
    assert err <= FORCE_TOL[name], err
    tol = TRAJ_TOL[name]
    for k, ref in (("x", "x1"), ("y", "y1"), ("vx", "vx1"), ("vy", "vy1")):
        assert np.max(np.abs(first[k] - g[ref])) <= tol * np.abs(g[ref]).max(), ref
    for k, ref in (("x", "x3"), ("y", "y3"), ("vx", "vx3"), ("vy", "vy3")):
        assert np.max(np.abs(last[k] - g[ref])) <= 3 * tol * np.abs(g[ref]).max(), ref
    for r_ in recs:  # FillOutputArray: interleaved positions
        assert np.array_equal(r_["out"][0::2], r_["x"]) and np.array_equal(r_["out"][1::2], r_["y"])
