// Command line with the reference's flags (pentilm/StellarSolver main.cpp:6-103,
// README.md:47-55): -disk | -plummer | -colliding-disks, -opengl, -benchmark,
// -debug, -fullscreen, -iterations=<n>, -timestep=<f>, -gravity=<f>,
// -dampening=<f>.  Additions: -n=<bodies> (the reference hard-codes 512*256),
// -mode=reference|plain|mixed, -theta=<f>, -eps2=<f>, -graph, -image=<file.ppm>.
// Headless: the reference's OpenGL viewer needs a graphics stack; -opengl
// still fills the host output buffer every step, and -image writes the final
// frame (the viewer's view, rendered by bh_render) to a PPM file.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "BarnesHutParticleSystem.h"
#include "SimulationParameters.h"

namespace {

bool flag(int argc, char** argv, const char* name) {
    for (int i = 1; i < argc; ++i)
        if (argv[i][0] == '-' && std::strcmp(argv[i] + 1, name) == 0) return true;
    return false;
}

const char* value(int argc, char** argv, const char* name) {
    size_t len = std::strlen(name);
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (a[0] == '-' && std::strncmp(a + 1, name, len) == 0 && a[1 + len] == '=')
            return a + 2 + len;
    }
    return nullptr;
}

int int_param(int argc, char** argv, const char* name, int def) {
    const char* v = value(argc, argv, name);
    return v ? std::atoi(v) : def;
}

float float_param(int argc, char** argv, const char* name, float def) {
    const char* v = value(argc, argv, name);
    return v ? (float)std::atof(v) : def;
}

void device_banner() {
    int dev = 0;
    cudaDeviceProp p;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        std::cout << "no CUDA device" << std::endl;
        return;
    }
    std::cout << "**************************************************************************\n"
              << "Device " << dev << ": " << p.name << "  sm_" << p.major << p.minor << "  "
              << p.multiProcessorCount << " SMs  " << (p.totalGlobalMem >> 20) << " MiB\n"
              << "Engine: " << bh_version() << "\n"
              << "**************************************************************************"
              << std::endl;
}

}  // namespace

int main(int argc, char** argv) {
    SimulationParameters parameters;
    if (flag(argc, argv, "plummer"))
        parameters.model = plummer_model;
    else if (flag(argc, argv, "colliding-disks"))
        parameters.model = colliding_disk_model;
    else
        parameters.model = disk_model;
    parameters.opengl = flag(argc, argv, "opengl");
    parameters.debug = flag(argc, argv, "debug");
    parameters.benchmark = flag(argc, argv, "benchmark");
    parameters.fullscreen = flag(argc, argv, "fullscreen");
    parameters.iterations = int_param(argc, argv, "iterations", 50);
    parameters.timestep = float_param(argc, argv, "timestep", 0.001f);
    parameters.gravity = float_param(argc, argv, "gravity", 1.0f);
    parameters.dampening = float_param(argc, argv, "dampening", 1.0f);
    const int n = int_param(argc, argv, "n", 512 * 256);

    device_banner();
    if (parameters.opengl)
        std::cout << "-opengl: no graphics stack here; running headless, output buffer filled"
                  << std::endl;
    BarnesHutParticleSystem particles(parameters, n);
    bh_params e = particles.getEngineParams();
    if (const char* m = value(argc, argv, "mode")) {
        if (!std::strcmp(m, "plain")) e.mode = BH_MODE_PLAIN;
        else if (!std::strcmp(m, "mixed")) e.mode = BH_MODE_MIXED;
        else e.mode = BH_MODE_REFERENCE;
    }
    e.theta = float_param(argc, argv, "theta", e.theta);
    e.eps2 = float_param(argc, argv, "eps2", e.eps2);
    e.use_graph = flag(argc, argv, "graph") ? 1 : 0;
    particles.setEngineParams(e);
    particles.reset();
    for (int i = 0; i < parameters.iterations; i++) particles.update();
    const float* out = particles.getOutputBuffer();
    if (parameters.opengl && n > 0)
        std::printf("body 0 at (%g, %g)\n", out[0], out[1]);
    if (const char* img = value(argc, argv, "image")) {
        if (!particles.writeImage(img)) {
            std::fprintf(stderr, "cannot write %s\n", img);
            return 1;
        }
        std::printf("image written to %s\n", img);
    }
    return 0;
}
