// BarnesHutParticleSystem on the engine's C ABI.
//   reset()  generates the reference's initial conditions and uploads them
//            (BarnesHutParticleSystem.cpp:350-372);
//   update() advances one step (:301-347); with `benchmark` it prints
//            "Timestep: <k>    Elapsed time: <ms>" (:323-325); with `opengl`
//            it fills the host output buffer (:327-329); with `debug` it checks
//            the tree invariants of debug.cpp:23-174 on the engine's tree.
#include "BarnesHutParticleSystem.h"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>


namespace {
void check(int st, const char* what) {
    if (st != BH_OK) {
        std::fprintf(stderr, "%s: %s (%s)\n", what, bh_status_string(st), bh_last_error());
        std::exit(1);
    }
}
}  // namespace

BarnesHutParticleSystem::BarnesHutParticleSystem(const SimulationParameters p, const int n)
    : parameters(p), step(0), numParticles(n), numNodes(2 * n + 12000), sys(nullptr) {
    bh_default_params(&engine);
    engine.gravity = p.gravity;
    engine.timestep = p.timestep;
    engine.dampening = p.dampening;
    create();
}

void BarnesHutParticleSystem::create() {
    h_mass.assign(numParticles, 0.f);
    h_x.assign(numParticles, 0.f);
    h_y.assign(numParticles, 0.f);
    h_vx.assign(numParticles, 0.f);
    h_vy.assign(numParticles, 0.f);
    h_ax.assign(numParticles, 0.f);
    h_ay.assign(numParticles, 0.f);
    h_output.assign(2 * (size_t)numNodes, 0.f);
    check(bh_create(&engine, numParticles, -1, &sys), "bh_create");
}

BarnesHutParticleSystem::BarnesHutParticleSystem(const BarnesHutParticleSystem& o)
    : parameters(o.parameters),
      step(o.step),
      numParticles(o.numParticles),
      numNodes(o.numNodes),
      engine(o.engine),
      sys(nullptr) {
    create();
    h_output = o.h_output;
    if (o.sys && bh_get_state(o.sys, h_x.data(), h_y.data(), h_vx.data(), h_vy.data(),
                              h_mass.data(), nullptr) == BH_OK) {
        bh_sync(o.sys, nullptr);
        check(bh_set_state(sys, h_x.data(), h_y.data(), h_vx.data(), h_vy.data(), h_mass.data(),
                           nullptr),
              "bh_set_state");
    }
}

BarnesHutParticleSystem& BarnesHutParticleSystem::operator=(const BarnesHutParticleSystem& o) {
    if (this != &o) {
        BarnesHutParticleSystem tmp(o);
        std::swap(parameters, tmp.parameters);
        std::swap(step, tmp.step);
        std::swap(numParticles, tmp.numParticles);
        std::swap(numNodes, tmp.numNodes);
        std::swap(engine, tmp.engine);
        std::swap(sys, tmp.sys);
        std::swap(h_mass, tmp.h_mass);
        std::swap(h_x, tmp.h_x);
        std::swap(h_y, tmp.h_y);
        std::swap(h_vx, tmp.h_vx);
        std::swap(h_vy, tmp.h_vy);
        std::swap(h_ax, tmp.h_ax);
        std::swap(h_ay, tmp.h_ay);
        std::swap(h_output, tmp.h_output);
    }
    return *this;
}

BarnesHutParticleSystem::~BarnesHutParticleSystem() {
    if (sys) bh_destroy(sys);
}

int BarnesHutParticleSystem::getNumParticles() { return numParticles; }

void BarnesHutParticleSystem::setEngineParams(const bh_params& p) {
    engine = p;
    check(bh_set_params(sys, &engine), "bh_set_params");
}

void BarnesHutParticleSystem::reset() {
    const int n = numParticles;
    int model = parameters.model == plummer_model          ? BH_MODEL_PLUMMER
                : parameters.model == colliding_disk_model ? BH_MODEL_COLLIDING_DISKS
                                                           : BH_MODEL_DISK;
    check(bh_initial_conditions(model, n, parameters.gravity, h_mass.data(), h_x.data(),
                                h_y.data(), h_vx.data(), h_vy.data()),
          "bh_initial_conditions");
    check(bh_set_state(sys, h_x.data(), h_y.data(), h_vx.data(), h_vy.data(), h_mass.data(),
                       nullptr),
          "bh_set_state");
    step = 0;
}

void BarnesHutParticleSystem::update() {
    auto t0 = std::chrono::steady_clock::now();
    check(bh_step(sys, 1, nullptr), "bh_step");
    check(bh_sync(sys, nullptr), "bh_step (device status)");
    float elapsed =
        std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (parameters.benchmark) {
        std::cout << "Timestep: " << step << "    " << "Elapsed time: " << elapsed << std::endl;
    }
    if (parameters.opengl) {
        check(bh_get_state(sys, h_x.data(), h_y.data(), nullptr, nullptr, nullptr, nullptr),
              "bh_get_state");
        check(bh_sync(sys, nullptr), "bh_get_state");
        for (int i = 0; i < numParticles; ++i) {
            h_output[2 * i] = h_x[i];
            h_output[2 * i + 1] = h_y[i];
        }
    }
    if (parameters.debug) runDebugTests();
    step++;
}

const float* BarnesHutParticleSystem::getOutputBuffer() { return h_output.data(); }

bool BarnesHutParticleSystem::writeImage(const char* path, int width, int height) {
    std::vector<unsigned char> rgba((size_t)width * height * 4);
    check(bh_render(sys, width, height, -25.0f, 25.0f, -25.0f, 25.0f, rgba.data(), nullptr),
          "bh_render");
    check(bh_sync(sys, nullptr), "bh_sync");
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    std::fprintf(f, "P6\n%d %d\n255\n", width, height);
    std::vector<unsigned char> rgb((size_t)width * height * 3);
    for (size_t p = 0; p < (size_t)width * height; ++p)
        for (int c = 0; c < 3; ++c) rgb[3 * p + c] = rgba[4 * p + c];
    const bool ok = std::fwrite(rgb.data(), 1, rgb.size(), f) == rgb.size();
    return std::fclose(f) == 0 && ok;
}

// debug.cpp:23-174, restated on the engine's tree and run on the device
// (bh_check); one line per invariant, in the reference's format.
void BarnesHutParticleSystem::runDebugTests() {
    unsigned failed = 0;
    check(bh_check(sys, nullptr, &failed), "bh_check");
    auto line = [&](const char* what, unsigned bits) {
        std::cout << what << " RESULT = " << ((failed & bits) ? "FAIL: " : "PASS: ") << std::endl;
    };
    line("COUNT ARRAY TEST 1", BH_CHECK_COUNT);
    line("CHILD ARRAY TEST 1", BH_CHECK_CHILD_SUM);
    line("CHILD ARRAY TEST 2", BH_CHECK_CHILD_RANGE);
    line("CHILD ARRAY TEST 3", BH_CHECK_PARENT);
    line("SORTED ARRAY TEST 1", BH_CHECK_PERMUTATION);
    line("SORTED ARRAY TEST 2", BH_CHECK_KEYS_SORTED);
    line("BOUNDING BOX TEST 1", BH_CHECK_BOX);
    line("MASS SUM TEST 1", BH_CHECK_MASS);
}
