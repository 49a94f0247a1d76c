// Host class with the reference's public interface
// (pentilm/StellarSolver BarnesHutParticleSystem.h:62-71), implemented on the
// engine's C ABI (include/stellar_bh.h) instead of nine raw-pointer launches.
#ifndef SSG_BARNESHUTPARTICLESYSTEM_H
#define SSG_BARNESHUTPARTICLESYSTEM_H

#include <vector>

#include "SimulationParameters.h"
#include "stellar_bh.h"

class BarnesHutParticleSystem {
   private:
    SimulationParameters parameters;
    int step;
    int numParticles;
    int numNodes;  // 2n + 12000, the reference's node capacity (BarnesHutParticleSystem.cpp:33)
    bh_params engine;
    bh_system* sys;
    std::vector<float> h_mass, h_x, h_y, h_vx, h_vy, h_ax, h_ay;
    std::vector<float> h_output;  // 2*numNodes floats: x,y of the bodies first

    void create();
    void runDebugTests();

   public:
    BarnesHutParticleSystem(const SimulationParameters p, const int n);
    // Copies carry the state (the reference's copy reallocates without copying data).
    BarnesHutParticleSystem(const BarnesHutParticleSystem& system);
    BarnesHutParticleSystem& operator=(const BarnesHutParticleSystem& system);
    ~BarnesHutParticleSystem();

    int getNumParticles();
    void update();
    void reset();

    const float* getOutputBuffer();
    // Headless stand-in for the reference's viewer frame (StellarSolverVisualizer.cpp:
    // 208-253): the current positions as one-pixel points over [-25, 25]^2, written to
    // `path` as a binary PPM (P6, RGB).  Returns false if the file cannot be written.
    bool writeImage(const char* path, int width = 1000, int height = 1000);

    // Additions: the engine settings that the reference fixes at compile time.
    void setEngineParams(const bh_params& p);
    const bh_params& getEngineParams() const { return engine; }
    bh_system* handle() { return sys; }
};

#endif
