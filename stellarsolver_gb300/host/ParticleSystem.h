// Abstract particle system with the reference's interface
// (pentilm/StellarSolver ParticleSystem.h:7-23).
#ifndef SSG_PARTICLESYSTEM_H
#define SSG_PARTICLESYSTEM_H

#include "SimulationParameters.h"

class ParticleSystem {
   public:
    SimulationParameters parameters;

    ParticleSystem(const SimulationParameters p, const int n) : parameters(p) { (void)n; }
    virtual ~ParticleSystem() {}

    virtual int getNumParticles() = 0;
    virtual void update() = 0;
    virtual void reset() = 0;
    virtual float* getOutputBuffer() = 0;
};

#endif
