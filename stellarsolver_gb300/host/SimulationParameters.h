// Simulation parameters with the reference's fields and meaning
// (pentilm/StellarSolver SimulationParameters.h:6-25).  `iterations` is a
// float there too.  Engine settings that the reference fixes at compile time
// (theta, eps2, the force-walk mode) live in bh_params (include/stellar_bh.h).
#ifndef SSG_SIMULATIONPARAMETERS_H
#define SSG_SIMULATIONPARAMETERS_H

typedef enum Model { disk_model, colliding_disk_model, plummer_model } Model;

typedef struct SimulationParameters {
    Model model;
    bool opengl;
    bool debug;
    bool benchmark;
    bool fullscreen;
    float iterations;
    float timestep;
    float gravity;
    float dampening;
} SimulationParameters;

#endif
