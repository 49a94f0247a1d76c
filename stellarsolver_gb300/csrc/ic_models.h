// The reference's initial-condition models (BarnesHutParticleSystem.cpp:390-560),
// producing the same numbers: std::default_random_engine with its default seed,
// the same uniform_real_distribution<float> objects drawn in the same order,
// and the same float/double mix in the formulas.
#ifndef SSG_IC_MODELS_H
#define SSG_IC_MODELS_H

namespace ssg_ic {

// Plummer model: r = a / sqrt(u^-0.666666 - 1); speeds by rejection sampling of
// s^2 (1-s^2)^3.5; isotropic directions in the plane.
void plummer(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n);

// One disk: body 0 of mass 2e5 at rest, the others on circular orbits of radius
// U[1.5, 12] with speed sqrt(G * 2e5 / r), counter-clockwise.
void disk(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n,
          float gravity);

// Two disks: masses 1e5 (at rest at the origin) and 2.5e4 (body 1, 20 away);
// bodies 2..3n/4 orbit body 0 at U[1.5, 12], the rest orbit body 1 at U[1, 5].
void colliding_disks(float* mass, float* x, float* y, float* vx, float* vy, float* ax, float* ay,
                     int n, float gravity);

}  // namespace ssg_ic

#endif
