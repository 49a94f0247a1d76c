// C++-linkage exports with the exact names and signatures of the reference's
// Particle_cuda.cuh:5-13, so the reference's unmodified host sources (which
// include their own header) link against this library.  Each forwards to the
// same implementation as the C-linkage entry points.
#include "bh_compat.h"

void SetDrawArray(float* ptr, float* x, float* y, int n) { ssg::compat_SetDrawArray(ptr, x, y, n); }
void ResetArrays(int* mutex, float* x, float* y, float* mass, int* count, int* start, int* sorted, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m) { ssg::compat_ResetArrays(mutex, x, y, mass, count, start, sorted, child, index, left, right, bottom, top, n, m); }
void ComputeBoundingBox(int* mutex, float* x, float* y, float* left, float* right, float* bottom, float* top, int n) { ssg::compat_ComputeBoundingBox(mutex, x, y, left, right, bottom, top, n); }
void BuildQuadTree(float* x, float* y, float* mass, int* count, int* start, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m) { ssg::compat_BuildQuadTree(x, y, mass, count, start, child, index, left, right, bottom, top, n, m); }
void ComputeCentreOfMass(float* x, float* y, float* mass, int* index, int n) { ssg::compat_ComputeCentreOfMass(x, y, mass, index, n); }
void SortParticles(int* count, int* start, int* sorted, int* child, int* index, int n) { ssg::compat_SortParticles(count, start, sorted, child, index, n); }
void CalculateForces(float* x, float* y, float* vx, float* vy, float* ax, float* ay, float* mass, int* sorted, int* child, float* left, float* right, int n, float g) { ssg::compat_CalculateForces(x, y, vx, vy, ax, ay, mass, sorted, child, left, right, n, g); }
void IntegrateParticles(float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n, float dt, float d) { ssg::compat_IntegrateParticles(x, y, vx, vy, ax, ay, n, dt, d); }
void FillOutputArray(float* x, float* y, float* out, int n) { ssg::compat_FillOutputArray(x, y, out, n); }
