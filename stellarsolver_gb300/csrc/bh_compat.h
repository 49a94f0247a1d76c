// Implementations behind both the C-linkage (include/Particle_cuda.cuh) and the
// C++-linkage (the reference's own Particle_cuda.cuh) wrapper names.
#pragma once
namespace ssg {
void compat_SetDrawArray(float* ptr, float* x, float* y, int n);
void compat_ResetArrays(int* mutex, float* x, float* y, float* mass, int* count, int* start, int* sorted, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m);
void compat_ComputeBoundingBox(int* mutex, float* x, float* y, float* left, float* right, float* bottom, float* top, int n);
void compat_BuildQuadTree(float* x, float* y, float* mass, int* count, int* start, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m);
void compat_ComputeCentreOfMass(float* x, float* y, float* mass, int* index, int n);
void compat_SortParticles(int* count, int* start, int* sorted, int* child, int* index, int n);
void compat_CalculateForces(float* x, float* y, float* vx, float* vy, float* ax, float* ay, float* mass, int* sorted, int* child, float* left, float* right, int n, float g);
void compat_IntegrateParticles(float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n, float dt, float d);
void compat_FillOutputArray(float* x, float* y, float* out, int n);
}  // namespace ssg
