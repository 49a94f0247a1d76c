/* Particle_cuda.cuh -- drop-in replacement for the reference's launch-wrapper
 * header (pentilm/StellarSolver Particle_cuda.cuh:5-13).
 *
 * Same nine functions, same names, same argument lists and meaning, same
 * array layout: SoA device arrays of length m = 2n+12000 (bodies 0..n-1,
 * cells n..m-1), child[4*node + slot] with the root in slots child[0..3]
 * (BarnesHutParticleSystem.cpp:33, kernels.cu:159).  They are exported with C
 * linkage from libstellar_bh.so, so the reference's own
 * BarnesHutParticleSystem.cpp compiles against this header unchanged and links
 * against this library instead of Particle_cuda.cu + kernels.cu.
 *
 * Differences from the reference, all deliberate:
 *  - no locks or spin-waits: the tree is built from sorted quadrant keys;
 *  - errors are recorded instead of ignored: bh_compat_status() returns the
 *    first BH_* status since the last bh_compat_clear_status();
 *  - launch shapes are sized from n (no hand-matched blockSize/gridSize,
 *    README.md:59);
 *  - the compile-time constants theta = 0.5 and eps2 = 0.025
 *    (kernels.cu:8-9) are the defaults of bh_compat_set_constants();
 *  - a root child that is a single body interacts directly (the reference
 *    walks it as a node, which drops it or, for body 0, counts the root twice).
 * Work is issued on the stream set by bh_compat_set_stream (default: the
 * legacy default stream, like the reference).
 */
#ifndef PARTICLE_CUDA_CUH_SSG
#define PARTICLE_CUDA_CUH_SSG

#ifdef __cplusplus
extern "C" {
#endif

/* Particle_cuda.cu:8-11: ptr[2i], ptr[2i+1] = x[i], y[i] for i < n. */
void SetDrawArray(float *ptr, float *x, float *y, int n);

/* Particle_cuda.cu:14-17 / kernels.cu:25-59: child = -1, count = 1 (bodies)
 * or 0 (cells), cell x/y/mass = 0, start = -1, sorted = 0, *index = n, box and
 * mutex = 0. */
void ResetArrays(int *mutex, float *x, float *y, float *mass, int *count, int *start, int *sorted,
                 int *child, int *index, float *left, float *right, float *bottom, float *top,
                 int n, int m);

/* Particle_cuda.cu:20-23 / kernels.cu:62-114: merge min/max of x and y into
 * *left..*top (lock-free; mutex unused). */
void ComputeBoundingBox(int *mutex, float *x, float *y, float *left, float *right, float *bottom,
                        float *top, int n);

/* Particle_cuda.cu:26-29 / kernels.cu:117-271: the quadtree of the bodies in
 * the box: one cell per key prefix shared by >= 2 bodies, numbered from n;
 * cell x/y/mass hold sum(m*x), sum(m*y), sum(m); count, start = -1, *index. */
void BuildQuadTree(float *x, float *y, float *mass, int *count, int *start, int *child, int *index,
                   float *left, float *right, float *bottom, float *top, int n, int m);

/* Particle_cuda.cu:32-35 / kernels.cu:275-288: x /= mass, y /= mass for cells
 * n..*index-1. */
void ComputeCentreOfMass(float *x, float *y, float *mass, int *index, int n);

/* Particle_cuda.cu:38-41 / kernels.cu:292-336: sorted[] = bodies in depth-first
 * order over child slots 0..3, start[cell] = first position of each cell.  On
 * the arrays of the last BuildQuadTree on this device (same child array and
 * n) both come from that build's workspace (depth-first order is its key
 * order); otherwise the cells are walked level by level. */
void SortParticles(int *count, int *start, int *sorted, int *child, int *index, int n);

/* Particle_cuda.cu:44-47 / kernels.cu:340-435: warp-vote walk; g is unused,
 * as in the reference.  Above 98,304 bodies, on the arrays of the last
 * BuildQuadTree on this device, the walk runs on that build's compressed tree
 * (the same interaction set; forces equal to 1e-5 of their RMS, the summation
 * order differs); otherwise it walks child[]. */
void CalculateForces(float *x, float *y, float *vx, float *vy, float *ax, float *ay, float *mass,
                     int *sorted, int *child, float *left, float *right, int n, float g);

/* Particle_cuda.cu:50-53 / kernels.cu:522-537: v += dt*a; x += d*dt*v. */
void IntegrateParticles(float *x, float *y, float *vx, float *vy, float *ax, float *ay, int n,
                        float dt, float d);

/* Particle_cuda.cu:56-59 / kernels.cu:541-553: out[2i], out[2i+1] = x[i], y[i]. */
void FillOutputArray(float *x, float *y, float *out, int n);

/* ---- additions (no reference counterpart) ---- */

/* Opening angle and softening used by CalculateForces (defaults 0.5, 0.025). */
void bh_compat_set_constants(float theta, float eps2);
/* Stream for the wrappers (cudaStream_t as void*; NULL = legacy stream). */
void bh_compat_set_stream(void *stream);
/* First BH_* status recorded by a wrapper in this thread since the last clear;
 * synchronises the compat stream first so device-side errors are included. */
int bh_compat_status(void);
void bh_compat_clear_status(void);
/* Release the scratch the wrappers keep between calls (keys, sort and tree
 * buffers grown on demand on the current device). */
void bh_compat_release(void);

/* BuildQuadTree for callers that cannot allocate device memory.  No
 * counterpart in the reference.  Such callers include a host that owns the
 * whole device-memory budget, a real-time loop that cannot afford an
 * allocation stall, and code whose allocator the library cannot call.
 * BuildQuadTree grows a cached workspace with cudaMalloc; this variant calls
 * no cudaMalloc/cudaFree and no allocating library routine.  Its scratch is
 * one static device array sized for at most 65536 bodies (about 8.5 MiB), which
 * every GPU that loads the library holds until the process exits.
 *   - Same arguments and outputs as BuildQuadTree.  Returns a BH_* status:
 *     BH_ERR_CAPACITY for n > 65536 (see bh_last_error), else the build's
 *     device status.  A failure is also recorded for bh_compat_status().
 *   - Synchronous: it waits on the compat stream and copies its status word
 *     to the host before it returns, so it cannot be called while a stream is
 *     being captured or a CUDA graph is being built.
 *   - The first call on a device resolves the array's device address
 *     (cudaGetSymbolAddress) once for that device.
 *   - All calls share the one array and it keeps the last call's contents.
 *     Calls that overlap on the GPU (other host threads, other streams) race;
 *     serialise them.
 *   - Only this tree build is free of allocation.  ComputeBoundingBox,
 *     SortParticles and CalculateForces (and BuildQuadTree) still keep a
 *     cudaMalloc'ed workspace per device, allocated on their first call and
 *     grown when a larger layout needs it; bh_compat_release frees it. */
int BuildQuadTreeNoAlloc(float *x, float *y, float *mass, int *count, int *start, int *child,
                         int *index, float *left, float *right, float *bottom, float *top, int n,
                         int m);

#ifdef __cplusplus
}
#endif
#endif /* PARTICLE_CUDA_CUH_SSG */
