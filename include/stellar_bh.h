/* stellar_bh.h -- C ABI of the GB300 (sm_103a) 2D Barnes-Hut engine.
 *
 * Drop-in boundary for the per-step pipeline of pentilm/StellarSolver:
 *   BarnesHutParticleSystem::update()   BarnesHutParticleSystem.cpp:301-347
 *   the nine launch wrappers            Particle_cuda.cuh:5-13 / Particle_cuda.cu:8-59
 * Plain C types only: pointers, sizes, ints and floats.  Every call returns a
 * status code (BH_OK == 0); the reference's wrappers return void and never
 * check errors (Particle_cuda.cu:8-59).  Streams are passed as `void*`
 * (a cudaStream_t, NULL = the legacy default stream).  Calls on one handle are
 * not thread-safe; different handles are independent.
 *
 * Body arrays at this boundary are in the caller's order (the order in which
 * bh_set_state received them), like the reference's d_x/d_y/... arrays
 * (BarnesHutParticleSystem.cpp:63-69).
 */
#ifndef STELLAR_BH_H
#define STELLAR_BH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define BH_OK 0
#define BH_ERR_ARG 1            /* bad argument (NULL handle, n < 1, bad mode ...) */
#define BH_ERR_DUPLICATE_KEYS 2 /* two bodies share all 32 key levels; the reference
                                   would split forever (kernels.cu:197-252) */
#define BH_ERR_NONFINITE 3      /* NaN/Inf position */
#define BH_ERR_CAPACITY 4       /* more bodies/cells than the buffers hold */
#define BH_ERR_STACK 5          /* walk stack overflow (raise stack_depth) */
#define BH_ERR_CUDA 6           /* a CUDA runtime call failed; see bh_last_error() */
#define BH_ERR_NOMEM 7          /* device or host allocation failed */
#define BH_ERR_STATE 8          /* call out of order (e.g. step before set_state) */
#define BH_ERR_NO_DEVICE 9      /* no CUDA device, or not an sm_103 device */
#define BH_ERR_TREE 10          /* a traversal exceeded its bound: the tree is not a valid
                                   tree of the keys (never for a valid build; reported
                                   instead of looping), or a bounded wait of the walk's
                                   shared groups ran out */

/* ---------------------------------------------------------------- modes */
/* REFERENCE: the reference's force law and opening rule, bit-for-bit tree:
 *   monopole, cell accepted iff every body of the 32-body group has
 *   (w^2/theta) <= |d|^2 + eps2 (kernels.cu:395-406), root children always
 *   opened, G not applied (kernels.cu:340: `g` unused), Euler-Cromer update
 *   v += dt*a; x += (d*dt)*v (kernels.cu:529-533).
 * PLAIN: accuracy mode in FP32: quadrupole moments; a node is approximated
 *   iff min over the group's bodies |COM - p| > l/theta + |COM - cell centre|
 *   (l = larger cell side) and G M l^3 / d^5 <= alpha |a_old| (previous
 *   step's |a|; the first step after bh_set_state bootstraps it with a
 *   geometric-only pass at opening angle max(theta, 1.25) with monopole cells);
 *   leaf buckets; G applied.
 * MIXED: PLAIN plus compensated (Kahan) force sums and positions kept as
 *   hi + lo float pairs. */
#define BH_MODE_REFERENCE 0
#define BH_MODE_PLAIN 1
#define BH_MODE_MIXED 2

/* Mirrors SimulationParameters (SimulationParameters.h:14-25) plus the
 * constants the reference fixes at compile time (kernels.cu:5-9). */
typedef struct bh_params {
    int mode;          /* BH_MODE_* */
    float theta;       /* opening angle; reference constant 0.5 (kernels.cu:9) */
    float eps2;        /* softening squared; reference constant 0.025 (kernels.cu:8) */
    float gravity;     /* G (SimulationParameters.gravity); ignored in REFERENCE mode */
    float timestep;    /* dt (SimulationParameters.timestep) */
    float dampening;   /* d: x += d*dt*v (SimulationParameters.dampening) */
    int leaf_bucket;   /* bodies per leaf in PLAIN/MIXED walks; 0 = tuned default */
    int block_size;    /* walk threads per block; 0 = tuned default */
    int stack_depth;   /* walk stack entries per warp; 0 = tuned default */
    int use_graph;     /* 1 = replay the step as a CUDA graph */
    float alpha;       /* PLAIN/MIXED relative opening tolerance: a cell of mass M and size l
                          at distance d is approximated only if G M l^3 / d^5 <= alpha |a_old|
                          (Springel 2005-style); 0 = geometric rule only; default 0.01 */
    int bodies_per_lane; /* PLAIN/MIXED walk: a warp walks the tree once for 32 (1) or 64 (2)
                            consecutive bodies; 0 = tuned default */
    int share_tail;      /* PLAIN/MIXED walk, shared groups: the owner of a shared walk group
                            walks the tree, warps between groups evaluate its interactions.
                            Results are bit-identical with or without sharing.  k > 0: the
                            heavy groups and the last k groups handed out; 0 = default: the
                            heavy groups when the walk has no more groups than the GPU has
                            resident walk warps (about 2^17 bodies on GB300); -1 = none */
} bh_params;

typedef struct bh_system bh_system;

/* Counters of the last bh_step call (device-side, read back on request). */
typedef struct bh_stats {
    int64_t interactions;  /* body-node interactions in the last step */
    int32_t cells;         /* reference-tree cells (key prefixes shared by >= 2 bodies) */
    int32_t nodes;         /* branching quadtree nodes */
    int32_t max_depth;     /* deepest leaf level */
    int32_t status;        /* sticky device status (BH_* code) */
    float box[4];          /* left, right, bottom, top of the last step */
    int32_t max_stack;     /* deepest walk stack of the last step (PLAIN/MIXED) */
    int32_t walk_rounds;   /* warp rounds of node tests in the last step (PLAIN/MIXED) */
    int32_t nodes_tested;  /* nodes tested by the walk in the last step (PLAIN/MIXED) */
    int64_t cell_interactions; /* of `interactions`, body-cell (quadrupole) ones (PLAIN/MIXED) */
} bh_stats;

/* Fill p with the reference's defaults: mode REFERENCE, theta 0.5, eps2 0.025,
 * G 1, dt 0.001, dampening 1 (main.cpp:92-95, kernels.cu:8-9). */
void bh_default_params(bh_params* p);

/* BarnesHutParticleSystem(p, n) (BarnesHutParticleSystem.cpp:28-84): allocate
 * device storage for n bodies.  No reference counterpart for `device`:
 * device ordinal (-1 = current). */
int bh_create(const bh_params* p, int n, int device, bh_system** out);

/* A batch of nsys independent systems in one handle (no reference
 * counterpart: the reference runs one system).  System k's bodies occupy
 * [bh_system_offset(s, k), + sizes[k]) of every body array passed to or from
 * the handle; each system has its own box, tree and walk, and every phase is
 * one launch over the whole batch.  bh_step advances all systems. */
int bh_ensemble_create(const bh_params* p, int nsys, const int* sizes, int device,
                       bh_system** out);
int bh_num_systems(const bh_system* s);
int bh_system_offset(const bh_system* s, int k);

/* ~BarnesHutParticleSystem (BarnesHutParticleSystem.cpp:249-292). */
int bh_destroy(bh_system* s);

int bh_set_params(bh_system* s, const bh_params* p);
int bh_get_params(const bh_system* s, bh_params* p);
int bh_num_bodies(const bh_system* s); /* getNumParticles() (BarnesHutParticleSystem.cpp:295) */

/* reset()'s host-to-device copy (BarnesHutParticleSystem.cpp:364-371).  Any
 * pointer may be host or device memory (cudaMemcpyDefault).  Accelerations
 * start at zero.  Asynchronous on `stream`, like cudaMemcpyAsync.  x and y
 * are copied on `stream`; vx, vy and mass on the handle's own copy stream,
 * overlapped with the next step's box, keys and sort, and ordered before the
 * work of the next call on the handle (bh_step joins them just before the
 * reorder), on that call's stream.  So pinned host or device sources must stay
 * unchanged until `stream` has passed the next call on the handle, e.g.
 * bh_step or bh_sync (pageable host memory is staged before the call
 * returns). */
int bh_set_state(bh_system* s, const float* x, const float* y, const float* vx,
                 const float* vy, const float* mass, void* stream);

/* Accelerations of the state just loaded by bh_set_state (caller's order,
 * host or device pointers), like the reference's reset() upload of d_ax/d_ay
 * (BarnesHutParticleSystem.cpp:370-371).  PLAIN/MIXED use |a| as the scale of
 * the relative opening rule, so the next step skips the bootstrap pass.
 * Copied on the handle's copy stream like bh_set_state's vx, vy and mass, with
 * the same rule for the sources. */
int bh_set_accel(bh_system* s, const float* ax, const float* ay, void* stream);

/* Copy the current state out in the caller's order (any of the pointers may be
 * NULL to skip it).  For MIXED mode x/y are hi+lo rounded to float. */
int bh_get_state(bh_system* s, float* x, float* y, float* vx, float* vy, float* mass,
                 void* stream);

/* Accelerations of the last step, caller's order (d_ax/d_ay of the reference). */
int bh_get_accel(bh_system* s, float* ax, float* ay, void* stream);

/* Positions as hi/lo pairs (MIXED keeps lo; other modes return lo = 0). */
int bh_get_positions_hilo(bh_system* s, float* xhi, float* xlo, float* yhi, float* ylo,
                          void* stream);

/* update() x steps (BarnesHutParticleSystem.cpp:301-347): bbox, keys, radix
 * sort, tree, moments, force walk fused with the integration.  Asynchronous on
 * `stream`; the returned status covers launch errors only.  Device-side errors
 * (duplicate keys, non-finite input, stack overflow) are sticky and reported
 * by bh_sync / bh_get_stats. */
int bh_step(bh_system* s, int steps, void* stream);

/* Wait for `stream`, then return the sticky device status. */
int bh_sync(bh_system* s, void* stream);

int bh_get_stats(bh_system* s, bh_stats* out, void* stream);

/* Headless rendering of the current positions, in place of the reference's
 * OpenGL viewer (StellarSolverVisualizer.cpp:4-20, 208-253: one-pixel points,
 * glm::ortho(-25, 25, -25, 25) on a 1000x1000 window, colour (1,1,1,0.1)
 * blended with (GL_SRC_ALPHA, GL_ONE) over a (0,0,0,0.5) clear).  A body at
 * (x, y) lights pixel column floor((x - x0) * width / (x1 - x0)) and row
 * floor((y - y0) * height / (y1 - y0)) counted from the bottom; rgba receives
 * width*height RGBA8 pixels, top row first.  A pixel hit by c bodies has
 * colour min(1, 0.1 c) and alpha min(1, 0.5 + 0.01 c), rounded to 1/255.
 * rgba may be host or device memory; the copy is ordered on `stream`. */
int bh_render(bh_system* s, int width, int height, float x0, float x1, float y0, float y1,
              unsigned char* rgba, void* stream);

/* Tree invariants of the last step, checked on the device.  The reference
 * copies every tree array to the host and checks it there (debug.cpp:23-174,
 * BarnesHutParticleSystem.cpp:331-344); here the same invariants, stated for
 * the engine's binary radix tree, run as three kernels.  *failed receives the
 * BH_CHECK_* bits of the invariants that do not hold (0: all hold).
 * Synchronous.  Checks the tree of the last bh_step (or bh_energy, which
 * builds one for the current positions); BH_ERR_STATE before the first step
 * after bh_set_state. */
#define BH_CHECK_COUNT 1u         /* a node's range is not the union of its children's (count test) */
#define BH_CHECK_CHILD_SUM 2u     /* some position is not a leaf child exactly once (child test 1) */
#define BH_CHECK_CHILD_RANGE 4u   /* a child index outside its system (child tests 2-3) */
#define BH_CHECK_PARENT 8u        /* parent links do not point back */
#define BH_CHECK_KEYS_SORTED 16u  /* keys not ascending within a system */
#define BH_CHECK_PERMUTATION 32u  /* positions' caller indices not a permutation (sorted tests) */
#define BH_CHECK_BOX 64u          /* left > right or bottom > top (bounding box test) */
#define BH_CHECK_MASS 128u        /* a node's mass is not the sum of its children's */
int bh_check(bh_system* s, void* stream, unsigned* failed);

/* Copy a named internal array of the last step to host memory (test and
 * debugging aid).  Names and element types:
 *   "box" f32[4] (left, right, bottom, top of system 0), "boxes" f32[4 nseg]
 *   (every system's), "keys" u64[n] (sorted), "perm" i32[n] (caller index of each
 *   sorted position), "node_left" "node_right" "node_split" "node_first"
 *   "node_last" "node_parent" i32[n], "node_m" "node_mx" "node_my" "node_cx"
 *   "node_cy" f32[n] (node arrays have n entries; entry n-1 is unused),
 *   "accel_sorted" f32[2n] (ax then ay), "share" i32[4] (the last walk's shared
 *   groups: slices handed out from the queue, slices reserved, pool batches
 *   reserved, slices taken back by their owners).
 * Returns BH_ERR_ARG for an unknown name or a too small buffer. */
int bh_get_debug(bh_system* s, const char* name, void* host_out, size_t bytes, void* stream);

/* Phases timed by bh_step_profiled, in order. */
#define BH_NUM_PHASES 9 /* bbox, keys, sort, reorder, build, moments and walk records,
                          bootstrap (accuracy modes, first step after bh_set_state),
                          frontier (accuracy modes: shared walk starts and heavy groups),
                          walk (the force walk kernel alone) */

/* One step (never graph-replayed) with CUDA events at the phase boundaries;
 * synchronises, then ADDS each phase's milliseconds to phase_ms[0..8].
 * No reference counterpart (the reference times the whole step only,
 * BarnesHutParticleSystem.cpp:303-321). */
int bh_step_profiled(bh_system* s, void* stream, float* phase_ms);

/* FP64 O(N^2) direct-sum accelerations at ns caller indices idx[] for the
 * current state (hi+lo positions in MIXED mode), times G (1 in REFERENCE
 * mode).  Results to host arrays.  Diagnostic for the force-error report; no
 * reference counterpart.  Synchronous. */
int bh_direct_sum_f64(bh_system* s, int ns, const int* idx, double* ax, double* ay);

/* FP64 energy and momentum of every system of the handle at the current
 * positions: out[4k+0] kinetic 0.5 sum m v^2, out[4k+1] potential
 * 0.5 sum m phi with phi from a tree walk over a tree of the current
 * positions (geometric opening rule, quadrupole cells, softened like the
 * forces, per-body sums in FP64), out[4k+2..3] momentum.  The state is not
 * changed.  Synchronous.  No reference counterpart. */
int bh_energy(bh_system* s, void* stream, double* out);

/* The same diagnostics recorded on the device after every `every`-th step of
 * bh_step, into a ring of `capacity` records of 4*systems doubles (layout as
 * bh_energy).  In graph mode the diagnostics pass is captured once as its own
 * CUDA graph and launched after every k-th step graph; no host synchronisation.
 * every = 0 turns the log off.  Resets the record count. */
int bh_set_energy_log(bh_system* s, int every, int capacity);
/* Synchronises `stream`; *records = records written since bh_set_energy_log
 * (record r follows step every*(r+1)); out receives the last
 * min(*records, capacity, max_records) of them, oldest first. */
int bh_get_energy_log(bh_system* s, double* out, int max_records, int* records, void* stream);

/* Measure the device's FP32 FMA throughput (TFLOP/s, 2 flops per FMA) with
 * register-only kernels on every SM, one of scalar FFMA chains and one of
 * packed FP32x2 FFMA2 chains (the instruction the force walk issues); the
 * larger is the roofline denominator of the force walk.  device -1 = current.
 * No reference counterpart. */
int bh_measure_fp32_peak(int device, double* tflops);
/* The same probe, both figures: *scalar (FFMA) and *packed (FFMA2). */
int bh_measure_fp32_peaks(int device, double* scalar, double* packed);

/* The reference's initial conditions, number for number: the Model enum of
 * SimulationParameters.h:8-13 and the generators of
 * BarnesHutParticleSystem.cpp:390-560 (std::default_random_engine, default
 * seed).  Host arrays of n floats; accelerations start at zero.  gravity
 * enters the disk velocities only, as in the reference. */
#define BH_MODEL_DISK 0
#define BH_MODEL_COLLIDING_DISKS 1
#define BH_MODEL_PLUMMER 2
int bh_initial_conditions(int model, int n, float gravity, float* mass, float* x, float* y,
                          float* vx, float* vy);

/* Choose the accuracy walk's shape for the current state: the stack depth
 * from the deepest stack of one step (x1.5), then the fastest of block sizes
 * {128, 256} x leaf buckets {4, 8, 16}, each timed over two steps from the
 * same saved state.  The state is restored afterwards, and the chosen values
 * are stored in the system's parameters (and copied to *chosen if not NULL).
 * REFERENCE mode has nothing to tune.  Replaces the reference's hand-matched
 * blockSize/gridSize constants (Particle_cuda.cu:5-6, README.md:59).
 * Allocates a temporary state backup; synchronous. */
int bh_autotune(bh_system* s, void* stream, bh_params* chosen);

/* Human-readable text for a status code, and the last CUDA error seen by the
 * library in this thread. */
const char* bh_status_string(int status);
const char* bh_last_error(void);

/* Library build identification: "<version> sm_103a". */
const char* bh_version(void);

#ifdef __cplusplus
}
#endif
#endif /* STELLAR_BH_H */
