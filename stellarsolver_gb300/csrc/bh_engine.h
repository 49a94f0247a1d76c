// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "bh_walk.cuh"
#include "stellar_bh.h"

namespace ssg {

extern thread_local std::string g_last_error;
int cuda_fail(cudaError_t e, const char* what);

// Everything the walk launch needs for one step of one batch.
struct StepArgs {
    int mode;
    Segs segs;
    Groups groups;   // groups of 32 consecutive bodies
    Groups groups2;  // groups of 64 (accuracy walk with two bodies per lane)
    WalkIn in;
    WalkOut out;
    const float4* recA;
    const float4* recB;
    const int4* recC;
    const int4* recD;
    float eps2, G, dt, ddt, alpha;
    int* status;
    unsigned long long* inter;
    int* work;   // [0] reference walk, [1] bootstrap pass, [2] accuracy walk
    int* fresh;  // set by bh_set_state: the next step bootstraps |a_old|
    int* max_stack;  // deepest accuracy-walk stack of the step
    int bucket, stack, warps;  // accuracy-walk shape: leaf bucket, stack entries, warps/block
    int bpl;                   // accuracy walk: bodies per lane (1 or 2)
    int walk_grid_ref, walk_grid_acc;
    Frontier frontier;  // shared walk starts (main accuracy pass)
    Heavy heavy;        // heavy walk groups first (main accuracy pass)
    Share share;        // shared walk groups (main accuracy pass)
};

cudaError_t launch_walk(const StepArgs& a, cudaStream_t st, int part);
cudaError_t init_walk_attributes();
int normalized_bucket(int b);
int normalized_stack(int s);
int normalized_bpl(int b);
int normalized_warps(int block);

// Create a batch of independent systems of the given sizes (bh_create is the
// single-system case).
int system_create(const bh_params* p, const int* sizes, int nseg, int device, bh_system** out);

}  // namespace ssg
