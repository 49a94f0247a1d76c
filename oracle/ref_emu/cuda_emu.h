// Test infrastructure (oracle), never shipped: a CPU emulation of the few CUDA
// built-ins that the reference's kernels.cu uses, so that the reference's own
// kernel source can be compiled unmodified with g++ and executed on the host.
//
// Execution model (see ref_launch.cpp):
//   * one thread block per launch (gridDim.x == 1, blockDim.x <= 256);
//   * "fiber" launches run every CUDA thread as a ucontext fiber on ONE OS
//     thread; __syncthreads() and __all() are the only switch points, and
//     released fibers resume in thread-index order, which reproduces the
//     warp-lockstep ordering the reference relies on (lane 0 writes the shared
//     stack before the other lanes read it, kernels.cu:371-417);
//   * "pthread" launches run every CUDA thread as an OS thread; used only for
//     sort_kernel, whose spin on start[] (kernels.cu:316-335) needs true
//     concurrency.  The kernels are compiled at -O0 so that every global
//     access is a real load, like the reference's own -G build (Makefile:4).
//
// __shared__ becomes a function-local static: with a single block per launch
// that is exactly block-shared storage.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

struct emu_uint3 {
    unsigned x, y, z;
};

struct EmuThread;
struct EmuThreadIds {
    emu_uint3 tid;
    emu_uint3 bid;
};
extern thread_local EmuThreadIds* emu_cur_ids;
extern emu_uint3 emu_blockDim;
extern emu_uint3 emu_gridDim;

#define threadIdx (emu_cur_ids->tid)
#define blockIdx (emu_cur_ids->bid)
#define blockDim (emu_blockDim)
#define gridDim (emu_gridDim)

void emu_syncthreads();
int emu_vote_all(int pred);

static inline void __syncthreads() { emu_syncthreads(); }
static inline int __all(int pred) { return emu_vote_all(pred); }
static inline int __all_sync(unsigned, int pred) { return emu_vote_all(pred); }
static inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }

static inline int atomicCAS(int* addr, int compare, int val) {
    __atomic_compare_exchange_n(addr, &compare, val, false, __ATOMIC_SEQ_CST,
                                __ATOMIC_SEQ_CST);
    return compare;  // the old value in both outcomes
}
static inline int atomicExch(int* addr, int val) {
    return __atomic_exchange_n(addr, val, __ATOMIC_SEQ_CST);
}
static inline int atomicAdd(int* addr, int val) {
    return __atomic_fetch_add(addr, val, __ATOMIC_SEQ_CST);
}
static inline float atomicAdd(float* addr, float val) {
    unsigned* ua = reinterpret_cast<unsigned*>(addr);
    unsigned old = __atomic_load_n(ua, __ATOMIC_SEQ_CST);
    for (;;) {
        float f;
        std::memcpy(&f, &old, 4);
        float nf = f + val;
        unsigned nu;
        std::memcpy(&nu, &nf, 4);
        if (__atomic_compare_exchange_n(ua, &old, nu, false, __ATOMIC_SEQ_CST,
                                        __ATOMIC_SEQ_CST))
            return f;
    }
}

// CUDA's device rsqrt is an approximation; the host stand-in is the correctly
// rounded 1/sqrt, so forces from this emulation differ from a GPU run of the
// reference by a few ulp per term (within every force tolerance used here).
static inline float rsqrt(float v) { return 1.0f / std::sqrt(v); }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
