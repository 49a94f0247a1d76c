// Test infrastructure (oracle), never shipped.  Host launcher for the
// reference's kernels.cu compiled with g++ through cuda_emu.h.
//
// Each entry point mirrors one launch wrapper of Particle_cuda.cu:8-59 (same
// argument list), plus a leading `block` argument: the emulated launch is
// always ONE block of `block` threads (power of two, 32..256), so the kernels'
// grid-stride loops run with stride == block.  Return value: 0 on success,
// -1 if the fiber scheduler found a deadlock (threads of a warp split between a
// vote and a barrier, which is undefined behaviour on a real GPU as well).
#include <pthread.h>
#include <ucontext.h>

#include <cstdlib>
#include <functional>
#include <vector>

#include "cuda_emu.h"
#include "kernels.cuh"

thread_local EmuThreadIds* emu_cur_ids = nullptr;
emu_uint3 emu_blockDim = {1, 1, 1};
emu_uint3 emu_gridDim = {1, 1, 1};

namespace {

enum FiberState { RUNNABLE, AT_BARRIER, AT_VOTE, EXITED };

struct Fiber {
    ucontext_t ctx;
    EmuThreadIds ids;
    FiberState state;
    int vote;
    int vote_result;
    std::vector<char> stack;
};

ucontext_t g_sched_ctx;
std::vector<Fiber>* g_fibers = nullptr;
Fiber* g_cur = nullptr;
const std::function<void()>* g_body = nullptr;
bool g_pthread_mode = false;
constexpr size_t kFiberStack = 256 * 1024;

void fiber_entry() {
    (*g_body)();
    g_cur->state = EXITED;
    swapcontext(&g_cur->ctx, &g_sched_ctx);
}

int launch_fibers(int block, const std::function<void()>& body) {
    std::vector<Fiber> fibers(block);
    g_fibers = &fibers;
    g_body = &body;
    g_pthread_mode = false;
    emu_blockDim = {(unsigned)block, 1, 1};
    emu_gridDim = {1, 1, 1};
    for (int i = 0; i < block; ++i) {
        Fiber& f = fibers[i];
        f.ids.tid = {(unsigned)i, 0, 0};
        f.ids.bid = {0, 0, 0};
        f.state = RUNNABLE;
        f.stack.resize(kFiberStack);
        getcontext(&f.ctx);
        f.ctx.uc_stack.ss_sp = f.stack.data();
        f.ctx.uc_stack.ss_size = f.stack.size();
        f.ctx.uc_link = nullptr;
        makecontext(&f.ctx, fiber_entry, 0);
    }
    const int warps = (block + 31) / 32;
    for (;;) {
        for (int i = 0; i < block; ++i) {
            if (fibers[i].state != RUNNABLE) continue;
            g_cur = &fibers[i];
            emu_cur_ids = &g_cur->ids;
            swapcontext(&g_sched_ctx, &g_cur->ctx);
        }
        int live = 0, at_bar = 0;
        for (auto& f : fibers) {
            if (f.state != EXITED) ++live;
            if (f.state == AT_BARRIER) ++at_bar;
        }
        if (live == 0) break;
        bool released = false;
        for (int w = 0; w < warps; ++w) {
            int lo = 32 * w, hi = lo + 32 < block ? lo + 32 : block;
            int wl = 0, wv = 0, all = 1;
            for (int i = lo; i < hi; ++i) {
                if (fibers[i].state == EXITED) continue;
                ++wl;
                if (fibers[i].state == AT_VOTE) {
                    ++wv;
                    all &= (fibers[i].vote != 0);
                }
            }
            if (wl > 0 && wv == wl) {
                for (int i = lo; i < hi; ++i) {
                    if (fibers[i].state == AT_VOTE) {
                        fibers[i].vote_result = all;
                        fibers[i].state = RUNNABLE;
                    }
                }
                released = true;
            }
        }
        if (!released && at_bar == live) {
            for (auto& f : fibers)
                if (f.state == AT_BARRIER) f.state = RUNNABLE;
            released = true;
        }
        if (!released) {
            std::fprintf(stderr, "ref_emu: deadlock (live=%d at_barrier=%d)\n", live, at_bar);
            g_fibers = nullptr;
            return -1;
        }
    }
    g_fibers = nullptr;
    g_cur = nullptr;
    emu_cur_ids = nullptr;
    return 0;
}

struct PthreadArg {
    EmuThreadIds ids;
    const std::function<void()>* body;
};

void* pthread_entry(void* p) {
    PthreadArg* a = static_cast<PthreadArg*>(p);
    emu_cur_ids = &a->ids;
    (*a->body)();
    return nullptr;
}

int launch_pthreads(int block, const std::function<void()>& body) {
    g_pthread_mode = true;
    emu_blockDim = {(unsigned)block, 1, 1};
    emu_gridDim = {1, 1, 1};
    std::vector<PthreadArg> args(block);
    std::vector<pthread_t> th(block);
    pthread_attr_t attr;
    pthread_attr_init(&attr);
    pthread_attr_setstacksize(&attr, kFiberStack);
    for (int i = 0; i < block; ++i) {
        args[i].ids.tid = {(unsigned)i, 0, 0};
        args[i].ids.bid = {0, 0, 0};
        args[i].body = &body;
        pthread_create(&th[i], &attr, pthread_entry, &args[i]);
    }
    for (int i = 0; i < block; ++i) pthread_join(th[i], nullptr);
    pthread_attr_destroy(&attr);
    g_pthread_mode = false;
    return 0;
}

bool block_ok(int block) {
    return block >= 32 && block <= 256 && (block & (block - 1)) == 0;
}

}  // namespace

void emu_syncthreads() {
    if (g_pthread_mode) {
        std::fprintf(stderr, "ref_emu: __syncthreads in a pthread launch\n");
        std::abort();
    }
    g_cur->state = AT_BARRIER;
    swapcontext(&g_cur->ctx, &g_sched_ctx);
}

int emu_vote_all(int pred) {
    if (g_pthread_mode) {
        std::fprintf(stderr, "ref_emu: __all in a pthread launch\n");
        std::abort();
    }
    g_cur->vote = pred;
    g_cur->state = AT_VOTE;
    swapcontext(&g_cur->ctx, &g_sched_ctx);
    return g_cur->vote_result;
}

extern "C" {

int refemu_ResetArrays(int block, int* mutex, float* x, float* y, float* mass, int* count,
                       int* start, int* sorted, int* child, int* index, float* left,
                       float* right, float* bottom, float* top, int n, int m) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] {
        reset_arrays_kernel(mutex, x, y, mass, count, start, sorted, child, index, left, right,
                            bottom, top, n, m);
    });
}

int refemu_ComputeBoundingBox(int block, int* mutex, float* x, float* y, float* left,
                              float* right, float* bottom, float* top, int n) {
    if (!block_ok(block) || n < block) return -2;
    return launch_fibers(block, [&] {
        compute_bounding_box_kernel(mutex, x, y, left, right, bottom, top, n);
    });
}

int refemu_BuildQuadTree(int block, float* x, float* y, float* mass, int* count, int* start,
                         int* child, int* index, float* left, float* right, float* bottom,
                         float* top, int n, int m) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] {
        build_tree_kernel(x, y, mass, count, start, child, index, left, right, bottom, top, n, m);
    });
}

int refemu_ComputeCentreOfMass(int block, float* x, float* y, float* mass, int* index, int n) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] { centre_of_mass_kernel(x, y, mass, index, n); });
}

int refemu_SortParticles(int block, int* count, int* start, int* sorted, int* child, int* index,
                         int n) {
    if (!block_ok(block)) return -2;
    return launch_pthreads(block, [&] { sort_kernel(count, start, sorted, child, index, n); });
}

int refemu_CalculateForces(int block, float* x, float* y, float* vx, float* vy, float* ax,
                           float* ay, float* mass, int* sorted, int* child, float* left,
                           float* right, int n, float g) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] {
        compute_forces_kernel(x, y, vx, vy, ax, ay, mass, sorted, child, left, right, n, g);
    });
}

int refemu_IntegrateParticles(int block, float* x, float* y, float* vx, float* vy, float* ax,
                              float* ay, int n, float dt, float d) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] { update_kernel(x, y, vx, vy, ax, ay, n, dt, d); });
}

int refemu_FillOutputArray(int block, float* x, float* y, float* out, int n) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] { copy_kernel(x, y, out, n); });
}

int refemu_SetDrawArray(int block, float* ptr, float* x, float* y, int n) {
    if (!block_ok(block)) return -2;
    return launch_fibers(block, [&] { set_draw_array_kernel(ptr, x, y, n); });
}

}  // extern "C"
