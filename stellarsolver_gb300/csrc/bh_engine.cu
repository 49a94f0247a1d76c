// Host side of the C ABI (include/stellar_bh.h): owns the device arena of one
// batch of systems and enqueues the per-step pipeline of bh_device.cuh /
// bh_walk.cuh on the caller's stream, optionally as a replayed CUDA graph.
//
// Replaces BarnesHutParticleSystem (BarnesHutParticleSystem.cpp:28-378):
// allocation in one arena instead of 19 cudaMalloc calls (:54-83), update() as
// bh_step (:301-347) without the per-step event synchronisation (:318).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bh_check.cuh"
#include "bh_engine.h"
#include "bh_render.cuh"
#include "bh_walk.cuh"
#include "stellar_bh.h"

using namespace ssg;

namespace ssg {
thread_local std::string g_last_error;

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return BH_ERR_CUDA;
}
}  // namespace ssg

#define CK(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return ssg::cuda_fail(e_, #call);     \
    } while (0)
// the same for calls that return a status code
#define RC(call)                                                     \
    do {                                                             \
        int rc_ = (call);                                            \
        if (rc_ != BH_OK) return rc_;                                \
    } while (0)

namespace {

constexpr int kWalkWarps = 8;  // accuracy walk: default warps per block
constexpr int kDefaultStack = 768;  // deepest measured: 670 (2D Plummer, N = 2^24)
constexpr int kMaxStack = 2048;
constexpr int kDefaultBucket = 8;
constexpr int kDefaultBpl = 1;  // bodies per lane of the accuracy walk
constexpr int kMaxBucket = 32;
// worst case: 8 warps x (staging + 2048-entry stack + 32-body buckets + slice list)
constexpr int kMaxWalkSmem = 8 * acc_warp_bytes(AccShape{kMaxStack, kMaxBucket, 2}, true);
constexpr int kBboxThreads = 256;
constexpr int kBboxChunk = 2048;

int walk_grid_cap(int device_sms, int blocks_per_sm) { return device_sms * std::max(1, blocks_per_sm); }

// Per-step words: 2 x u64 interaction counts, then bh_system::work (11 ints):
//   work[0..2] walk scheduling, [3..5] walk statistics, [6..8] the energy pass,
//   [9] the sort's run overflow flag, [10] heavy walk groups listed.
// A step's key kernel clears the counts and work[0..5] (kStepZero words), the
// two flags, and the shared walk groups' counters and slice states; the
// energy pass's tree build clears all but the counts and work[0..5].
constexpr int kStepWords = 16;
constexpr int kWorkSortOverflow = 9;
constexpr int kWorkHeavy = 10;
constexpr int kStepFlags = 2;
constexpr int kStepZero = 4 + 6;
// Shared walk groups: pool batches per body (a quarter of the worst case of
// one batch per 32 interactions of every body), slices at most one per two batches.
constexpr int kShareBatchDiv = 4;

// Parts of a step: all of it, or split after the sort (bh_step joins the input
// copies of bh_set_state in between).
enum StepPart { kStepAll = 0, kStepPre = 1, kStepPost = 2 };
constexpr int kGraphs = 6;
constexpr int kGraphCarried = 5;  // a whole step on the box carried from the last walk
constexpr int kTrialSteps = 8;                     // bh_autotune: timed steps per run at most
constexpr size_t kTrialFlushBytes = 256ull << 20;  // bh_autotune: written before each timed step

template <typename T>
T* carve(char*& cur, size_t count) {
    T* p = reinterpret_cast<T*>(cur);
    size_t bytes = (sizeof(T) * count + 255) & ~size_t(255);
    cur += bytes;
    return p;
}

template <typename T>
size_t span(size_t count) {
    return (sizeof(T) * count + 255) & ~size_t(255);
}

}  // namespace

// ------------------------------------------------------------------ walk dispatch

namespace ssg {

// Opt the accuracy walk into the largest shared-memory size it may use, once,
// at creation (never while a graph is being captured).
template <int BPL>
static cudaError_t walk_attributes(int bytes) {
    cudaError_t e = cudaFuncSetAttribute(k_walk_acc<false, false, false, BPL>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_walk_acc<false, false, true, BPL>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_walk_acc<true, false, false, BPL>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_walk_acc<false, true, false, BPL>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_walk_acc<false, false, false, BPL, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_walk_acc<true, false, false, BPL, true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e;
}

cudaError_t init_walk_attributes() {
    cudaError_t e = walk_attributes<1>(kMaxWalkSmem);
    if (e == cudaSuccess) e = walk_attributes<2>(kMaxWalkSmem);
    return e;
}

template <bool MIXED, int BPL>
static cudaError_t launch_acc(const StepArgs& a, cudaStream_t st, int part) {
    const AccShape sh{a.stack, a.bucket, BPL};
    const Groups& gr = BPL == 2 ? a.groups2 : a.groups;
    const int warps = a.warps;
    const size_t smem = (size_t)warps * acc_warp_bytes(sh);
    int grid = std::min(a.walk_grid_acc, (gr.ngroups + warps - 1) / warps);
    if (grid < 1) grid = 1;
    if (part == 0) {
        // bootstrap pass: exits at once unless bh_set_state left the state fresh.  Always
        // 64-body groups: its cost is the traversal, which they halve per body.
        const AccShape sb{a.stack, a.bucket, 2};
        const size_t smb = (size_t)warps * acc_warp_bytes(sb);
        int gb = std::min(a.walk_grid_acc, (a.groups2.ngroups + warps - 1) / warps);
        if (gb < 1) gb = 1;
        return launch_pdl(k_walk_acc<false, true, false, 2>, gb, warps * 32, smb, st, sb, a.segs,
                          a.groups2, a.in, a.recA, a.recB, a.recC, a.recD, a.eps2, a.G, a.dt,
                          a.ddt, a.alpha, a.out, a.status, a.inter, a.work + 1, a.fresh,
                          a.max_stack, (double*)nullptr, Frontier{}, Heavy{}, Share{});
    } else if (a.share.ctr) {
        // shared groups; the pool holds sums for one or two bodies per lane: half
        // the batches with two
        Share shr = a.share;
        shr.cap_batches /= BPL;
        shr.cap_slices = std::min(shr.cap_slices, shr.cap_batches);
        return launch_pdl(k_walk_acc<MIXED, false, false, BPL, true>, grid, warps * 32,
                          (size_t)warps * acc_warp_bytes(sh, true), st, sh, a.segs, gr, a.in,
                          a.recA, a.recB, a.recC, a.recD, a.eps2, a.G, a.dt, a.ddt, a.alpha,
                          a.out, a.status, a.inter, a.work + 2, a.fresh, a.max_stack,
                          (double*)nullptr, a.frontier, a.heavy, shr);
    } else {
        return launch_pdl(k_walk_acc<MIXED, false, false, BPL>, grid, warps * 32, smem, st, sh,
                          a.segs, gr, a.in, a.recA, a.recB, a.recC, a.recD, a.eps2, a.G, a.dt,
                          a.ddt, a.alpha, a.out, a.status, a.inter, a.work + 2, a.fresh,
                          a.max_stack, (double*)nullptr, a.frontier, a.heavy, Share{});
    }
}

// part 0: the accuracy modes' bootstrap pass (nothing in REFERENCE mode);
// part 1: the walk.
cudaError_t launch_walk(const StepArgs& a, cudaStream_t st, int part) {
    if (a.mode == BH_MODE_REFERENCE) {
        if (part == 0) return cudaSuccess;
        int grid = std::min(a.walk_grid_ref, (a.groups.ngroups + kVoteWarps - 1) / kVoteWarps);
        if (grid < 1) grid = 1;
        return launch_pdl(k_walk_vote, grid, kVoteWarps * 32, 0, st, a.segs, a.groups, a.in, a.recA,
                          a.recC, a.eps2, a.dt, a.ddt, a.out, a.status, a.inter, a.work, a.frontier);
    }
    if (a.bpl == 2)
        return a.mode == BH_MODE_MIXED ? launch_acc<true, 2>(a, st, part)
                                       : launch_acc<false, 2>(a, st, part);
    return a.mode == BH_MODE_MIXED ? launch_acc<true, 1>(a, st, part)
                                   : launch_acc<false, 1>(a, st, part);
}

int normalized_bucket(int b) { return b <= 0 ? kDefaultBucket : std::min(b, kMaxBucket); }
int normalized_stack(int s) { return s <= 0 ? kDefaultStack : std::max(64, std::min(s, kMaxStack)); }
int normalized_bpl(int b) { return b == 2 ? 2 : (b <= 0 ? kDefaultBpl : 1); }
int normalized_warps(int block) {
    int w = block <= 0 ? kWalkWarps : block / 32;
    return std::max(1, std::min(w, 8));
}

}  // namespace ssg

// ------------------------------------------------------------------ bh_system

struct bh_system {
    bh_params p{};
    int n = 0;
    int device = 0;
    int sms = 0;
    int nseg = 1;
    std::vector<int> h_off;

    char* arena = nullptr;
    size_t arena_bytes = 0;

    // state: [0] current (key order of the last step), [1] scratch / gathered
    BodyPtrs st[2]{};
    uint64_t *keys = nullptr, *keys_alt = nullptr, *keys3 = nullptr;  // keys3: third sort buffer
    uint32_t *vals = nullptr, *vals_alt = nullptr, *vals3 = nullptr;
    uint64_t* kfinal = nullptr;  // sorted keys after the last pass
    uint32_t* vfinal = nullptr;  // permutation after the last pass
    uint32_t *hist = nullptr, *totals = nullptr;
    int tiles = 0;
    int* box_next = nullptr;  // [4 nseg] the next step's box, folded by the integrating walk
    bool box_valid = false;   // box_next is the box of the current positions (host's record)
    int* box_ord = nullptr;
    int *seg_off = nullptr, *seg_of_pos = nullptr, *gseg_off = nullptr, *gseg_off2 = nullptr;
    int *chunk_seg = nullptr, *chunk_begin = nullptr, *chunk_end = nullptr;
    int nchunks = 0;
    int ngroups = 0, ngroups2 = 0;  // groups of 32 and of 64 bodies
    int nsupers = 0;                // walk super-groups (frontiers), all systems
    int* sup_off = nullptr;         // [nseg+1] first super-group of each system
    TreePtrs tree{};
    int* counter = nullptr;
    NodeSums sums{};
    Records rec{};
    float *ax = nullptr, *ay = nullptr;
    int* status = nullptr;
    unsigned long long* inter = nullptr;
    int* work = nullptr;   // 3 scheduling counters, walk stack peak, rounds, tests; reset every step
                           // [6..8]: scratch of bh_energy
    double* diag = nullptr;  // bh_energy: 4 sums per system
    int* fresh = nullptr;  // 1 after bh_set_state: bootstrap |a_old| in the next step
    int* flist = nullptr;   // walk frontiers, kFrontierCap per super-group
    int* heavy = nullptr;   // heavy walk groups of the step (k_frontier)
    // shared walk groups: the batch pool (entries, and sums for one body per
    // lane: half as many batches with two) and the slice table
    int* share_idx = nullptr;
    float2* share_sum = nullptr;
    int* share_ctr = nullptr;    // [kCtrWords] counters, then the slice states
    int* share_state = nullptr;
    int4* share_desc = nullptr;
    int share_batches = 0, share_slices = 0;
    unsigned long long* seg_cost = nullptr;  // [nseg] walk cost of each system, this step
    int* mean_cost = nullptr;                // [nseg] mean walk-group cost, last step
    int2* fcount = nullptr;  // per super-group: (nodes to test, accepted cells); -1: the root
    bool fresh_host = false;  // the host's record of *fresh: the bootstrap pass is launched
                              // only in steps that follow bh_set_state
    int seg_passes = 0;
    int high_passes = 4;  // radix passes of the sort's fast path (k_sort_fixup)

    int walk_grid_ref = 0, walk_grid_acc = 0;
    int walk_warps_resident = 0;  // accuracy walk warps resident at once (default shape)
    bool have_state = false;
    bool caller_order = false;  // true from bh_set_state until the next step

    uint32_t* image = nullptr;  // bh_render: per-pixel counts, then RGBA8
    size_t image_pixels = 0;

    // energy log: FP64 diagnostics after every `energy_every`-th bh_step
    int energy_every = 0, energy_cap = 0;
    long long energy_steps = 0;     // steps since bh_set_energy_log
    double* elog = nullptr;         // [energy_cap][4 * nseg] ring
    int* elog_count = nullptr;      // records written (device)
    cudaGraph_t egraph = nullptr;   // captured diagnostics pass (graph mode)
    cudaGraphExec_t egraph_exec = nullptr;

    cudaStream_t cap_stream = nullptr;
    cudaStream_t cond_stream = nullptr;  // captures the body of the sort's conditional node
    // a graph branch beside the tree build: the reorder (captures only)
    cudaStream_t fork_stream = nullptr;
    cudaEvent_t fork_event = nullptr, join_event = nullptr;
    // Step graphs: [0] / [1] one step without / with the bootstrap pass; [2] the
    // step up to the sort; [3] / [4] the rest, without / with the bootstrap pass
    // (the first step after bh_set_state: the input copies join in between).
    cudaGraph_t graph[kGraphs] = {};
    cudaGraphExec_t graph_exec[kGraphs] = {};

    // Input copies that no kernel before the reorder reads (vx, vy, mass; the
    // accelerations of bh_set_accel) run on copy_stream, overlapped with the
    // next step's box, keys and sort; in_event marks their end.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t in_event = nullptr;
    cudaEvent_t order_event = nullptr;  // `stream`'s work before a copy_stream copy
    bool in_pending = false;            // copies on copy_stream that no step has joined yet
};

namespace {

void drop_graph(bh_system* s) {
    for (int b = 0; b < kGraphs; ++b) {
        if (s->graph_exec[b]) cudaGraphExecDestroy(s->graph_exec[b]);
        if (s->graph[b]) cudaGraphDestroy(s->graph[b]);
        s->graph_exec[b] = nullptr;
        s->graph[b] = nullptr;
    }
    if (s->egraph_exec) cudaGraphExecDestroy(s->egraph_exec);
    if (s->egraph) cudaGraphDestroy(s->egraph);
    s->egraph_exec = nullptr;
    s->egraph = nullptr;
}

bool params_ok(const bh_params* p) {
    if (!p) return false;
    if (p->mode < BH_MODE_REFERENCE || p->mode > BH_MODE_MIXED) return false;
    if (!(p->theta > 0.0f) || !(p->eps2 >= 0.0f)) return false;
    if (p->mode == BH_MODE_REFERENCE && !(p->eps2 > 0.0f)) return false;
    return true;
}

ssg::StepArgs step_args(bh_system* s) {
    ssg::StepArgs a{};
    a.mode = s->p.mode;
    a.segs = Segs{s->nseg, s->seg_off, s->nseg > 1 ? s->seg_of_pos : nullptr};
    a.groups = Groups{s->ngroups, s->nseg > 1 ? s->gseg_off : nullptr};
    a.groups2 = Groups{s->ngroups2, s->nseg > 1 ? s->gseg_off2 : nullptr};
    const BodyPtrs& g = s->st[1];
    const BodyPtrs& c = s->st[0];
    bool mixed = s->p.mode == BH_MODE_MIXED;
    a.in = WalkIn{g.x, g.y, g.vx, g.vy, g.m, mixed ? g.xlo : nullptr, mixed ? g.ylo : nullptr, g.id,
                  g.amag, g.gcost};
    a.out = WalkOut{c.x, c.y, c.vx, c.vy, c.m, mixed ? c.xlo : nullptr, mixed ? c.ylo : nullptr, c.id,
                    s->ax, s->ay, c.amag, c.gcost, s->box_next};
    a.recA = s->rec.A;
    a.recB = s->rec.B;
    a.recC = s->rec.C;
    a.recD = s->rec.D;
    a.eps2 = s->p.eps2;
    a.G = s->p.gravity;
    a.dt = s->p.timestep;
    a.ddt = s->p.dampening * s->p.timestep;  // kernels.cu:532: d*dt, in float
    a.alpha = s->p.alpha;
    a.status = s->status;
    a.inter = s->inter;
    a.work = s->work;
    a.fresh = s->fresh;
    a.max_stack = s->work + 3;
    a.bucket = normalized_bucket(s->p.leaf_bucket);
    a.stack = normalized_stack(s->p.stack_depth);
    a.bpl = normalized_bpl(s->p.bodies_per_lane);
    a.warps = normalized_warps(s->p.block_size);
    a.walk_grid_ref = s->walk_grid_ref;
    a.walk_grid_acc = s->walk_grid_acc;
    // shared walk starts: super-groups of 512 bodies counted from each system's start
    a.frontier = Frontier{s->flist, s->fcount, s->nseg > 1 ? s->sup_off : nullptr};
    a.heavy = Heavy{s->heavy, s->work + kWorkHeavy, s->mean_cost, s->seg_cost};
    // Shared walk groups.  share_tail > 0: the heavy groups and the last
    // share_tail groups handed out; 0 (default): the heavy groups, when the walk
    // has no more groups than the GPU has resident walk warps (measured faster
    // there, slower above); -1: none.
    const int ng = a.bpl == 2 ? s->ngroups2 : s->ngroups;
    if (s->p.share_tail > 0 || (s->p.share_tail == 0 && ng <= s->walk_warps_resident))
        a.share = Share{s->share_ctr, s->share_state, s->share_desc, s->share_idx, s->share_sum,
                        s->share_batches, s->share_slices, std::min(std::max(s->p.share_tail, 0), ng)};
    return a;
}

// Phases 0-3 of a step: box, keys, sort.  The sorted keys and permutation end
// in keys_alt / vals_alt, or in keys3 / vals3 after an odd number of
// system-index passes.  carry: the box is the one the last walk folded
// (box_next), no box kernel.  fold: this step's walk folds the next box, so
// box_next is reset once the keys are made.
int enqueue_sort(bh_system* s, cudaStream_t st, cudaEvent_t* ev, bool keep_stats, bool carry,
                 bool fold) {
    const int n = s->n;
    auto mark = [&](int k) -> cudaError_t { return ev ? cudaEventRecord(ev[k], st) : cudaSuccess; };
    Segs segs{s->nseg, s->seg_off, s->nseg > 1 ? s->seg_of_pos : nullptr};
    const BodyPtrs& cur = s->st[0];
    const int tb = 256, nb = (n + tb - 1) / tb;
    uint64_t *k0 = s->keys, *kA = s->keys_alt, *kB = s->keys3;
    uint32_t *v0 = s->vals, *vA = s->vals_alt, *vB = s->vals3;
    if (!carry) CK(cudaMemsetAsync(s->box_ord, 0, sizeof(int) * 4 * s->nseg, st));  // origin box
    CK(mark(0));
    if (!carry)
        CK(launch_pdl(k_bbox<kBboxThreads>, s->nchunks, kBboxThreads, 0, st, cur.x, cur.y,
                      s->chunk_seg, s->chunk_begin, s->chunk_end, s->box_ord, s->status));
    CK(mark(1));
    // keys and positions; the moments counters and the step's words cleared
    CK(launch_pdl(k_keys_step, nb, tb, 0, st, cur.x, cur.y, n, segs,
                  carry ? (const int*)s->box_next : (const int*)s->box_ord, s->keys, s->vals,
                  s->counter, reinterpret_cast<int*>(s->inter), keep_stats ? 0 : kStepZero,
                  s->work + kWorkSortOverflow, kStepFlags, s->share_ctr, kCtrWords + s->share_slices,
                  s->seg_cost, s->mean_cost, carry ? s->box_ord : (int*)nullptr));
    CK(mark(2));

    // Sort (stable, by key, then by system): LSD passes over the key's top
    // 8 * high_passes bits (the high word), then k_sort_fixup orders each run
    // of equal high words by the whole key.  A run longer than kFixupRun
    // (bodies packed into one 2^-12 or 2^-16 box cell) makes the step take
    // the full 8-pass sort from the original keys: in a
    // graph behind a conditional node that only the fixup switches on, in
    // stream order as kernels that return at once unless the flag is set.
    int* overflow = s->work + kWorkSortOverflow;
    auto pass = [&](auto launch, cudaStream_t q, const uint64_t* ki, const uint32_t* vi, uint64_t* ko,
                    uint32_t* vo, int shift, int use_seg, const int* only_if) -> cudaError_t {
        cudaError_t e = launch(k_radix_hist, s->tiles, kSortThreads, 0, q, ki, vi, n, shift, use_seg,
                               s->seg_of_pos, s->hist, s->tiles, only_if);
        if (e == cudaSuccess)
            e = launch(k_radix_scan, 256, kSortThreads, 0, q, s->hist, s->tiles, s->totals, only_if);
        if (e == cudaSuccess)
            e = launch(k_radix_scatter, s->tiles, kSortThreads, 0, q, ki, vi, ko, vo, n, shift, use_seg,
                       s->seg_of_pos, s->hist, s->totals, s->tiles, only_if);
        return e;
    };
    auto pdl = [](auto... a) { return launch_pdl(a...); };
    auto plain = [](auto... a) { return launch_plain(a...); };
    // the full sort: k0 -> kB -> kA -> ... -> kA (8 passes)
    auto full_sort = [&](auto launch, cudaStream_t q, const int* only_if) -> cudaError_t {
        const uint64_t* ki = k0;
        const uint32_t* vi = v0;
        for (int ps = 0; ps < 8; ++ps) {
            uint64_t* ko = (ps & 1) ? kA : kB;
            uint32_t* vo = (ps & 1) ? vA : vB;
            cudaError_t e = pass(launch, q, ki, vi, ko, vo, 8 * ps, 0, only_if);
            if (e != cudaSuccess) return e;
            ki = ko;
            vi = vo;
        }
        return cudaSuccess;
    };
    cudaStreamCaptureStatus cstat = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cstat));
    const bool capturing = cstat == cudaStreamCaptureStatusActive;
    cudaGraph_t cgraph = nullptr;
    cudaGraphConditionalHandle cond = 0;
    if (capturing) {
        CK(cudaStreamGetCaptureInfo(st, &cstat, nullptr, &cgraph, nullptr, nullptr, nullptr));
        CK(cudaGraphConditionalHandleCreate(&cond, cgraph, 0, cudaGraphCondAssignDefault));
    }
    // high words: k0 -> ... -> kB (the last pass writes kB, the fixup kA)
    {
        const uint64_t* ki = k0;
        const uint32_t* vi = v0;
        for (int ps = 0; ps < s->high_passes; ++ps) {
            const bool to_a = ((s->high_passes - 1 - ps) & 1) != 0;
            uint64_t* ko = to_a ? kA : kB;
            uint32_t* vo = to_a ? vA : vB;
            CK(pass(pdl, st, ki, vi, ko, vo, 64 - 8 * (s->high_passes - ps), 0, nullptr));
            ki = ko;
            vi = vo;
        }
    }
    // the fixup also resets box_next for this step's walk (fold)
    CK(launch_pdl(k_sort_fixup, nb, tb, 0, st, n, 64 - 8 * s->high_passes, kB, vB, kA, vA, overflow,
                  cond, capturing ? 1 : 0, fold ? s->box_next : (int*)nullptr, 4 * s->nseg));
    if (capturing) {
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        CK(cudaStreamGetCaptureInfo(st, &cstat, nullptr, &cgraph, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode = nullptr;
        CK(cudaGraphAddNode(&cnode, cgraph, deps, nullptr, ndeps, &cp));
        CK(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
        if (!s->cond_stream) return BH_ERR_STATE;  // created before the capture began
        CK(cudaStreamBeginCaptureToGraph(s->cond_stream, cp.conditional.phGraph_out[0], nullptr,
                                         nullptr, 0, cudaStreamCaptureModeRelaxed));
        cudaError_t e = full_sort(plain, s->cond_stream, nullptr);
        cudaGraph_t body = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(s->cond_stream, &body);
        if (e != cudaSuccess) return cuda_fail(e, "conditional sort body");
        if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture (sort body)");
    } else {
        // stream order: one cooperative kernel that returns at once unless the
        // fixup set the flag (the 24 flag-gated kernels where none can be formed)
        cudaError_t e = cudaSuccess;
        if (!launch_full_sort_grid(k0, v0, kA, vA, kB, vB, n, s->hist, s->totals, s->tiles, overflow,
                                   st, &e))
            e = full_sort(pdl, st, overflow);
        CK(e);
    }
    uint64_t *ka = kA, *kb = kB;
    uint32_t *va = vA, *vb = vB;
    for (int ps = 0; ps < s->seg_passes; ++ps) {  // then the system index
        CK(pass(pdl, st, ka, va, kb, vb, 8 * ps, 1, nullptr));
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    CK(mark(3));
    return BH_OK;
}

// Box, keys, sort, reorder, tree, moments and walk records of the current
// state (phases 0-5; the walk records in the accuracy layout when `accuracy`).
// ev (optional): events recorded at the phase boundaries.  keep_stats: leave
// the last step's interaction counts and walk statistics (the energy pass).
// part: kStepPre stops after the sort, kStepPost starts at the reorder.
// carry, fold: see enqueue_sort.
int enqueue_front(bh_system* s, cudaStream_t st, bool accuracy, cudaEvent_t* ev,
                  bool keep_stats = false, int part = kStepAll, bool carry = false,
                  bool fold = false) {
    const int n = s->n;
    auto mark = [&](int k) -> cudaError_t { return ev ? cudaEventRecord(ev[k], st) : cudaSuccess; };
    const bool mixed = s->p.mode == BH_MODE_MIXED;
    Segs segs{s->nseg, s->seg_off, s->nseg > 1 ? s->seg_of_pos : nullptr};
    const BodyPtrs& cur = s->st[0];
    const int tb = 256, nb = (n + tb - 1) / tb;
    if (part != kStepPost) {
        int rc = enqueue_sort(s, st, ev, keep_stats, carry, fold);
        if (rc != BH_OK) return rc;
    }
    // the sorted keys and permutation: in kA after the fixup, moved by each
    // system-index pass
    uint64_t* ka = (s->seg_passes & 1) ? s->keys3 : s->keys_alt;
    uint32_t* va = (s->seg_passes & 1) ? s->vals3 : s->vals_alt;
    s->kfinal = ka;
    s->vfinal = va;
    if (part == kStepPre) return BH_OK;

    BodyPtrs src = cur, dst = s->st[1];
    if (!mixed) {
        src.xlo = src.ylo = nullptr;
        dst.xlo = dst.ylo = nullptr;
    }
    if (!accuracy) {
        src.amag = dst.amag = nullptr;
        src.gcost = dst.gcost = nullptr;
    }
    // The reorder and the tree build both start from the sort and write
    // disjoint arrays; in a graph they are two branches that run side by side
    // (the build is instruction-bound, the reorder waits on memory).
    cudaStreamCaptureStatus cstat = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cstat));
    const bool fork = cstat == cudaStreamCaptureStatusActive && s->fork_stream;
    if (fork) {
        CK(cudaEventRecord(s->fork_event, st));
        CK(cudaStreamWaitEvent(s->fork_stream, s->fork_event, 0));
        CK(launch_plain(k_gather, nb, tb, 0, s->fork_stream, n, va, src, dst));
        CK(cudaEventRecord(s->join_event, s->fork_stream));
    } else {
        CK(launch_pdl(k_gather, nb, tb, 0, st, n, va, src, dst));
    }
    CK(mark(4));
    CK(launch_pdl(k_build, nb, tb, 0, st, ka, n, segs, s->tree, s->status));
    if (fork) CK(cudaStreamWaitEvent(st, s->join_event, 0));
    CK(mark(5));
    CK(launch_pdl(k_moments, (n + kMomentsThreads - 1) / kMomentsThreads, kMomentsThreads, 0, st, n,
                  accuracy ? 1 : 0, dst.x, dst.y, dst.m, s->tree.climb, s->tree.leaf_parent,
                  s->counter, s->sums, s->status));
    CK(launch_pdl(k_records, nb, tb, 0, st, n, segs, accuracy ? 1 : 0, s->p.theta, s->p.gravity,
                  s->box_ord, ka, s->tree, s->sums, s->rec));
    CK(cudaGetLastError());
    CK(mark(6));
    return BH_OK;
}

// One step: the front half, then the bootstrap pass (accuracy modes, fresh
// state only) and the walk fused with the integration (phases 6-7).
// boot < 0: the bootstrap pass is launched iff bh_set_state came since the last
// step (the host's record, cleared here); 0 / 1: left out / launched (graph capture).
// carry < 0: a whole step takes the box folded by the last walk iff the host's
// record says it is the box of the current positions; 0 / 1: box kernel /
// carried (graph capture).  The walk folds the next step's box.  The host's
// record is updated here for steps enqueued outside a capture, and by bh_step
// for graph launches.
int enqueue_step(bh_system* s, cudaStream_t st, cudaEvent_t* ev = nullptr, int boot = -1,
                 int part = kStepAll, int carry = -1) {
    auto mark = [&](int k) -> cudaError_t { return ev ? cudaEventRecord(ev[k], st) : cudaSuccess; };
    const bool carried = carry < 0 ? (part == kStepAll && s->box_valid) : carry > 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cap));
    const bool capturing = cap == cudaStreamCaptureStatusActive;
    int rc = enqueue_front(s, st, s->p.mode != BH_MODE_REFERENCE, ev, false, part, carried, true);
    if (rc != BH_OK) return rc;
    if (!capturing) s->box_valid = false;  // box_next is reset by this step's sort
    if (part == kStepPre) return rc;
    const bool with_boot = boot < 0 ? s->fresh_host : boot > 0;
    if (boot < 0) s->fresh_host = false;
    StepArgs a = step_args(s);
    if (with_boot) CK(launch_walk(a, st, 0));
    CK(mark(7));
    constexpr int kFW = 8;  // warps (super-groups) per block
    const int fblocks = (s->nsupers + kFW - 1) / kFW;
    if (a.mode != BH_MODE_REFERENCE) {
        CK(launch_pdl(k_frontier<kFW>, fblocks, kFW * 32, 0, st, a.segs, s->nsupers, a.in.x, a.in.y,
                      a.in.amag, a.recA, a.recC, a.recD, a.bucket, 32 * a.bpl, a.alpha, s->flist,
                      s->fcount, a.frontier.sup_off, a.in.gcost,
                      s->nseg > 1 ? (a.bpl == 2 ? s->gseg_off2 : s->gseg_off) : nullptr,
                      s->mean_cost, s->heavy, s->work + kWorkHeavy, a.eps2));
    } else {
        // the reference rule's frontiers (leaves hold one body: bucket 1)
        CK(launch_pdl(k_frontier<kFW, true>, fblocks, kFW * 32, 0, st, a.segs, s->nsupers, a.in.x,
                      a.in.y, (const float*)nullptr, a.recA, a.recC, a.recD, 1, 32, 0.0f, s->flist,
                      s->fcount, a.frontier.sup_off, (const int*)nullptr, (const int*)nullptr,
                      (const int*)nullptr, (int*)nullptr, (int*)nullptr, a.eps2));
    }
    CK(mark(8));
    CK(launch_walk(a, st, 1));
    CK(mark(9));
    if (!capturing) s->box_valid = true;
    return BH_OK;
}

// FP32 FMA throughput probe: 8 independent FMA chains per thread, no memory
// traffic except one store per thread (kept so the chains are not removed).
// 128 FMAs (256 flops) per thread and iteration.
__global__ void __launch_bounds__(256) k_ffma_peak(float* out, int iters, float a, float b) {
    float v0 = threadIdx.x * 1e-3f, v1 = v0 + 1.f, v2 = v0 + 2.f, v3 = v0 + 3.f;
    float v4 = v0 + 4.f, v5 = v0 + 5.f, v6 = v0 + 6.f, v7 = v0 + 7.f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            v0 = fmaf(v0, a, b); v1 = fmaf(v1, a, b); v2 = fmaf(v2, a, b); v3 = fmaf(v3, a, b);
            v4 = fmaf(v4, a, b); v5 = fmaf(v5, a, b); v6 = fmaf(v6, a, b); v7 = fmaf(v7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7;
}

// The same with packed FP32x2 FMAs (__ffma2_rn, the force walk's instruction):
// 8 independent chains of float2, 64 FFMA2 = 128 FMAs (256 flops) per thread
// and iteration.
__global__ void __launch_bounds__(256) k_ffma2_peak(float* out, int iters, float a, float b) {
    const float s = threadIdx.x * 1e-3f;
    float2 v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = make_float2(s + c, s + c + 0.5f);
    const float2 av = make_float2(a, a), bv = make_float2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
#pragma unroll
            for (int c = 0; c < 8; ++c) v[c] = __ffma2_rn(v[c], av, bv);
        }
    }
    float acc = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) acc += v[c].x + v[c].y;
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// FP64 direct sum for a sample of targets: grid (target tiles, source chunks),
// partial sums per chunk, reduced in a fixed order by k_direct_reduce.
constexpr int kDirThreads = 256;
constexpr int kDirChunks = 64;

__global__ void __launch_bounds__(kDirThreads) k_direct_partial(
    int n, const float* __restrict__ xh, const float* __restrict__ xl, const float* __restrict__ yh,
    const float* __restrict__ yl, const float* __restrict__ m, int ns, const int* __restrict__ idx,
    double eps2, double* __restrict__ part) {
    __shared__ double sx[kDirThreads], sy[kDirThreads], sm[kDirThreads];
    __shared__ int sid[kDirThreads];
    const int t = blockIdx.x * kDirThreads + threadIdx.x;
    const bool active = t < ns;
    const int ti = active ? idx[t] : -1;
    const double px = active ? (double)xh[ti] + (xl ? (double)xl[ti] : 0.0) : 0.0;
    const double py = active ? (double)yh[ti] + (yl ? (double)yl[ti] : 0.0) : 0.0;
    const int per = (n + gridDim.y - 1) / gridDim.y;
    const int beg = blockIdx.y * per, end = min(n, beg + per);
    double ax = 0.0, ay = 0.0;
    for (int base = beg; base < end; base += kDirThreads) {
        int j = base + threadIdx.x;
        __syncthreads();
        if (j < end) {
            sx[threadIdx.x] = (double)xh[j] + (xl ? (double)xl[j] : 0.0);
            sy[threadIdx.x] = (double)yh[j] + (yl ? (double)yl[j] : 0.0);
            sm[threadIdx.x] = m[j];
            sid[threadIdx.x] = j;
        } else {
            sid[threadIdx.x] = -1;
        }
        __syncthreads();
        const int cnt = min(kDirThreads, end - base);
        if (active) {
            for (int k = 0; k < cnt; ++k) {
                if (sid[k] == ti) continue;
                double dx = sx[k] - px, dy = sy[k] - py;
                double r2 = dx * dx + dy * dy + eps2;
                double inv = 1.0 / (r2 * sqrt(r2));
                ax += sm[k] * dx * inv;
                ay += sm[k] * dy * inv;
            }
        }
    }
    if (active) {
        part[(size_t)blockIdx.y * 2 * ns + t] = ax;
        part[(size_t)blockIdx.y * 2 * ns + ns + t] = ay;
    }
}

__global__ void k_direct_reduce(int ns, int chunks, const double* __restrict__ part, double G,
                                double* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * ns) return;
    double acc = 0.0;
    for (int c = 0; c < chunks; ++c) acc += part[(size_t)c * 2 * ns + t];
    out[t] = G * acc;
}

// The stream and events of the reorder's graph branch (created before a capture).
int make_fork_stream(bh_system* s) {
    if (s->fork_stream) return BH_OK;
    CK(cudaStreamCreateWithFlags(&s->fork_stream, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&s->fork_event, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&s->join_event, cudaEventDisableTiming));
    return BH_OK;
}

// The copy stream starts its next copy after the work enqueued on `st` so far.
int copy_stream_after(bh_system* s, cudaStream_t st) {
    if (!s->copy_stream) {
        CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&s->in_event, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&s->order_event, cudaEventDisableTiming));
    }
    CK(cudaEventRecord(s->order_event, st));
    CK(cudaStreamWaitEvent(s->copy_stream, s->order_event, 0));
    return BH_OK;
}

// The input copies still on the copy stream come before `st`'s next work.
int join_inputs(bh_system* s, cudaStream_t st) {
    if (!s->in_pending) return BH_OK;
    CK(cudaStreamWaitEvent(st, s->in_event, 0));
    s->in_pending = false;
    return BH_OK;
}

// The same for calls without a stream: the host waits for the copies.
int settle_inputs(bh_system* s) {
    if (!s->in_pending) return BH_OK;
    CK(cudaStreamSynchronize(s->copy_stream));
    s->in_pending = false;
    return BH_OK;
}

// Capture of graph slot `slot` (see bh_system::graph).
int build_graph(bh_system* s, int slot) {
    if (!s->cap_stream) CK(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
    if (!s->cond_stream) CK(cudaStreamCreateWithFlags(&s->cond_stream, cudaStreamNonBlocking));
    RC(make_fork_stream(s));
    const int part = (slot < 2 || slot == kGraphCarried) ? kStepAll : slot == 2 ? kStepPre : kStepPost;
    const int boot = (slot == 1 || slot == 4) ? 1 : 0;
    CK(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_step(s, s->cap_stream, nullptr, boot, part, slot == kGraphCarried ? 1 : 0);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
    if (st != BH_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    s->graph[slot] = g;
    CK(cudaGraphInstantiate(&s->graph_exec[slot], g, 0));
    return BH_OK;
}

// State of a freshly loaded system: caller order, zero position tails and
// accelerations, status cleared, bootstrap pass requested.
// The previous state's walk-group costs in caller order: kept[id[i]] = gcost[i].
// They only order the walk's groups (heaviest first), never change a result,
// so a state that continues the previous one keeps its schedule.
__global__ void k_keep_cost(int n, const int* __restrict__ id, const int* __restrict__ gcost,
                            int* __restrict__ kept) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) kept[id[i]] = gcost[i];
}

// kept: costs from k_keep_cost, or NULL for none (every group of equal weight)
__global__ void k_state_init(int n, int* id, float* xlo, float* ylo, float* ax, float* ay,
                             float* amag, int* gcost, const int* kept, int* fresh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        id[i] = i;
        xlo[i] = 0.0f;
        ylo[i] = 0.0f;
        ax[i] = 0.0f;
        ay[i] = 0.0f;
        amag[i] = 0.0f;
        gcost[i] = kept ? kept[i] : 0;
    }
    if (i == 0) *fresh = 1;
}

// out[id[j]] = in[j] for up to four arrays
__global__ void k_scatter4(int n, const int* __restrict__ id, const float* a0, const float* a1,
                           const float* a2, const float* a3, float* o0, float* o1, float* o2,
                           float* o3) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int i = id[j];
    if (a0) o0[i] = a0[j];
    if (a1) o1[i] = a1[j];
    if (a2) o2[i] = a2[j];
    if (a3) o3[i] = a3[j];
}

int status_code(int bits, int mode) {
    if (bits & ST_NONFINITE) return BH_ERR_NONFINITE;
    if ((bits & ST_DUP) && mode == BH_MODE_REFERENCE) return BH_ERR_DUPLICATE_KEYS;
    if (bits & ST_STACK) return BH_ERR_STACK;
    if (bits & ST_CAPACITY) return BH_ERR_CAPACITY;
    if (bits & ST_TREE) return BH_ERR_TREE;
    return BH_OK;
}

}  // namespace

namespace ssg {

int system_create(const bh_params* p, const int* sizes, int nseg, int device, bh_system** out) {
    if (!out || !params_ok(p) || nseg < 1 || !sizes) return BH_ERR_ARG;
    *out = nullptr;
    long long total = 0;
    for (int i = 0; i < nseg; ++i) {
        if (sizes[i] < 1) return BH_ERR_ARG;
        total += sizes[i];
    }
    if (total > (1ll << 30)) return BH_ERR_CAPACITY;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        g_last_error = "no CUDA device";
        return BH_ERR_NO_DEVICE;
    }
    if (device < 0) CK(cudaGetDevice(&device));
    CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) {
        g_last_error = "device is not Blackwell (sm_103a build)";
        return BH_ERR_NO_DEVICE;
    }

    bh_system* s = new bh_system();
    s->p = *p;
    s->n = (int)total;
    s->device = device;
    s->sms = prop.multiProcessorCount;
    s->nseg = nseg;
    s->h_off.resize(nseg + 1);
    s->h_off[0] = 0;
    for (int i = 0; i < nseg; ++i) s->h_off[i + 1] = s->h_off[i] + sizes[i];
    const size_t N = (size_t)s->n;
    s->tiles = (int)((N + kSortTile - 1) / kSortTile);
    s->seg_passes = nseg == 1 ? 0 : (nseg <= 256 ? 1 : 2);
    s->high_passes = *std::max_element(sizes, sizes + nseg) <= kShortSortMax ? 3 : 4;

    // chunk table for the box reduction and group table for the walks
    std::vector<int> cseg, cbeg, cend, goff(nseg + 1, 0), goff2(nseg + 1, 0), soff(nseg + 1, 0);
    for (int sg = 0; sg < nseg; ++sg) {
        for (int b = s->h_off[sg]; b < s->h_off[sg + 1]; b += kBboxChunk) {
            cseg.push_back(sg);
            cbeg.push_back(b);
            cend.push_back(std::min(b + kBboxChunk, s->h_off[sg + 1]));
        }
        goff[sg + 1] = goff[sg] + (sizes[sg] + 31) / 32;
        goff2[sg + 1] = goff2[sg] + (sizes[sg] + 63) / 64;
        soff[sg + 1] = soff[sg] + num_supers(sizes[sg]);
    }
    s->nchunks = (int)cseg.size();
    s->ngroups = goff[nseg];
    s->ngroups2 = goff2[nseg];
    s->nsupers = soff[nseg];

    size_t bytes = 0;
    bytes += 2 * (8 * span<float>(N) + 2 * span<int>(N));
    bytes += 3 * span<uint64_t>(N) + 3 * span<uint32_t>(N);
    bytes += span<uint32_t>((size_t)256 * s->tiles) + span<uint32_t>(256);
    bytes += span<int>(4 * (size_t)nseg);
    bytes += span<int>(4 * (size_t)nseg) + 3 * span<int>(nseg + 1) + span<int>(N);
    bytes += 3 * span<int>(s->nchunks);
    bytes += 8 * span<int>(N) + span<int4>(N);                  // tree arrays, counter, climb
    bytes += 2 * span<float4>(N);                               // node sums
    bytes += 2 * span<float4>(N) + 2 * span<int4>(N);           // walk records
    bytes += 2 * span<float>(N) + span<int>(1) + span<int>(kStepWords) +
             span<double>(4 * (size_t)nseg) + span<int>(1);
    bytes += span<int>((size_t)s->nsupers * kFrontierCap) + span<int2>((size_t)s->nsupers) +
             span<int>(nseg + 1) + span<int>((size_t)s->ngroups) +
             span<unsigned long long>(nseg) + span<int>(nseg);
    // (below 2^27: the walk's slice list packs a first batch times 16 in an int)
    s->share_batches = (int)std::max<size_t>(64, std::min<size_t>(N / kShareBatchDiv, 1u << 26));
    // the key kernel's threads (n rounded up to 256) clear the counters and slice states
    s->share_slices = std::min((int)((N + 255) / 256 * 256) - kCtrWords, s->share_batches / 2);
    bytes += span<int>((size_t)s->share_batches * 32) + span<float2>((size_t)s->share_batches * 32) +
             span<int>(kCtrWords + (size_t)s->share_slices) + span<int4>((size_t)s->share_slices);
    cudaError_t e = cudaMalloc(&s->arena, bytes);
    if (e != cudaSuccess) {
        cuda_fail(e, "cudaMalloc(arena)");
        delete s;
        return BH_ERR_NOMEM;
    }
    s->arena_bytes = bytes;
    char* c = s->arena;
    for (int k = 0; k < 2; ++k) {
        BodyPtrs& b = s->st[k];
        b.x = carve<float>(c, N);
        b.y = carve<float>(c, N);
        b.vx = carve<float>(c, N);
        b.vy = carve<float>(c, N);
        b.m = carve<float>(c, N);
        b.xlo = carve<float>(c, N);
        b.ylo = carve<float>(c, N);
        b.id = carve<int>(c, N);
        b.amag = carve<float>(c, N);
        b.gcost = carve<int>(c, N);
    }
    s->keys = carve<uint64_t>(c, N);
    s->keys_alt = carve<uint64_t>(c, N);
    s->keys3 = carve<uint64_t>(c, N);
    s->vals = carve<uint32_t>(c, N);
    s->vals_alt = carve<uint32_t>(c, N);
    s->vals3 = carve<uint32_t>(c, N);
    s->hist = carve<uint32_t>(c, (size_t)256 * s->tiles);
    s->totals = carve<uint32_t>(c, 256);
    s->box_next = carve<int>(c, 4 * (size_t)nseg);
    s->box_ord = carve<int>(c, 4 * (size_t)nseg);
    s->seg_off = carve<int>(c, nseg + 1);
    s->gseg_off = carve<int>(c, nseg + 1);
    s->gseg_off2 = carve<int>(c, nseg + 1);
    s->seg_of_pos = carve<int>(c, N);
    s->chunk_seg = carve<int>(c, s->nchunks);
    s->chunk_begin = carve<int>(c, s->nchunks);
    s->chunk_end = carve<int>(c, s->nchunks);
    s->tree.left = carve<int>(c, N);
    s->tree.right = carve<int>(c, N);
    s->tree.parent = carve<int>(c, N);
    s->tree.leaf_parent = carve<int>(c, N);
    s->tree.split = carve<int>(c, N);
    s->tree.first = carve<int>(c, N);
    s->tree.last = carve<int>(c, N);
    s->counter = carve<int>(c, N);
    s->tree.climb = carve<int4>(c, N);
    s->sums.s0 = carve<float4>(c, N);
    s->sums.s1 = carve<float4>(c, N);
    s->rec.A = carve<float4>(c, kRecStride * N);  // A and D interleaved
    s->rec.B = carve<float4>(c, N);
    s->rec.C = carve<int4>(c, N);
    s->rec.D = reinterpret_cast<int4*>(s->rec.A) + 1;
    s->ax = carve<float>(c, N);
    s->ay = carve<float>(c, N);
    s->status = carve<int>(c, 1);
    {
        // inter (2 x u64: all interactions, body-cell ones), then work: the first
        // kStepZero words are cleared by every step's key kernel
        int* w = carve<int>(c, kStepWords);
        s->inter = reinterpret_cast<unsigned long long*>(w);
        s->work = w + 4;
    }
    s->diag = carve<double>(c, 4 * (size_t)nseg);
    s->fresh = carve<int>(c, 1);
    s->flist = carve<int>(c, (size_t)s->nsupers * kFrontierCap);
    s->fcount = carve<int2>(c, (size_t)s->nsupers);
    s->sup_off = carve<int>(c, nseg + 1);
    s->heavy = carve<int>(c, (size_t)s->ngroups);
    s->seg_cost = carve<unsigned long long>(c, nseg);
    s->mean_cost = carve<int>(c, nseg);
    s->share_idx = carve<int>(c, (size_t)s->share_batches * 32);
    s->share_sum = carve<float2>(c, (size_t)s->share_batches * 32);
    s->share_ctr = carve<int>(c, kCtrWords + (size_t)s->share_slices);
    s->share_state = s->share_ctr + kCtrWords;
    s->share_desc = carve<int4>(c, (size_t)s->share_slices);

    std::vector<int> sop;
    if (nseg > 1) {
        sop.resize(N);
        for (int sg = 0; sg < nseg; ++sg)
            for (int b = s->h_off[sg]; b < s->h_off[sg + 1]; ++b) sop[b] = sg;
    }
    int rc = BH_OK;
    auto up = [&](void* dst, const void* src, size_t b) {
        if (rc == BH_OK && b) {
            cudaError_t e2 = cudaMemcpy(dst, src, b, cudaMemcpyHostToDevice);
            if (e2 != cudaSuccess) rc = cuda_fail(e2, "cudaMemcpy(tables)");
        }
    };
    up(s->seg_off, s->h_off.data(), sizeof(int) * (nseg + 1));
    up(s->gseg_off, goff.data(), sizeof(int) * (nseg + 1));
    up(s->gseg_off2, goff2.data(), sizeof(int) * (nseg + 1));
    up(s->sup_off, soff.data(), sizeof(int) * (nseg + 1));
    if (nseg > 1) up(s->seg_of_pos, sop.data(), sizeof(int) * N);
    up(s->chunk_seg, cseg.data(), sizeof(int) * s->nchunks);
    up(s->chunk_begin, cbeg.data(), sizeof(int) * s->nchunks);
    up(s->chunk_end, cend.data(), sizeof(int) * s->nchunks);
    if (rc == BH_OK && cudaMemset(s->status, 0, sizeof(int)) != cudaSuccess) rc = BH_ERR_CUDA;
    if (rc == BH_OK && cudaMemset(s->fresh, 0, sizeof(int)) != cudaSuccess) rc = BH_ERR_CUDA;
    if (rc == BH_OK && cudaMemset(s->seg_cost, 0, sizeof(unsigned long long) * nseg) != cudaSuccess)
        rc = BH_ERR_CUDA;
    if (rc == BH_OK) {
        cudaError_t ea = init_walk_attributes();
        if (ea != cudaSuccess) rc = cuda_fail(ea, "cudaFuncSetAttribute(walk)");
    }
    if (rc == BH_OK) {
        int bref = 0, bacc = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &bref, k_walk_vote, kVoteWarps * 32, 0);
        // grid cap from the worst-case shape; the walks fetch groups dynamically
        const AccShape sh{kDefaultStack, kDefaultBucket, 1};
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bacc, k_walk_acc<true, false>,
                                                      kWalkWarps * 32,
                                                      (size_t)kWalkWarps * acc_warp_bytes(sh));
        s->walk_grid_ref = walk_grid_cap(s->sms, bref) * 4;
        s->walk_grid_acc = walk_grid_cap(s->sms, bacc) * 4;
        s->walk_warps_resident = walk_grid_cap(s->sms, bacc) * kWalkWarps;
        cudaGetLastError();
    }
    if (rc != BH_OK) {
        cudaFree(s->arena);
        delete s;
        return rc;
    }
    *out = s;
    return BH_OK;
}

}  // namespace ssg

// ------------------------------------------------------------------ C ABI

extern "C" {

void bh_default_params(bh_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->mode = BH_MODE_REFERENCE;
    p->theta = 0.5f;   // kernels.cu:9
    p->eps2 = 0.025f;  // kernels.cu:8
    p->gravity = 1.0f;     // main.cpp:94
    p->timestep = 0.001f;  // main.cpp:93
    p->dampening = 1.0f;   // main.cpp:95
    p->leaf_bucket = 0;
    p->block_size = 0;
    p->stack_depth = 0;
    p->use_graph = 0;
    p->alpha = 0.01f;
    p->bodies_per_lane = 0;
}

int bh_create(const bh_params* p, int n, int device, bh_system** out) {
    return ssg::system_create(p, &n, 1, device, out);
}

int bh_ensemble_create(const bh_params* p, int nsys, const int* sizes, int device,
                       bh_system** out) {
    if (nsys < 1 || nsys > 65536 || !sizes) return BH_ERR_ARG;
    return ssg::system_create(p, sizes, nsys, device, out);
}

int bh_num_systems(const bh_system* s) { return s ? s->nseg : -1; }

int bh_system_offset(const bh_system* s, int k) {
    if (!s || k < 0 || k > s->nseg) return -1;
    return s->h_off[k];
}

int bh_destroy(bh_system* s) {
    if (!s) return BH_ERR_ARG;
    cudaSetDevice(s->device);
    if (s->copy_stream) {
        cudaStreamSynchronize(s->copy_stream);
        cudaStreamDestroy(s->copy_stream);
        cudaEventDestroy(s->in_event);
        cudaEventDestroy(s->order_event);
    }
    drop_graph(s);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    if (s->cond_stream) cudaStreamDestroy(s->cond_stream);
    if (s->fork_stream) {
        cudaStreamDestroy(s->fork_stream);
        cudaEventDestroy(s->fork_event);
        cudaEventDestroy(s->join_event);
    }
    cudaFree(s->image);
    cudaFree(s->elog);
    cudaFree(s->elog_count);
    cudaFree(s->arena);
    delete s;
    return BH_OK;
}

int bh_set_params(bh_system* s, const bh_params* p) {
    if (!s || !params_ok(p)) return BH_ERR_ARG;
    bool mode_change = p->mode != s->p.mode;
    s->p = *p;
    drop_graph(s);
    if (mode_change && s->have_state) {
        // lo words only exist in MIXED mode; start them at zero
        CK(cudaSetDevice(s->device));
        RC(settle_inputs(s));
        CK(cudaMemset(s->st[0].xlo, 0, sizeof(float) * s->n));
        CK(cudaMemset(s->st[0].ylo, 0, sizeof(float) * s->n));
    }
    return BH_OK;
}

int bh_get_params(const bh_system* s, bh_params* p) {
    if (!s || !p) return BH_ERR_ARG;
    *p = s->p;
    return BH_OK;
}

int bh_num_bodies(const bh_system* s) { return s ? s->n : -1; }

int bh_set_state(bh_system* s, const float* x, const float* y, const float* vx, const float* vy,
                 const float* mass, void* stream) {
    if (!s || !x || !y || !vx || !vy || !mass) return BH_ERR_ARG;
    s->box_valid = false;  // new positions: the next step takes the box kernel
    CK(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t b = sizeof(float) * s->n;
    const BodyPtrs& c = s->st[0];
    // x and y on `stream`: the next step's box and keys read them.  What only
    // the reorder reads first goes on the copy stream and overlaps the box,
    // keys and sort; the next call on the handle joins it:
    // - the initialisation of the other body arrays, while x and y are copied
    //   (a handle that held a state keeps its bodies' walk-group costs, by
    //   caller index);
    // - then vx, vy and mass.
    RC(copy_stream_after(s, st));
    const int* kept = nullptr;
    if (s->have_state && s->p.mode != BH_MODE_REFERENCE) {
        k_keep_cost<<<(s->n + 255) / 256, 256, 0, s->copy_stream>>>(s->n, c.id, c.gcost,
                                                                    s->st[1].gcost);
        CK(cudaGetLastError());
        kept = s->st[1].gcost;
    }
    k_state_init<<<(s->n + 255) / 256, 256, 0, s->copy_stream>>>(
        s->n, c.id, c.xlo, c.ylo, s->ax, s->ay, c.amag, c.gcost, kept, s->fresh);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(s->status, 0, sizeof(int), st));
    CK(cudaMemcpyAsync(c.x, x, b, cudaMemcpyDefault, st));
    CK(cudaMemcpyAsync(c.y, y, b, cudaMemcpyDefault, st));
    RC(copy_stream_after(s, st));  // the link is free again
    CK(cudaMemcpyAsync(c.vx, vx, b, cudaMemcpyDefault, s->copy_stream));
    CK(cudaMemcpyAsync(c.vy, vy, b, cudaMemcpyDefault, s->copy_stream));
    CK(cudaMemcpyAsync(c.m, mass, b, cudaMemcpyDefault, s->copy_stream));
    CK(cudaEventRecord(s->in_event, s->copy_stream));
    s->in_pending = true;
    s->have_state = true;
    s->caller_order = true;
    s->fresh_host = true;
    return BH_OK;
}

__global__ void k_amag(int n, const float* ax, const float* ay, float* amag, float* sax, float* say,
                       int* fresh) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *fresh = 0;  // |a| is known: no bootstrap pass in the next step
    if (i < n) {
        float a = ax[i], b = ay[i];
        amag[i] = sqrtf(a * a + b * b);
        sax[i] = a;
        say[i] = b;
    }
}

int bh_set_accel(bh_system* s, const float* ax, const float* ay, void* stream) {
    if (!s || !ax || !ay) return BH_ERR_ARG;
    if (!s->have_state || !s->caller_order) return BH_ERR_STATE;  // only right after bh_set_state
    CK(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t b = sizeof(float) * s->n;
    BodyPtrs& t = s->st[1];
    // on the copy stream, after bh_set_state's state initialisation (`stream`),
    // overlapped with the next step's box, keys and sort like vx, vy and mass
    RC(copy_stream_after(s, st));
    CK(cudaMemcpyAsync(t.x, ax, b, cudaMemcpyDefault, s->copy_stream));
    CK(cudaMemcpyAsync(t.y, ay, b, cudaMemcpyDefault, s->copy_stream));
    k_amag<<<(s->n + 255) / 256, 256, 0, s->copy_stream>>>(s->n, t.x, t.y, s->st[0].amag, s->ax,
                                                           s->ay, s->fresh);
    CK(cudaGetLastError());
    CK(cudaEventRecord(s->in_event, s->copy_stream));
    s->in_pending = true;
    s->fresh_host = false;
    return BH_OK;
}

static int scatter_out(bh_system* s, const float* a0, const float* a1, const float* a2,
                       const float* a3, float* o0, float* o1, float* o2, float* o3,
                       cudaStream_t st) {
    // stage in the scratch body arrays, then one copy per requested output
    BodyPtrs& tmp = s->st[1];
    float* t[4] = {tmp.x, tmp.y, tmp.vx, tmp.vy};
    const float* in[4] = {a0, a1, a2, a3};
    float* outp[4] = {o0, o1, o2, o3};
    k_scatter4<<<(s->n + 255) / 256, 256, 0, st>>>(
        s->n, s->st[0].id, outp[0] ? in[0] : nullptr, outp[1] ? in[1] : nullptr,
        outp[2] ? in[2] : nullptr, outp[3] ? in[3] : nullptr, t[0], t[1], t[2], t[3]);
    CK(cudaGetLastError());
    const size_t b = sizeof(float) * s->n;
    for (int k = 0; k < 4; ++k)
        if (outp[k]) CK(cudaMemcpyAsync(outp[k], t[k], b, cudaMemcpyDefault, st));
    return BH_OK;
}

int bh_get_state(bh_system* s, float* x, float* y, float* vx, float* vy, float* mass,
                 void* stream) {
    if (!s) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    const BodyPtrs& c = s->st[0];
    int rc = scatter_out(s, c.x, c.y, c.vx, c.vy, x, y, vx, vy, st);
    if (rc != BH_OK || !mass) return rc;
    return scatter_out(s, c.m, nullptr, nullptr, nullptr, mass, nullptr, nullptr, nullptr, st);
}

int bh_get_accel(bh_system* s, float* ax, float* ay, void* stream) {
    if (!s) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    return scatter_out(s, s->ax, s->ay, nullptr, nullptr, ax, ay, nullptr, nullptr,
                       (cudaStream_t)stream);
}

int bh_get_positions_hilo(bh_system* s, float* xhi, float* xlo, float* yhi, float* ylo,
                          void* stream) {
    if (!s) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    const BodyPtrs& c = s->st[0];
    return scatter_out(s, c.x, c.xlo, c.y, c.ylo, xhi, xlo, yhi, ylo, (cudaStream_t)stream);
}

int build_energy_graph(bh_system* s);
int enqueue_energy_log(bh_system* s, cudaStream_t st);

int bh_step(bh_system* s, int steps, void* stream) {
    if (!s || steps < 0) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    cudaStream_t st = (cudaStream_t)stream;
    if (s->p.use_graph) {
        auto ensure = [&](int slot) -> int {
            if (s->graph_exec[slot]) return BH_OK;
            // the capture stream must see the state that `stream` produced
            cudaEvent_t ev;
            CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CK(cudaEventRecord(ev, st));
            if (!s->cap_stream) CK(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
            CK(cudaStreamWaitEvent(s->cap_stream, ev, 0));
            cudaEventDestroy(ev);
            return build_graph(s, slot);
        };
        for (int k = 0; k < steps; ++k) {
            const int gi = s->fresh_host ? 1 : 0;  // with the bootstrap pass after bh_set_state
            if (s->in_pending) {
                // bh_set_state's copies run on: box, keys and sort first, then
                // the join, then the rest of the step
                int rc = ensure(2);
                if (rc == BH_OK) rc = ensure(3 + gi);
                if (rc != BH_OK) return rc;
                CK(cudaGraphLaunch(s->graph_exec[2], st));
                RC(join_inputs(s, st));
                CK(cudaGraphLaunch(s->graph_exec[3 + gi], st));
            } else {
                const int slot = (gi == 0 && s->box_valid) ? kGraphCarried : gi;
                int rc = ensure(slot);
                if (rc != BH_OK) return rc;
                CK(cudaGraphLaunch(s->graph_exec[slot], st));
            }
            s->box_valid = true;  // every step graph ends with the folding walk
            s->fresh_host = false;
            s->caller_order = false;
            if (s->energy_every > 0 && ++s->energy_steps % s->energy_every == 0) {
                if (!s->egraph_exec) {
                    // the capture stream must see what `stream` has produced
                    cudaEvent_t ev;
                    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                    CK(cudaEventRecord(ev, st));
                    CK(cudaStreamWaitEvent(s->cap_stream, ev, 0));
                    cudaEventDestroy(ev);
                    int rc = build_energy_graph(s);
                    if (rc != BH_OK) return rc;
                }
                CK(cudaGraphLaunch(s->egraph_exec, st));
            }
        }
        return BH_OK;
    }
    for (int k = 0; k < steps; ++k) {
        int rc = BH_OK;
        if (s->in_pending) {
            const int boot = s->fresh_host ? 1 : 0;
            s->fresh_host = false;
            rc = enqueue_step(s, st, nullptr, boot, kStepPre);
            if (rc == BH_OK) rc = join_inputs(s, st);
            if (rc == BH_OK) rc = enqueue_step(s, st, nullptr, boot, kStepPost);
        } else {
            rc = enqueue_step(s, st);
        }
        if (rc != BH_OK) return rc;
        s->caller_order = false;
        if (s->energy_every > 0 && ++s->energy_steps % s->energy_every == 0) {
            rc = enqueue_energy_log(s, st);
            if (rc != BH_OK) return rc;
        }
    }
    return BH_OK;
}

int bh_sync(bh_system* s, void* stream) {
    if (!s) return BH_ERR_ARG;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    int bits = 0;
    CK(cudaMemcpy(&bits, s->status, sizeof(int), cudaMemcpyDeviceToHost));
    return status_code(bits, s->p.mode);
}

int bh_get_stats(bh_system* s, bh_stats* out, void* stream) {
    if (!s || !out) return BH_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    int bits = 0;
    unsigned long long inter[2] = {0, 0};
    int box[4] = {0, 0, 0, 0};
    int wst[3] = {0, 0, 0};
    CK(cudaMemcpy(wst, s->work + 3, sizeof(wst), cudaMemcpyDeviceToHost));
    out->max_stack = wst[0];
    out->walk_rounds = wst[1];
    out->nodes_tested = wst[2];
    CK(cudaMemcpy(&bits, s->status, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(inter, s->inter, sizeof(inter), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(box, s->box_ord, sizeof(box), cudaMemcpyDeviceToHost));
    out->status = status_code(bits, s->p.mode);
    out->interactions = (int64_t)inter[0];
    out->cell_interactions = (int64_t)inter[1];
    for (int k = 0; k < 4; ++k) {
        int i = box[k];
        int b = i >= 0 ? i : (i ^ 0x7fffffff);
        std::memcpy(&out->box[k], &b, 4);
    }
    // tree shape from the split levels (host pass over n ints; debugging aid)
    std::vector<int> split(s->n), parent(s->n);
    CK(cudaMemcpy(split.data(), s->tree.split, sizeof(int) * s->n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(parent.data(), s->tree.parent, sizeof(int) * s->n, cudaMemcpyDeviceToHost));
    long long cells = 0;
    int nodes = 0, maxd = 0;
    for (int i = 0; i < s->n; ++i) {
        int sp = split[i];
        if (sp < 0) continue;
        int pa = parent[i];
        if (pa >= 0 && (sp & 1) && split[pa] == sp - 1) continue;  // merged
        ++nodes;
        int L = sp >> 1;
        int Lp = pa >= 0 ? (split[pa] >> 1) : 0;
        // cells of the reference tree owned by this node: its chain and itself
        cells += (pa >= 0) ? (L - Lp) : L;
        maxd = std::max(maxd, L + 1);
    }
    out->cells = (int32_t)cells;
    out->nodes = nodes;
    out->max_depth = maxd;
    return BH_OK;
}

int bh_render(bh_system* s, int width, int height, float x0, float x1, float y0, float y1,
              unsigned char* rgba, void* stream) {
    if (!s || !rgba || width <= 0 || height <= 0 || (long long)width * height > (1ll << 28) ||
        !(x1 > x0) || !(y1 > y0))
        return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t pixels = (size_t)width * height;
    if (pixels > s->image_pixels) {
        CK(cudaStreamSynchronize(st));  // the old buffer may still be read
        cudaFree(s->image);
        s->image = nullptr;
        s->image_pixels = 0;
        CK(cudaMalloc(&s->image, sizeof(uint32_t) * pixels));
        s->image_pixels = pixels;
    }
    const float sx = (float)width / (x1 - x0), sy = (float)height / (y1 - y0);
    CK(cudaMemsetAsync(s->image, 0, sizeof(uint32_t) * pixels, st));
    k_splat<<<(s->n + 255) / 256, 256, 0, st>>>(s->n, s->st[0].x, s->st[0].y, width, height, x0,
                                                sx, y0, sy, s->image);
    k_shade<<<(int)((pixels + 255) / 256), 256, 0, st>>>((int)pixels, s->image);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rgba, s->image, sizeof(uint32_t) * pixels, cudaMemcpyDefault, st));
    return BH_OK;
}

int bh_check(bh_system* s, void* stream, unsigned* failed) {
    if (!s || !failed) return BH_ERR_ARG;
    if (!s->have_state || s->caller_order || !s->kfinal) return BH_ERR_STATE;  // needs a step
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    const int n = s->n;
    // scratch: the key buffer the last sort did not end in, and the arrival counters
    auto* acc = reinterpret_cast<unsigned long long*>(s->kfinal == s->keys ? s->keys_alt : s->keys);
    auto* flags = reinterpret_cast<unsigned*>(acc + 2);
    CK(cudaMemsetAsync(acc, 0, 3 * sizeof(unsigned long long), st));
    CK(cudaMemsetAsync(s->counter, 0, sizeof(int) * n, st));
    Segs segs{s->nseg, s->seg_off, s->nseg > 1 ? s->seg_of_pos : nullptr};
    const int nb = (n + 255) / 256;
    k_check_nodes<<<nb, 256, 0, st>>>(n, segs, s->tree, s->st[1].m, s->sums, acc, flags);
    k_check_bodies<<<nb, 256, 0, st>>>(n, segs, s->kfinal, s->st[0].id, s->counter, s->box_ord,
                                       flags);
    k_check_seen<<<nb, 256, 0, st>>>(n, s->counter, flags);
    CK(cudaGetLastError());
    unsigned long long h[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    unsigned f = (unsigned)(h[2] & 0xffffffffull);
    const unsigned long long nn = (unsigned long long)n;
    if (h[0] != nn * (nn - 1) / 2 || h[1] != nn) f |= CK_CHILD_SUM;
    *failed = f;
    return BH_OK;
}

int bh_get_debug(bh_system* s, const char* name, void* host_out, size_t bytes, void* stream) {
    if (!s || !name || !host_out) return BH_ERR_ARG;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    const size_t N = (size_t)s->n;
    const void* src = nullptr;
    size_t need = 0;
    std::string nm(name);
    if (nm == "box" || nm == "boxes") {
        // the last step's box of system 0 (box) or of every system (boxes: 4 nseg floats)
        const size_t words = nm == "box" ? 4 : 4 * (size_t)s->nseg;
        if (bytes < 4 * words) return BH_ERR_ARG;
        std::vector<int> box(words);
        CK(cudaMemcpy(box.data(), s->box_ord, 4 * words, cudaMemcpyDeviceToHost));
        float* f = (float*)host_out;
        for (size_t k = 0; k < words; ++k) {
            int i = box[k];
            int b = i >= 0 ? i : (i ^ 0x7fffffff);
            std::memcpy(&f[k], &b, 4);
        }
        return BH_OK;
    }
    if (nm == "accel_sorted") {
        if (bytes < 8 * N) return BH_ERR_ARG;
        CK(cudaMemcpy(host_out, s->ax, 4 * N, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy((char*)host_out + 4 * N, s->ay, 4 * N, cudaMemcpyDeviceToHost));
        return BH_OK;
    }
    if (nm == "share") {  // the last walk's Share counters
        if (bytes < 4 * 4) return BH_ERR_ARG;
        std::vector<int> ctr(kCtrWords);
        CK(cudaMemcpy(ctr.data(), s->share_ctr, 4 * kCtrWords, cudaMemcpyDeviceToHost));
        const int at[4] = {kCtrHead, kCtrTail, kCtrBatches, kCtrBack};
        for (int k = 0; k < 4; ++k) static_cast<int*>(host_out)[k] = ctr[at[k]];
        return BH_OK;
    }
    if (nm == "keys") { src = s->kfinal; need = 8 * N; }
    else if (nm == "perm") { src = s->st[0].id; need = 4 * N; }
    else if (nm == "node_left") { src = s->tree.left; need = 4 * N; }
    else if (nm == "node_right") { src = s->tree.right; need = 4 * N; }
    else if (nm == "node_split") { src = s->tree.split; need = 4 * N; }
    else if (nm == "node_first") { src = s->tree.first; need = 4 * N; }
    else if (nm == "node_last") { src = s->tree.last; need = 4 * N; }
    else if (nm == "node_parent") { src = s->tree.parent; need = 4 * N; }
    else {
        // node sums: one float of the 16-byte records, a strided copy
        const float* f = nullptr;
        if (nm == "node_m") f = &s->sums.s0->x;
        else if (nm == "node_mx") f = &s->sums.s0->y;
        else if (nm == "node_my") f = &s->sums.s0->z;
        else if (nm == "node_cx") f = &s->sums.s0->w;
        else if (nm == "node_cy") f = &s->sums.s1->x;
        else return BH_ERR_ARG;
        if (bytes < 4 * N) return BH_ERR_ARG;
        CK(cudaMemcpy2D(host_out, 4, f, sizeof(float4), 4, N, cudaMemcpyDeviceToHost));
        return BH_OK;
    }
    if (!src) return BH_ERR_STATE;
    if (bytes < need) return BH_ERR_ARG;
    CK(cudaMemcpy(host_out, src, need, cudaMemcpyDeviceToHost));
    return BH_OK;
}

int bh_step_profiled(bh_system* s, void* stream, float* phase_ms) {
    if (!s || !phase_ms) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t ev[BH_NUM_PHASES + 1];
    for (auto& e : ev) CK(cudaEventCreate(&e));
    int rc = enqueue_step(s, st, ev);
    s->caller_order = false;
    if (rc == BH_OK) {
        CK(cudaEventSynchronize(ev[BH_NUM_PHASES]));
        for (int k = 0; k < BH_NUM_PHASES; ++k) {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            phase_ms[k] += ms;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

int bh_direct_sum_f64(bh_system* s, int ns, const int* idx, double* ax, double* ay) {
    if (!s || ns < 1 || !idx || !ax || !ay) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    for (int k = 0; k < ns; ++k)
        if (idx[k] < 0 || idx[k] >= s->n) return BH_ERR_ARG;
    CK(cudaSetDevice(s->device));
    RC(settle_inputs(s));
    const BodyPtrs& c = s->st[0];
    BodyPtrs& t = s->st[1];
    bool mixed = s->p.mode == BH_MODE_MIXED;
    // caller-order copies in the scratch body arrays: x, y, m and the lo words
    k_scatter4<<<(s->n + 255) / 256, 256>>>(s->n, c.id, c.x, c.y, c.m, nullptr, t.x, t.y, t.vx,
                                             nullptr);
    CK(cudaGetLastError());
    if (mixed) {
        k_scatter4<<<(s->n + 255) / 256, 256>>>(s->n, c.id, c.xlo, c.ylo, nullptr, nullptr, t.xlo,
                                                 t.ylo, nullptr, nullptr);
        CK(cudaGetLastError());
    }
    int* d_idx = nullptr;
    double* d_part = nullptr;
    double* d_out = nullptr;
    CK(cudaMalloc(&d_idx, sizeof(int) * ns));
    CK(cudaMalloc(&d_part, sizeof(double) * 2 * (size_t)ns * kDirChunks));
    CK(cudaMalloc(&d_out, sizeof(double) * 2 * (size_t)ns));
    CK(cudaMemcpy(d_idx, idx, sizeof(int) * ns, cudaMemcpyHostToDevice));
    dim3 grid((ns + kDirThreads - 1) / kDirThreads, kDirChunks);
    k_direct_partial<<<grid, kDirThreads>>>(s->n, t.x, mixed ? t.xlo : nullptr, t.y,
                                            mixed ? t.ylo : nullptr, t.vx, ns, d_idx,
                                            (double)s->p.eps2, d_part);
    k_direct_reduce<<<(2 * ns + 255) / 256, 256>>>(ns, kDirChunks, d_part,
                                                   s->p.mode == BH_MODE_REFERENCE ? 1.0 : (double)s->p.gravity,
                                                   d_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(ax, d_out, sizeof(double) * ns, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ay, d_out + ns, sizeof(double) * ns, cudaMemcpyDeviceToHost);
    cudaFree(d_idx);
    cudaFree(d_part);
    cudaFree(d_out);
    if (e != cudaSuccess) return cuda_fail(e, "bh_direct_sum_f64");
    return BH_OK;
}

int bh_measure_fp32_peaks(int device, double* scalar, double* packed) {
    if (!scalar || !packed) return BH_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return BH_ERR_NO_DEVICE;
    if (device >= 0) CK(cudaSetDevice(device));
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float* out = nullptr;
    CK(cudaMalloc(&out, sizeof(float) * blocks * threads));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    // both kernels: 256 flops per thread and iteration; best of 5 after one warm-up
    const double flops = 256.0 * iters * (double)blocks * threads;
    double* res[2] = {scalar, packed};
    int rc = BH_OK;
    for (int kind = 0; kind < 2 && rc == BH_OK; ++kind) {
        float best = 1e30f;
        for (int rep = 0; rep < 6; ++rep) {
            cudaError_t e = cudaEventRecord(e0);
            if (kind == 0)
                k_ffma_peak<<<blocks, threads>>>(out, iters, 0.999f, 1e-6f);
            else
                k_ffma2_peak<<<blocks, threads>>>(out, iters, 0.999f, 1e-6f);
            if (e == cudaSuccess) e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(e1);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "bh_measure_fp32_peaks");
                break;
            }
            if (rep > 0) best = ms < best ? ms : best;
        }
        *res[kind] = flops / (best * 1e-3) / 1e12;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return rc;
}

int bh_measure_fp32_peak(int device, double* tflops) {
    if (!tflops) return BH_ERR_ARG;
    double a = 0.0, b = 0.0;
    int rc = bh_measure_fp32_peaks(device, &a, &b);
    if (rc == BH_OK) *tflops = a > b ? a : b;
    return rc;
}

// Per-system FP64 sums: out[4k..4k+3] += kinetic, potential (0.5 m phi), px, py.
// Reduced over the block first (one atomic per block and value) when the
// block's positions belong to one system, as systems are contiguous ranges.
__global__ void __launch_bounds__(256) k_energy_reduce(int n, Segs segs,
                                                       const float* __restrict__ m,
                                                       const float* __restrict__ vx,
                                                       const float* __restrict__ vy,
                                                       const double* __restrict__ pot,
                                                       double* __restrict__ out) {
    __shared__ double s_part[8][4];
    const int b0 = blockIdx.x * blockDim.x;
    const int i = b0 + threadIdx.x;
    double e[4] = {0.0, 0.0, 0.0, 0.0};
    int sg = 0;
    if (i < n) {
        const double mi = m[i], u = vx[i], v = vy[i];
        e[0] = 0.5 * mi * (u * u + v * v);
        e[1] = 0.5 * mi * pot[i];
        e[2] = mi * u;
        e[3] = mi * v;
        sg = seg_of(segs, i);
    }
    const int last = min(n, b0 + (int)blockDim.x) - 1;
    if (seg_of(segs, b0) != seg_of(segs, last)) {  // a block across two systems
        if (i < n)
            for (int k = 0; k < 4; ++k) atomicAdd(out + 4 * sg + k, e[k]);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) e[k] += __shfl_down_sync(kFull, e[k], o);
        if (lane == 0) s_part[warp][k] = e[k];
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        const int s0 = seg_of(segs, b0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double v = lane < nw ? s_part[lane][k] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
            if (lane == 0) atomicAdd(out + 4 * s0 + k, v);
        }
    }
}

// The diagnostics pass on `st`, no synchronisation: the tree of the current
// positions, a potential walk (FP64 sums per body), then per-system sums of
// kinetic and potential energy and momentum into s->diag.
int enqueue_energy(bh_system* s, cudaStream_t st) {
    int rc = enqueue_front(s, st, true, nullptr, true);  // tree of the current positions
    if (rc != BH_OK) return rc;
    StepArgs a = step_args(s);
    a.alpha = 0.0f;
    const AccShape sh{a.stack, a.bucket, a.bpl};
    const Groups& gr = a.bpl == 2 ? a.groups2 : a.groups;
    const size_t smem = (size_t)a.warps * acc_warp_bytes(sh);
    int grid = std::min(a.walk_grid_acc, (gr.ngroups + a.warps - 1) / a.warps);
    if (grid < 1) grid = 1;
    // the sort's spare key buffer holds the per-body potential (8 bytes per body)
    double* pot = reinterpret_cast<double*>(s->kfinal == s->keys ? s->keys_alt : s->keys);
    int* counter = s->work + 6;  // dynamic scheduling of this pass; work[7]: its stack peak
    CK(cudaMemsetAsync(counter, 0, 2 * sizeof(int), st));
    if (a.bpl == 2)
        k_walk_acc<false, false, true, 2><<<grid, a.warps * 32, smem, st>>>(
            sh, a.segs, gr, a.in, a.recA, a.recB, a.recC, a.recD, a.eps2, a.G, a.dt, a.ddt, 0.0f,
            a.out, a.status, a.inter, counter, a.fresh, s->work + 7, pot, Frontier{}, Heavy{},
            Share{});
    else
        k_walk_acc<false, false, true, 1><<<grid, a.warps * 32, smem, st>>>(
            sh, a.segs, gr, a.in, a.recA, a.recB, a.recC, a.recD, a.eps2, a.G, a.dt, a.ddt, 0.0f,
            a.out, a.status, a.inter, counter, a.fresh, s->work + 7, pot, Frontier{}, Heavy{},
            Share{});
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(s->diag, 0, sizeof(double) * 4 * s->nseg, st));
    Segs segs{s->nseg, s->seg_off, s->nseg > 1 ? s->seg_of_pos : nullptr};
    const BodyPtrs& g = s->st[1];
    k_energy_reduce<<<(s->n + 255) / 256, 256, 0, st>>>(s->n, segs, g.m, g.vx, g.vy, pot, s->diag);
    CK(cudaGetLastError());
    return BH_OK;
}

int bh_energy(bh_system* s, void* stream, double* out) {
    if (!s || !out) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    int rc = enqueue_energy(s, st);
    if (rc != BH_OK) return rc;
    CK(cudaMemcpyAsync(out, s->diag, sizeof(double) * 4 * s->nseg, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int bits = 0;
    CK(cudaMemcpy(&bits, s->status, sizeof(int), cudaMemcpyDeviceToHost));
    return status_code(bits, BH_MODE_PLAIN);
}

// Append s->diag to the ring log (one block).
__global__ void k_energy_log(const double* __restrict__ diag, int values, double* __restrict__ log,
                             int* __restrict__ count, int cap) {
    __shared__ int s_slot;
    if (threadIdx.x == 0) s_slot = *count % cap;
    __syncthreads();
    for (int i = threadIdx.x; i < values; i += blockDim.x) log[(size_t)s_slot * values + i] = diag[i];
    __syncthreads();
    if (threadIdx.x == 0) *count += 1;
}

int enqueue_energy_log(bh_system* s, cudaStream_t st) {
    int rc = enqueue_energy(s, st);
    if (rc != BH_OK) return rc;
    k_energy_log<<<1, 256, 0, st>>>(s->diag, 4 * s->nseg, s->elog, s->elog_count, s->energy_cap);
    CK(cudaGetLastError());
    return BH_OK;
}

int build_energy_graph(bh_system* s) {
    if (!s->cap_stream) CK(cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking));
    if (!s->cond_stream) CK(cudaStreamCreateWithFlags(&s->cond_stream, cudaStreamNonBlocking));
    RC(make_fork_stream(s));
    CK(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_energy_log(s, s->cap_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
    if (st != BH_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    s->egraph = g;
    CK(cudaGraphInstantiate(&s->egraph_exec, g, 0));
    return BH_OK;
}

int bh_set_energy_log(bh_system* s, int every, int capacity) {
    if (!s || every < 0 || (every > 0 && capacity <= 0)) return BH_ERR_ARG;
    CK(cudaSetDevice(s->device));
    CK(cudaDeviceSynchronize());  // no step may still write the old log
    cudaFree(s->elog);
    cudaFree(s->elog_count);
    s->elog = nullptr;
    s->elog_count = nullptr;
    if (s->egraph_exec) cudaGraphExecDestroy(s->egraph_exec);
    if (s->egraph) cudaGraphDestroy(s->egraph);
    s->egraph_exec = nullptr;
    s->egraph = nullptr;
    s->energy_every = 0;
    s->energy_cap = 0;
    s->energy_steps = 0;
    if (every == 0) return BH_OK;
    CK(cudaMalloc(&s->elog, sizeof(double) * 4 * s->nseg * (size_t)capacity));
    CK(cudaMalloc(&s->elog_count, sizeof(int)));
    CK(cudaMemset(s->elog_count, 0, sizeof(int)));
    s->energy_every = every;
    s->energy_cap = capacity;
    return BH_OK;
}

int bh_get_energy_log(bh_system* s, double* out, int max_records, int* records, void* stream) {
    if (!s || !records || (max_records > 0 && !out)) return BH_ERR_ARG;
    *records = 0;
    if (!s->energy_every) return BH_OK;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    int count = 0;
    CK(cudaMemcpy(&count, s->elog_count, sizeof(int), cudaMemcpyDeviceToHost));
    *records = count;
    // the last min(count, capacity, max_records) records, oldest first
    const int keep = std::min(std::min(count, s->energy_cap), std::max(max_records, 0));
    const size_t rec = 4 * (size_t)s->nseg;
    for (int r = 0; r < keep; ++r) {
        const int idx = count - keep + r;
        CK(cudaMemcpy(out + r * rec, s->elog + (size_t)(idx % s->energy_cap) * rec,
                      sizeof(double) * rec, cudaMemcpyDeviceToHost));
    }
    return BH_OK;
}

int bh_autotune(bh_system* s, void* stream, bh_params* chosen) {
    if (!s) return BH_ERR_ARG;
    if (!s->have_state) return BH_ERR_STATE;
    CK(cudaSetDevice(s->device));
    RC(join_inputs(s, (cudaStream_t)stream));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t N = (size_t)s->n;
    // scratch of this call, released on every way out; an early return (a
    // CUDA error) also puts back the parameters and the sort's pass count
    struct Scratch {
        bh_system* s;
        bh_params p;
        int passes;
        float* bk = nullptr;
        void* flush = nullptr;  // written before every timed step: larger than L2
        cudaEvent_t ev[2 * kTrialSteps] = {};
        bool done = false;
        ~Scratch() {
            if (bk) cudaFree(bk);
            if (flush) cudaFree(flush);
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (!done) {
                s->p = p;
                s->high_passes = passes;
                s->box_valid = false;
                drop_graph(s);
            }
        }
    } sc{s, s->p, s->high_passes};
    // back up the state the candidates will all start from
    CK(cudaMalloc(&sc.bk, N * 9 * sizeof(float) + sizeof(int)));
    if (cudaMalloc(&sc.flush, kTrialFlushBytes) != cudaSuccess) {  // optional: no flush then
        sc.flush = nullptr;
        cudaGetLastError();
    }
    float* bk = sc.bk;
    BodyPtrs& c = s->st[0];
    float* arrs[8] = {c.x, c.y, c.vx, c.vy, c.m, c.xlo, c.ylo, c.amag};
    const bool orig_fresh = s->fresh_host;
    auto save = [&]() -> int {
        for (int k = 0; k < 8; ++k)
            CK(cudaMemcpyAsync(bk + k * N, arrs[k], N * sizeof(float), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(bk + 8 * N, c.id, N * sizeof(int), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(bk + 9 * N, s->fresh, sizeof(int), cudaMemcpyDeviceToDevice, st));
        return BH_OK;
    };
    auto restore = [&]() -> int {
        for (int k = 0; k < 8; ++k)
            CK(cudaMemcpyAsync(arrs[k], bk + k * N, N * sizeof(float), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(c.id, bk + 8 * N, N * sizeof(int), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(s->fresh, bk + 9 * N, sizeof(int), cudaMemcpyDeviceToDevice, st));
        CK(cudaMemsetAsync(s->status, 0, sizeof(int), st));
        s->fresh_host = orig_fresh;
        s->box_valid = false;  // positions put back: box_next is a trial step's
        return BH_OK;
    };
    const bh_params orig = s->p;
    const bool orig_caller = s->caller_order;
    int rc = save();
    bh_params best = orig;
    if (rc == BH_OK && orig.mode != BH_MODE_REFERENCE) {
        // stack depth: 1.5x the deepest stack of one step with a generous stack
        s->p.stack_depth = kMaxStack;
        drop_graph(s);
        rc = enqueue_step(s, st);
        int peak = 0;
        if (rc == BH_OK) {
            cudaError_t e = cudaMemcpyAsync(&peak, s->work + 3, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) rc = cuda_fail(e, "bh_autotune");
        }
        const int stack = std::min(kMaxStack, std::max(256, ((peak * 3 / 2) + 127) / 128 * 128));
        const int blocks[2] = {128, 256};
        const int buckets[3] = {4, 8, 16};
        const int bpls[2] = {1, 2};
        if (rc == BH_OK)
            for (cudaEvent_t& e : sc.ev) CK(cudaEventCreate(&e));
        // one candidate from the saved state: a warm-up step (with the box
        // kernel and, if fresh, the bootstrap), then `steps` timed steps, each
        // after a write larger than L2 (a step's working set does not stay in
        // L2 from one step to the next at the sizes where the shapes differ);
        // ms per step, +inf if a step reported an error
        auto trial = [&](const bh_params& cand, int passes, int steps, float* ms) -> int {
            s->p = cand;
            s->p.use_graph = 0;
            s->high_passes = passes;
            drop_graph(s);
            int r = restore();
            if (r == BH_OK) r = enqueue_step(s, st);
            if (r != BH_OK) return r;
            steps = std::min(steps, kTrialSteps);
            for (int k = 0; k < steps && r == BH_OK; ++k) {
                if (sc.flush) CK(cudaMemsetAsync(sc.flush, k, kTrialFlushBytes, st));
                CK(cudaEventRecord(sc.ev[2 * k], st));
                r = enqueue_step(s, st);
                CK(cudaEventRecord(sc.ev[2 * k + 1], st));
            }
            if (r != BH_OK) return r;
            CK(cudaEventSynchronize(sc.ev[2 * steps - 1]));
            float t = 0.f;
            for (int k = 0; k < steps; ++k) {
                float tk = 0.f;
                CK(cudaEventElapsedTime(&tk, sc.ev[2 * k], sc.ev[2 * k + 1]));
                t += tk;
            }
            int bits = 0;
            CK(cudaMemcpy(&bits, s->status, sizeof(int), cudaMemcpyDeviceToHost));
            *ms = status_code(bits, cand.mode) == BH_OK ? t / (float)steps : 1e30f;
            return BH_OK;
        };
        // every shape for 3 steps, then the best three again, three times for 8
        // steps each in turn, by their fastest run: candidates within a few per
        // cent of one another are told apart by more than two steps
        const int size_rule = s->high_passes;
        std::vector<std::pair<float, bh_params>> cands;
        for (int li = 0; li < 2 && rc == BH_OK; ++li)
            for (int bi = 0; bi < 2 && rc == BH_OK; ++bi)
                for (int ki = 0; ki < 3 && rc == BH_OK; ++ki) {
                    bh_params cand = orig;
                    cand.block_size = blocks[bi];
                    cand.leaf_bucket = buckets[ki];
                    cand.bodies_per_lane = bpls[li];
                    cand.stack_depth = stack;
                    float ms = 1e30f;
                    rc = trial(cand, size_rule, 3, &ms);
                    cands.push_back({ms, cand});
                }
        if (rc == BH_OK) {
            std::stable_sort(cands.begin(), cands.end(),
                             [](const auto& a, const auto& b) { return a.first < b.first; });
            const int top = std::min<int>(3, (int)cands.size());
            std::vector<float> again(top, 1e30f);
            for (int round = 0; round < 3 && rc == BH_OK; ++round)
                for (int q = 0; q < top && rc == BH_OK; ++q) {
                    float ms = 1e30f;
                    rc = trial(cands[q].second, size_rule, kTrialSteps, &ms);
                    again[q] = std::min(again[q], ms);
                }
            int bq = 0;
            for (int q = 1; q < top; ++q)
                if (again[q] < again[bq]) bq = q;
            if (again[bq] < 1e30f) best = cands[bq].second;
        }
        // The sort's fast path with the chosen walk: 3 or 4 high-word passes.
        // The fixup's work grows with the bodies per 2^-12 cell, so the better
        // count depends on the density, not only on N; the size rule's choice
        // stays unless the other steps more than 1 % faster.
        float pass_ms[2] = {1e30f, 1e30f};
        for (int round = 0; round < 2 && rc == BH_OK; ++round)
            for (int hp = 3; hp <= 4 && rc == BH_OK; ++hp) {
                float ms = 1e30f;
                rc = trial(best, hp, kTrialSteps, &ms);
                pass_ms[hp - 3] = std::min(pass_ms[hp - 3], ms);
            }
        s->high_passes = size_rule;
        if (rc == BH_OK) {
            const float keep = pass_ms[size_rule - 3], other = pass_ms[4 - size_rule];
            if (other < 0.99f * keep) s->high_passes = 7 - size_rule;
        }
    }
    if (rc == BH_OK) rc = restore();
    if (rc == BH_OK) CK(cudaStreamSynchronize(st));
    sc.done = true;
    best.use_graph = orig.use_graph;
    s->p = rc == BH_OK ? best : orig;
    s->caller_order = orig_caller;
    drop_graph(s);
    if (chosen) *chosen = s->p;
    return rc;
}

const char* bh_status_string(int st) {
    switch (st) {
        case BH_OK: return "ok";
        case BH_ERR_ARG: return "invalid argument";
        case BH_ERR_DUPLICATE_KEYS: return "two bodies share all 32 quadtree levels";
        case BH_ERR_NONFINITE: return "non-finite position";
        case BH_ERR_CAPACITY: return "capacity exceeded";
        case BH_ERR_STACK: return "walk stack overflow";
        case BH_ERR_TREE: return "tree traversal bound exceeded";
        case BH_ERR_CUDA: return "CUDA error";
        case BH_ERR_NOMEM: return "out of memory";
        case BH_ERR_STATE: return "call out of order";
        case BH_ERR_NO_DEVICE: return "no suitable CUDA device";
        default: return "unknown status";
    }
}

const char* bh_last_error(void) { return ssg::g_last_error.c_str(); }

const char* bh_version(void) { return "0.1.0 sm_103a"; }

}  // extern "C"
