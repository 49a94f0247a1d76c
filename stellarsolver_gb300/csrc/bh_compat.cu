// The reference's nine launch wrappers (Particle_cuda.cuh:5-13) on the
// reference's own array layout, implemented with this library's kernels.
//
// BuildQuadTree sorts quadrant keys and builds the radix tree of
// bh_device.cuh, then writes it out in the reference layout: cells numbered
// from n in node order, a chain of single-child cells above every branching
// cell (the reference's tree is uncompressed, kernels.cu:197-252), child slots
// by quadrant digit, cell x/y/mass = sum(m*x), sum(m*y), sum(m) and count.
// SortParticles fills sorted[]/start[] by a level-by-level pass over the
// whole device (a cooperative grid, one grid barrier per tree level);
// CalculateForces is the warp-vote walk over child[] (kernels.cu:340-435).
// Scratch buffers (keys, sort, tree, frontier queues) are kept per device and
// grown on demand.  Each device also keeps the last tree layout a builder
// produced (its child[] pointer and m), which SortParticles and
// CalculateForces use to bound their reads of child[].
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "Particle_cuda.cuh"
#include "bh_compat.h"
#include "bh_device.cuh"
#include "bh_engine.h"
#include "stellar_bh.h"

using namespace ssg;

namespace {

struct CompatSettings {
    float theta = 0.5f;   // kernels.cu:9
    float eps2 = 0.025f;  // kernels.cu:8
    cudaStream_t stream = nullptr;
};
CompatSettings g_set;
thread_local int t_status = BH_OK;

void record(int st) {
    if (t_status == BH_OK && st != BH_OK) t_status = st;
}
void record_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) record(cuda_fail(e, what));
}

// ------------------------------------------------------------------ workspace

struct Workspace {
    int device = -1;
    size_t cap = 0;  // bodies
    size_t mcap = 0;  // nodes (m) for the frontier queues
    void* base = nullptr;
    unsigned gen = 0;  // allocations so far: a growth frees what the last build left
    uint64_t *keys, *keys_alt, *keys3;  // keys3: the third buffer of the high-word sort
    uint32_t *vals, *vals_alt, *vals3;
    int* overflow;                       // a run of equal high words longer than kFixupRun
    uint32_t *hist, *totals;
    int tiles;
    int* box_ord;
    int* seg_off;
    TreePtrs tree;
    int* counter;
    NodeSums sums;
    float *sx, *sy, *sm;
    int *ncell, *cbase, *bsum, *total;
    int *qa, *qb;
    int* qcount;  // three level counters of the SortParticles queues
    Records rec;  // REFERENCE walk records of the last build's tree (CalculateForces)
    int* flist;    // CalculateForces: the reference rule's walk frontiers (k_frontier)
    int2* fcount;
    unsigned long long* inter;  // CalculateForces: interactions (the walk's counter)
    int* work;                  // CalculateForces: the walk's group counter
    int* status;
};

// One workspace per device.  Held by pointer, so a workspace keeps its address
// when another device adds its own.
std::mutex g_ws_mu;
std::vector<std::unique_ptr<Workspace>> g_ws;

// The last tree layout built on each device (by BuildQuadTree or
// BuildQuadTreeNoAlloc): SortParticles and CalculateForces read child[] up to
// node m - 1 when they are given the same child array on the same device.
constexpr int kMaxDevices = 64;
struct Layout {
    const int* child = nullptr;
    int m = 0;
};
Layout g_layout[kMaxDevices];  // guarded by g_ws_mu

// The last BuildQuadTree on each device, for SortParticles: its child array
// and sizes, and the workspace (with its allocation count) that still holds
// its sort permutation, tree and cell numbering.  BuildQuadTreeNoAlloc clears
// it (its scratch is reused by the next call).
struct Built {
    const int* child = nullptr;
    int n = 0, m = 0;
    Workspace* w = nullptr;
    unsigned gen = 0;
};
Built g_built[kMaxDevices];  // guarded by g_ws_mu

int g_sms[kMaxDevices] = {};   // SM count per device, read once (guarded by g_ws_mu)

int current_device() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    return dev;
}

void set_built(const Built& b) {
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    g_built[dev] = b;
}

void set_layout(const int* child, int m) {
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    g_layout[dev] = Layout{child, m};
}

// Nodes of child[] that the last build on this device covers, or the
// reference's capacity 2n + 12000 (BarnesHutParticleSystem.cpp:33) for a
// layout no build of this process produced.
int layout_m(const int* child, int n) {
    const int dev = current_device();
    if (dev >= 0 && dev < kMaxDevices) {
        std::lock_guard<std::mutex> lk(g_ws_mu);
        if (g_layout[dev].child == child && g_layout[dev].m > 0) return g_layout[dev].m;
    }
    return 2 * n + 12000;
}

int device_sms() {
    const int dev = current_device();
    if (dev < 0) return 1;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    if (dev < kMaxDevices && g_sms[dev] > 0) return g_sms[dev];
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 1;
    if (dev < kMaxDevices) g_sms[dev] = sms;
    return sms;
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

// The current device's workspace with room for n bodies and m nodes, grown
// (cudaFree + cudaMalloc) when it is smaller.
Workspace* workspace(size_t n, size_t m) {
    const int dev = current_device();
    if (dev < 0) return nullptr;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    Workspace* w = nullptr;
    for (auto& x : g_ws)
        if (x->device == dev) w = x.get();
    if (w && w->cap >= n && w->mcap >= m) return w;
    if (!w) {
        g_ws.push_back(std::make_unique<Workspace>());
        w = g_ws.back().get();
        w->device = dev;
    }
    if (w->base) cudaFree(w->base);
    w->base = nullptr;
    size_t N = std::max(n, w->cap), M = std::max(m, w->mcap);
    int tiles = (int)((N + kSortTile - 1) / kSortTile);
    int nb = (int)((N + 1023) / 1024);
    size_t bytes = 3 * al(8 * N) + 3 * al(4 * N) + al(4) + al(4 * 256 * (size_t)tiles) +
                   al(4 * 256) + al(16) + al(8) + 8 * al(4 * N) + al(16 * N) + 2 * al(16 * N) +
                   3 * al(4 * N) + 2 * al(4 * N) + al(4 * (size_t)nb) + al(4) + 2 * al(4 * M) +
                   al(12) + 3 * al(16 * N) + al(8) + al(4) + al(4) +
                   al(4 * (size_t)num_supers((int)N) * kFrontierCap) + al(8 * (size_t)num_supers((int)N));
    ++w->gen;
    if (cudaMalloc(&w->base, bytes) != cudaSuccess) {
        w->base = nullptr;
        w->cap = w->mcap = 0;
        return nullptr;
    }
    char* c = (char*)w->base;
    auto take = [&](size_t b) {
        void* p = c;
        c += al(b);
        return p;
    };
    w->keys = (uint64_t*)take(8 * N);
    w->keys_alt = (uint64_t*)take(8 * N);
    w->keys3 = (uint64_t*)take(8 * N);
    w->vals = (uint32_t*)take(4 * N);
    w->vals_alt = (uint32_t*)take(4 * N);
    w->vals3 = (uint32_t*)take(4 * N);
    w->overflow = (int*)take(4);
    w->hist = (uint32_t*)take(4 * 256 * (size_t)tiles);
    w->totals = (uint32_t*)take(4 * 256);
    w->box_ord = (int*)take(16);
    w->seg_off = (int*)take(8);
    w->tree.left = (int*)take(4 * N);
    w->tree.right = (int*)take(4 * N);
    w->tree.parent = (int*)take(4 * N);
    w->tree.leaf_parent = (int*)take(4 * N);
    w->tree.split = (int*)take(4 * N);
    w->tree.first = (int*)take(4 * N);
    w->tree.last = (int*)take(4 * N);
    w->counter = (int*)take(4 * N);
    w->tree.climb = (int4*)take(16 * N);
    w->sums.s0 = (float4*)take(16 * N);
    w->sums.s1 = (float4*)take(16 * N);
    w->sx = (float*)take(4 * N);
    w->sy = (float*)take(4 * N);
    w->sm = (float*)take(4 * N);
    w->ncell = (int*)take(4 * N);
    w->cbase = (int*)take(4 * N);
    w->bsum = (int*)take(4 * (size_t)nb);
    w->total = (int*)take(4);
    w->qa = (int*)take(4 * M);
    w->qb = (int*)take(4 * M);
    w->qcount = (int*)take(12);
    w->rec.A = (float4*)take(16 * kRecStride * N);  // A and D interleaved
    w->rec.B = nullptr;
    w->rec.C = (int4*)take(16 * N);
    w->rec.D = reinterpret_cast<int4*>(w->rec.A) + 1;
    w->flist = (int*)take(4 * (size_t)num_supers((int)N) * kFrontierCap);
    w->fcount = (int2*)take(8 * (size_t)num_supers((int)N));
    w->inter = (unsigned long long*)take(8);
    w->work = (int*)take(4);
    w->status = (int*)take(4);
    w->tiles = tiles;
    w->cap = N;
    w->mcap = M;
    if (cudaMemset(w->status, 0, 4) != cudaSuccess) return nullptr;
    return w;
}

int blocks_for(long long n, int t) { return (int)std::max<long long>(1, (n + t - 1) / t); }

// ------------------------------------------------------------------ simple kernels

__global__ void k_c_setdraw(float* ptr, const float* x, const float* y, int n) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ptr[2 * i] = x[i];
        ptr[2 * i + 1] = y[i];
    }
}

__global__ void k_c_reset(int* mutex, float* x, float* y, float* mass, int* count, int* start,
                          int* sorted, int* child, int* index, float* left, float* right,
                          float* bottom, float* top, int n, int m, int child16) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) {
        if (child16) {  // one 16-byte store when the caller's array allows it
            reinterpret_cast<int4*>(child)[i] = make_int4(-1, -1, -1, -1);
        } else {
            child[4 * i] = -1;
            child[4 * i + 1] = -1;
            child[4 * i + 2] = -1;
            child[4 * i + 3] = -1;
        }
        if (i < n) {
            count[i] = 1;
        } else {
            x[i] = 0.0f;
            y[i] = 0.0f;
            mass[i] = 0.0f;
            count[i] = 0;
        }
        start[i] = -1;
        sorted[i] = 0;
    }
    if (i == 0) {
        *mutex = 0;
        *index = n;
        *left = 0.0f;
        *right = 0.0f;
        *bottom = 0.0f;
        *top = 0.0f;
    }
}

__device__ __forceinline__ void atomic_min_f(float* a, float v) {
    if (v >= 0.0f)
        atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else
        atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* a, float v) {
    if (v >= 0.0f)
        atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else
        atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

__global__ void __launch_bounds__(256) k_c_bbox(const float* x, const float* y, int n, float* left,
                                                float* right, float* bottom, float* top,
                                                int* status) {
    pdl_wait();
    float l = x[0], r = x[0], b = y[0], t = y[0];
    bool bad = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float xv = x[i], yv = y[i];
        bad |= !isfinite(xv) || !isfinite(yv);
        l = fminf(l, xv);
        r = fmaxf(r, xv);
        b = fminf(b, yv);
        t = fmaxf(t, yv);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        l = fminf(l, __shfl_xor_sync(kFull, l, o));
        r = fmaxf(r, __shfl_xor_sync(kFull, r, o));
        b = fminf(b, __shfl_xor_sync(kFull, b, o));
        t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
    }
    __shared__ float s[4][8];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][w] = l;
        s[1][w] = r;
        s[2][w] = b;
        s[3][w] = t;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, ST_NONFINITE);
    if (threadIdx.x == 0) {
        for (int k = 1; k < 8; ++k) {
            l = fminf(l, s[0][k]);
            r = fmaxf(r, s[1][k]);
            b = fminf(b, s[2][k]);
            t = fmaxf(t, s[3][k]);
        }
        l = fminf(l, s[0][0]);
        r = fmaxf(r, s[1][0]);
        b = fminf(b, s[2][0]);
        t = fmaxf(t, s[3][0]);
        // merged into the caller's values, which ResetArrays set to 0 (kernels.cu:108-111)
        atomic_min_f(left, l);
        atomic_max_f(right, r);
        atomic_min_f(bottom, b);
        atomic_max_f(top, t);
    }
}

__global__ void k_c_box_to_ord(const float* left, const float* right, const float* bottom,
                               const float* top, int* box_ord, int* seg_off, int n,
                               int* overflow) {
    pdl_wait();
    *overflow = 0;  // the run overflow flag of the sort that follows
    box_ord[0] = f2ord(*left);
    box_ord[1] = f2ord(*right);
    box_ord[2] = f2ord(*bottom);
    box_ord[3] = f2ord(*top);
    seg_off[0] = 0;
    seg_off[1] = n;
}

__global__ void k_c_gather3(int n, const uint32_t* perm, const float* x, const float* y,
                            const float* m, float* sx, float* sy, float* sm, int* counter) {
    pdl_wait();
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        counter[j] = 0;  // the moments' arrival counters
        uint32_t i = perm[j];
        sx[j] = x[i];
        sy[j] = y[i];
        sm[j] = m[i];
    }
}

// cells of the reference tree owned by each branching node: its chain of
// single-child cells and itself (the root node owns levels 1..L)
__global__ void k_c_ncells(int n, const int* split, const int* parent, int* ncell) {
    pdl_wait();
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    int sp = split[q], c = 0;
    if (sp >= 0) {
        int pa = parent[q];
        if (!(pa >= 0 && merged_into(sp, split[pa]))) {
            int L = sp >> 1;
            c = pa >= 0 ? L - (split[pa] >> 1) : L;
        }
    }
    ncell[q] = c;
}

// exclusive scan of n ints in blocks of 1024
__global__ void __launch_bounds__(1024) k_c_scan_block(const int* in, int* out, int* bsum, int n) {
    pdl_wait();
    __shared__ uint32_t tmp[32];
    int i = blockIdx.x * 1024 + threadIdx.x;
    uint32_t v = i < n ? (uint32_t)in[i] : 0u;
    uint32_t tot;
    uint32_t ex = block_excl_scan<1024>(v, &tot, tmp);
    if (i < n) out[i] = (int)ex;
    if (threadIdx.x == 0) bsum[blockIdx.x] = (int)tot;
}

__global__ void __launch_bounds__(1024) k_c_scan_top(int* bsum, int nb, int* total) {
    pdl_wait();
    __shared__ uint32_t tmp[32];
    uint32_t run = 0;
    for (int base = 0; base < nb; base += 1024) {
        int i = base + threadIdx.x;
        uint32_t v = i < nb ? (uint32_t)bsum[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan<1024>(v, &tot, tmp);
        if (i < nb) bsum[i] = (int)(run + ex);
        run += tot;
    }
    if (threadIdx.x == 0) *total = (int)run;
}

__global__ void k_c_scan_add(int* out, const int* bsum, int n) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / 1024];
}

__device__ __forceinline__ int digit_at(uint64_t key, int level) {  // level 1..32
    return (int)((key >> (64 - 2 * level)) & 3ull);
}

__global__ void k_c_materialize(int n, int m, TreePtrs t, const uint64_t* skeys,
                                const uint32_t* perm, const int* cbase, const int* total,
                                NodeSums sums, int* child, int* count, int* start, float* x,
                                float* y, float* mass, int* index, int* status) {
    pdl_wait();
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int tot = *total;
    if ((long long)n + tot > (long long)m) {
        if (q == 0) atomicOr(status, ST_CAPACITY);
        return;
    }
    if (q == 0) *index = n + tot;
    int sp = t.split[q];
    if (sp < 0) return;
    int pa = t.parent[q];
    if (pa >= 0 && merged_into(sp, t.split[pa])) return;
    int L = sp >> 1;
    if (L >= 32) {  // equal keys: no 33rd level to place them on
        atomicOr(status, ST_DUP);
        return;
    }
    int Lp = pa >= 0 ? (t.split[pa] >> 1) : 0;
    int nc = L - Lp;
    int b0 = n + cbase[q];
    uint64_t key = skeys[t.first[q]];
    int cnt = t.last[q] - t.first[q] + 1;
    const float4 s0 = sums.s0[q];
    const float M = s0.x, MX = s0.y, MY = s0.z;
    for (int k = 0; k < nc; ++k) {  // chain cells, then the node's own cell
        int id = b0 + k;
        int lev = Lp + 1 + k;
        if (k + 1 < nc) child[4 * id + digit_at(key, lev + 1)] = id + 1;
        count[id] = cnt;
        start[id] = -1;
        x[id] = MX;
        y[id] = MY;
        mass[id] = M;
    }
    if (pa < 0 && L >= 1) child[digit_at(key, 1)] = b0;  // root slot -> top of the chain
    const int own = nc > 0 ? b0 + nc - 1 : 0;
    int lr[2] = {t.left[q], t.right[q]};
    for (int s = 0; s < 2; ++s) {
        int c = lr[s];
        int cs[2] = {c, kNoChild};
        if (c >= 0 && merged_into(t.split[c], sp)) {
            cs[0] = t.left[c];
            cs[1] = t.right[c];
        }
        for (int u = 0; u < 2; ++u) {
            int cc = cs[u];
            if (cc == kNoChild) continue;
            if (cc < 0) {
                int b = ~cc;
                child[4 * own + digit_at(skeys[b], L + 1)] = (int)perm[b];
            } else {
                child[4 * own + digit_at(skeys[t.first[cc]], L + 1)] = n + cbase[cc];
            }
        }
    }
}

// SortParticles from the last build (kernels.cu:299-335 computes the same by a
// depth-first pass over the cells).  At every level a body's child index is
// (x < mid) + 2 (y < mid) (kernels.cu:144-157), the digit its key holds
// there, and every leaf holds one body, so the depth-first order over child
// indices 0..3 is ascending key order: sorted[] is the sort permutation, and
// a cell's start is the first sorted position of its bodies, the first body
// of the tree node whose chain of cells (k_c_materialize) holds it.  The
// same guards as k_c_materialize: nothing for cells it did not make.
__global__ void k_c_sort_from_build(int n, int m, TreePtrs t, const uint32_t* perm,
                                    const int* cbase, const int* total, int* start, int* sorted) {
    pdl_wait();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    sorted[q] = (int)perm[q];
    if ((long long)n + *total > (long long)m) return;  // ST_CAPACITY
    const int sp = t.split[q];
    if (sp < 0) return;
    const int pa = t.parent[q];
    if (pa >= 0 && merged_into(sp, t.split[pa])) return;
    const int L = sp >> 1;
    if (L >= 32) return;  // ST_DUP
    const int Lp = pa >= 0 ? (t.split[pa] >> 1) : 0;
    const int b0 = n + cbase[q], first = t.first[q];
    for (int k = 0; k < L - Lp; ++k) start[b0 + k] = first;
}

__global__ void k_c_com(float* x, float* y, const float* mass, const int* index, int n) {
    pdl_wait();
    int end = *index;
    for (int i = n + blockIdx.x * blockDim.x + threadIdx.x; i < end; i += gridDim.x * blockDim.x) {
        x[i] = __fdiv_rn(x[i], mass[i]);  // kernels.cu:283-284
        y[i] = __fdiv_rn(y[i], mass[i]);
    }
}

// sorted[]/start[] by levels from the root slot, one block (kernels.cu:292-336)
__global__ void __launch_bounds__(1024) k_c_sort(const int* count, int* start, int* sorted,
                                                 const int* child, int n, int mlimit, int* qa,
                                                 int* qb, int cap, int* status) {
    __shared__ int s_in, s_out, s_bad;
    if (threadIdx.x == 0) {
        int s = 0, k = 0;
        s_bad = 0;
        for (int i = 0; i < 4; ++i) {
            int node = child[i];
            if (node >= n) {
                if (node >= mlimit || k >= cap) {
                    s_bad = 1;
                    continue;
                }
                start[node] = s;
                s += count[node];
                qa[k++] = node;
            } else if (node >= 0) {
                if (s < n) sorted[s] = node;
                ++s;
            }
        }
        s_in = k;
    }
    __syncthreads();
    int* in = qa;
    int* out = qb;
    int level = 0;
    for (; level < 128; ++level) {
        const int cin = s_in;
        if (cin == 0) break;
        if (threadIdx.x == 0) s_out = 0;
        __syncthreads();
        for (int tt = threadIdx.x; tt < cin; tt += blockDim.x) {
            int cell = in[tt];
            int s = start[cell];
            for (int i = 0; i < 4; ++i) {
                int node = child[4 * cell + i];
                if (node >= n) {
                    if (node >= mlimit) {
                        s_bad = 1;
                        continue;
                    }
                    start[node] = s;
                    s += count[node];
                    int pos = atomicAdd(&s_out, 1);
                    if (pos < cap)
                        out[pos] = node;
                    else
                        s_bad = 1;
                } else if (node >= 0) {
                    if (s >= 0 && s < n)
                        sorted[s] = node;
                    else
                        s_bad = 1;
                    ++s;
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_in = min(s_out, cap);
        int* tmp = in;
        in = out;
        out = tmp;
        __syncthreads();
    }
    if (threadIdx.x == 0 && (s_bad || level == 128)) atomicOr(status, ST_CAPACITY);
}

// The same assignment over the whole device: a cooperative grid of one block
// per SM (fewer blocks make each grid barrier cheaper, and a level rarely holds
// more cells than the grid has threads) takes each level's cells in a grid-stride loop and appends the next
// level's cells with a global counter; one grid barrier per level.  A cell's
// start and its bodies' places depend only on its parent's start and the
// counts of its earlier siblings, so the result is the single block's (and the
// reference's, kernels.cu:292-336) whatever the order of a level's cells.
// Level counters rotate over three words: level L reads qcount[L % 3], fills
// qcount[(L + 1) % 3] and clears qcount[(L + 2) % 3], which nobody reads or
// writes during level L.
constexpr int kSortGridThreads = 512;
__global__ void __launch_bounds__(kSortGridThreads) k_c_sort_grid(const int* count, int* start, int* sorted,
                                                     const int* child, int n, int mlimit, int* qa,
                                                     int* qb, int cap, int* qcount, int* status,
                                                     int child16) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long gsize = (long long)gridDim.x * blockDim.x;
    bool bad = false;
    if (gid == 0) {
        int s = 0, k = 0;
        for (int i = 0; i < 4; ++i) {
            const int node = child[i];
            if (node >= n) {
                if (node >= mlimit || k >= cap) {
                    bad = true;
                    continue;
                }
                start[node] = s;
                s += count[node];
                qa[k++] = node;
            } else if (node >= 0) {
                if (s < n) sorted[s] = node;
                ++s;
            }
        }
        qcount[0] = k;
        qcount[1] = 0;
        qcount[2] = 0;
    }
    grid.sync();
    int* in = qa;
    int* out = qb;
    int level = 0;
    for (; level < 128; ++level) {
        const int cin = min(*(volatile int*)(qcount + level % 3), cap);
        if (cin == 0) break;  // the same value in every thread: read after the barrier
        int* next = qcount + (level + 1) % 3;
        if (gid == 0) qcount[(level + 2) % 3] = 0;
        for (long long tt = gid; tt < cin; tt += gsize) {
            int cell = __ldcg(in + tt);
            int s = __ldcg(start + cell);
            int ch[4];
            // a cell whose only child is a cell (the chains of the uncompressed
            // tree) gives that child its own start: followed down in this
            // thread, not level by level
            for (int chain = 0;; ++chain) {
                if (child16) {  // child[] 16-byte aligned: the four slots in one load
                    const int4 c4 = *reinterpret_cast<const int4*>(child + 4 * (size_t)cell);
                    ch[0] = c4.x, ch[1] = c4.y, ch[2] = c4.z, ch[3] = c4.w;
                } else {
#pragma unroll
                    for (int i = 0; i < 4; ++i) ch[i] = child[4 * (size_t)cell + i];
                }
                int only = -1, used = 0;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (ch[i] >= 0) {
                        only = ch[i];
                        ++used;
                    }
                }
                if (used != 1 || only < n || only >= mlimit || chain == 128) break;
                start[only] = s;
                cell = only;
            }
            int cnt[4], ncell = 0;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const bool is_cell = ch[i] >= n && ch[i] < mlimit;
                cnt[i] = is_cell ? count[ch[i]] : 0;
                ncell += is_cell;
            }
            int pos = ncell ? atomicAdd(next, ncell) : 0;  // this cell's slots in the next level
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int node = ch[i];
                if (node >= n) {
                    if (node >= mlimit) {
                        bad = true;
                        continue;
                    }
                    start[node] = s;
                    s += cnt[i];
                    if (pos < cap)
                        out[pos] = node;
                    else
                        bad = true;
                    ++pos;
                } else if (node >= 0) {
                    if (s >= 0 && s < n)
                        sorted[s] = node;
                    else
                        bad = true;
                    ++s;
                }
            }
        }
        grid.sync();
        int* tmp = in;
        in = out;
        out = tmp;
    }
    if (bad || (gid == 0 && level == 128)) atomicOr(status, ST_CAPACITY);
}

// The warp-vote walk on the reference layout (kernels.cu:340-435), with the
// engine's REFERENCE-mode machinery (k_walk_vote): lanes test up to 32 stack cells at once, each against the
// whole group (dp <= min over the group's bodies of r_b: the group box's
// nearest point bounds that minimum from below, the four extreme bodies from
// above, and the exact minimum is taken only in between), accepted cells and
// the bodies of opened cells are staged and evaluated 32 at a time with the
// reference's arithmetic (kernels.cu:403-411).  The stack holds cells to test
// with the dp of their level (kernels.cu:376, 395); the root's children are
// opened without a test (kernels.cu:370-388).  Only the summation order
// differs from the reference's.
template <int WARPS, int STACK>
__global__ void __launch_bounds__(WARPS * 32) k_c_forces_vote(
    const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ mass,
    const int* __restrict__ sorted, const int* __restrict__ child, const float* left,
    const float* right, int n, int mlimit, float theta, float eps2, float* ax, float* ay,
    int* status) {
    pdl_wait();
    __shared__ int s_node[WARPS][STACK];
    __shared__ float s_dp[WARPS][STACK];
    __shared__ float4 s_stage[WARPS][32];
    __shared__ int s_clist[WARPS][64];
    __shared__ int s_blist[WARPS][32 + 4 * 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    int* stack = s_node[w];
    float* sdp = s_dp[w];
    float4* stage = s_stage[w];
    int* clist = s_clist[w];
    int* blist = s_blist[w];
    const float radius = __fmul_rn(__fsub_rn(*right, *left), 0.5f);  // kernels.cu:349
    const float dp1 = __fdiv_rn(__fmul_rn(radius, radius), theta);    // :376
    const int groups = (n + 31) / 32;
    for (int g = blockIdx.x * WARPS + w; g < groups; g += gridDim.x * WARPS) {
        const int j = 32 * g + lane;
        const bool valid = j < n;
        const int b = sorted[valid ? j : 32 * g];  // invalid lanes mirror the group's first body
        const float px = x[b], py = y[b];
        float gx0 = px, gx1 = px, gy0 = py, gy1 = py;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx0 = fminf(gx0, __shfl_xor_sync(kFull, gx0, o));
            gx1 = fmaxf(gx1, __shfl_xor_sync(kFull, gx1, o));
            gy0 = fminf(gy0, __shfl_xor_sync(kFull, gy0, o));
            gy1 = fmaxf(gy1, __shfl_xor_sync(kFull, gy1, o));
        }
        float ext[4];  // y at min/max x, x at min/max y
        {
            const float key[4] = {gx0, gx1, gy0, gy1};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned hit = __ballot_sync(kFull, (q < 2 ? px : py) == key[q]);
                ext[q] = __shfl_sync(kFull, q < 2 ? py : px, __ffs(hit) - 1);
            }
        }
        float acx = 0.0f, acy = 0.0f;
        bool bad = false;
        int top = 0, ccnt = 0, bcnt = 0;
        auto interact = [&](int k) {
            for (int e = 0; e < k; ++e) {
                const float4 c = stage[e];
                float dx, dy;
                const float r = ref_r(c.x, c.y, px, py, eps2, &dx, &dy);
                const float ri = rsqrtf(r);
                const float f = c.z * ri * ri * ri;
                acx = fmaf(f, dx, acx);
                acy = fmaf(f, dy, acy);
            }
        };
        auto flush_cells = [&](int k) {  // the last k entries of clist
            __syncwarp();
            if (lane < k) {
                const int c = clist[ccnt - k + lane];
                stage[lane] = make_float4(x[c], y[c], mass[c], 0.0f);
            }
            __syncwarp();
            interact(k);
            ccnt -= k;
        };
        auto flush_bodies = [&](int k) {
            __syncwarp();
            if (lane < k) {
                const int c = blist[bcnt - k + lane];
                stage[lane] = make_float4(x[c], y[c], mass[c], 0.0f);
            }
            __syncwarp();
            interact(k);
            bcnt -= k;
        };
        // the root's children, opened without a test: their bodies interact,
        // their cells' children go to the body list or the stack (dp1 / 4)
        __syncwarp();
        if (lane == 0) {
            for (int i = 0; i < 4; ++i) {
                const int c = child[i];
                if (c >= 0 && c < n) {
                    blist[bcnt++] = c;
                } else if (c >= n && c < mlimit) {
                    for (int q = 0; q < 4; ++q) {
                        const int cc = child[4 * c + q];
                        if (cc < 0) continue;
                        if (cc >= mlimit) {
                            bad = true;
                        } else if (cc < n) {
                            blist[bcnt++] = cc;
                        } else {
                            stack[top] = cc;
                            sdp[top] = 0.25f * dp1;  // :395
                            ++top;
                        }
                    }
                }
            }
        }
        top = __shfl_sync(kFull, top, 0);
        bcnt = __shfl_sync(kFull, bcnt, 0);
        bad = __shfl_sync(kFull, bad ? 1 : 0, 0) != 0;
        __syncwarp();
        int rounds = 0;
        while (top > 0 && !bad) {
            if (++rounds > kMaxWalkRounds) {  // far beyond any valid tree (a cycle in child[])
                bad = true;
                break;
            }
            int k = min(32, top);
            if (top + 3 * k > STACK) {  // pop k, push <= 4k
                k = max((STACK - top) / 3, 0);
                if (k == 0) {
                    bad = true;
                    break;
                }
            }
            __syncwarp();
            const int node = lane < k ? stack[top - 1 - lane] : -1;
            const float dp = lane < k ? sdp[top - 1 - lane] : 0.0f;
            top -= k;
            float cx = 0.0f, cy = 0.0f;
            bool acc = false, need = false;
            if (node >= 0) {
                cx = x[node];
                cy = y[node];
                // lower bound of min_b r_b: the box's nearest point
                const float nx = fminf(fmaxf(cx, gx0), gx1), ny = fminf(fmaxf(cy, gy0), gy1);
                if (dp <= ref_r_only(cx, cy, nx, ny, eps2)) {
                    acc = true;
                } else {
                    float rhi = ref_r_only(cx, cy, gx0, ext[0], eps2);
                    rhi = fminf(rhi, ref_r_only(cx, cy, gx1, ext[1], eps2));
                    rhi = fminf(rhi, ref_r_only(cx, cy, ext[2], gy0, eps2));
                    rhi = fminf(rhi, ref_r_only(cx, cy, ext[3], gy1, eps2));
                    need = dp <= rhi;
                }
            }
            unsigned nm = __ballot_sync(kFull, need);
            while (nm) {  // the exact minimum over the group's bodies, one cell at a time
                const int src = __ffs(nm) - 1;
                nm &= nm - 1;
                const float sx = __shfl_sync(kFull, cx, src), sy = __shfl_sync(kFull, cy, src);
                float r = ref_r_only(sx, sy, px, py, eps2);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) r = fminf(r, __shfl_xor_sync(kFull, r, o));
                if (lane == src) acc = dp <= r;
            }
            const unsigned mc = __ballot_sync(kFull, acc);
            if (acc) clist[ccnt + __popc(mc & lt)] = node;
            ccnt += __popc(mc);
            const bool open = node >= 0 && !acc;
            int cs[4] = {-1, -1, -1, -1};
            if (open)
#pragma unroll
                for (int q = 0; q < 4; ++q) cs[q] = child[4 * node + q];
            int nb = 0, nn = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (cs[q] >= mlimit) {
                    bad = true;
                    cs[q] = -1;
                }
                nb += (cs[q] >= 0 && cs[q] < n);
                nn += (cs[q] >= n);
            }
            int tot;
            const int off = warp_excl_scan(nb | (nn << 16), &tot);
            __syncwarp();  // every lane has read its stack slot before children overwrite it
            if (open) {
                int* bw = blist + bcnt + (off & 0xffff);
                int* nw = stack + top + (off >> 16);
                float* dw = sdp + top + (off >> 16);
                const float cdp = 0.25f * dp;  // :395
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (cs[q] < 0) continue;
                    if (cs[q] < n) {
                        *bw++ = cs[q];  // bodies always interact (:395-399)
                    } else {
                        *nw++ = cs[q];
                        *dw++ = cdp;
                    }
                }
            }
            bcnt += tot & 0xffff;
            top += tot >> 16;
            bad = __any_sync(kFull, bad);
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
            while (bcnt >= 32) flush_bodies(32);
        }
        if (ccnt > 0) flush_cells(ccnt);
        if (bcnt > 0) flush_bodies(bcnt);
        if (bad && lane == 0) atomicOr(status, ST_STACK);
        if (valid) {
            ax[b] = acx;  // :428-429
            ay[b] = acy;
        }
    }
}

__global__ void k_c_integrate(float* x, float* y, float* vx, float* vy, const float* ax,
                              const float* ay, int n, float dt, float ddt) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float v = __fadd_rn(vx[i], __fmul_rn(dt, ax[i]));  // kernels.cu:529-533
        float u = __fadd_rn(vy[i], __fmul_rn(dt, ay[i]));
        vx[i] = v;
        vy[i] = u;
        x[i] = __fadd_rn(x[i], __fmul_rn(ddt, v));
        y[i] = __fadd_rn(y[i], __fmul_rn(ddt, u));
    }
}

int fetch_status(Workspace* w) {
    int bits = 0;
    if (!w) return BH_OK;
    if (cudaMemcpy(&bits, w->status, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BH_ERR_CUDA;
    cudaMemset(w->status, 0, 4);
    if (bits & ST_NONFINITE) return BH_ERR_NONFINITE;
    if (bits & ST_DUP) return BH_ERR_DUPLICATE_KEYS;
    if (bits & ST_STACK) return BH_ERR_STACK;
    if (bits & ST_CAPACITY) return BH_ERR_CAPACITY;
    if (bits & ST_TREE) return BH_ERR_TREE;
    return BH_OK;
}

// BuildQuadTree's launch sequence on the scratch of w, which must hold n
// bodies (shared by BuildQuadTree and BuildQuadTreeNoAlloc).  Keys of the
// bodies in the caller's box; the engine's sort: stable passes over the high
// word (3, or 4 above 2^21 bodies), then each run of equal high words put in
// whole-key order, and, only when a run is longer than kFixupRun, the 8-pass
// sort of the whole key (its kernels return at once unless the fixup raised
// the flag); the radix tree and its node sums, then the tree written out in
// the reference layout (child, count, start, cell x/y/mass, *index).
cudaError_t enqueue_build(Workspace& w, float* x, float* y, float* mass, int* count, int* start,
                          int* child, int* index, float* left, float* right, float* bottom,
                          float* top, int n, int m, cudaStream_t st) {
    const int nb = blocks_for(n, 256);
    cudaError_t e = launch_pdl(k_c_box_to_ord, 1, 1, 0, st, (const float*)left, (const float*)right,
                               (const float*)bottom, (const float*)top, w.box_ord, w.seg_off, n,
                               w.overflow);
    if (e != cudaSuccess) return e;
    Segs segs{1, w.seg_off, nullptr};
    // the kernels that wait for their predecessor (pdl_wait) are launched with
    // programmatic serialisation: each one's launch overlaps the previous one's
    // tail, which matters for the flag-gated full sort that returns at once
    e = launch_pdl(k_keys, nb, 256, 0, st, x, y, n, segs, (const int*)w.box_ord, w.keys, w.vals);
    if (e != cudaSuccess) return e;
    const int tiles = (n + kSortTile - 1) / kSortTile;
    auto pass = [&](const uint64_t* ki, const uint32_t* vi, uint64_t* ko, uint32_t* vo, int shift,
                    const int* only_if) {
        cudaError_t r = launch_pdl(k_radix_hist, tiles, kSortThreads, 0, st, ki, vi, n, shift, 0,
                                   (const int*)nullptr, w.hist, tiles, only_if);
        if (r == cudaSuccess)
            r = launch_pdl(k_radix_scan, 256, kSortThreads, 0, st, w.hist, tiles, w.totals, only_if);
        if (r == cudaSuccess)
            r = launch_pdl(k_radix_scatter, tiles, kSortThreads, 0, st, ki, vi, ko, vo, n, shift, 0,
                           (const int*)nullptr, (const uint32_t*)w.hist, (const uint32_t*)w.totals,
                           tiles, only_if);
        return r;
    };
    // high word: keys -> ... -> keys3, the fixup into keys_alt; the full sort
    // (if flagged) keys -> keys3 / keys_alt alternately -> keys_alt
    const int hp = n <= kShortSortMax ? 3 : 4;
    {
        const uint64_t* ki = w.keys;
        const uint32_t* vi = w.vals;
        for (int ps = 0; ps < hp; ++ps) {
            const bool to_alt = ((hp - 1 - ps) & 1) != 0;
            uint64_t* ko = to_alt ? w.keys_alt : w.keys3;
            uint32_t* vo = to_alt ? w.vals_alt : w.vals3;
            e = pass(ki, vi, ko, vo, 64 - 8 * (hp - ps), nullptr);
            if (e != cudaSuccess) return e;
            ki = ko;
            vi = vo;
        }
    }
    e = launch_pdl(k_sort_fixup, nb, 256, 0, st, n, 64 - 8 * hp, (const uint64_t*)w.keys3,
                   (const uint32_t*)w.vals3, w.keys_alt, w.vals_alt, w.overflow,
                   (cudaGraphConditionalHandle)0, 0, (int*)nullptr, 0);
    if (e != cudaSuccess) return e;
    if (!launch_full_sort_grid(w.keys, w.vals, w.keys_alt, w.vals_alt, w.keys3, w.vals3, n, w.hist,
                               w.totals, tiles, w.overflow, st, &e)) {
        const uint64_t* ki = w.keys;
        const uint32_t* vi = w.vals;
        for (int ps = 0; ps < 8; ++ps) {
            uint64_t* ko = (ps & 1) ? w.keys_alt : w.keys3;
            uint32_t* vo = (ps & 1) ? w.vals_alt : w.vals3;
            e = pass(ki, vi, ko, vo, 8 * ps, w.overflow);
            if (e != cudaSuccess) return e;
            ki = ko;
            vi = vo;
        }
    }
    if (e != cudaSuccess) return e;
    uint64_t* ka = w.keys_alt;
    uint32_t* va = w.vals_alt;
    e = launch_pdl(k_c_gather3, nb, 256, 0, st, n, (const uint32_t*)va, (const float*)x,
                   (const float*)y, (const float*)mass, w.sx, w.sy, w.sm, w.counter);
    if (e == cudaSuccess)
        e = launch_pdl(k_build, nb, 256, 0, st, (const uint64_t*)ka, n, segs, w.tree, w.status);
    if (e == cudaSuccess)
        e = launch_pdl(k_moments, (n + kMomentsThreads - 1) / kMomentsThreads, kMomentsThreads, 0,
                       st, n, 0, (const float*)w.sx, (const float*)w.sy, (const float*)w.sm,
                       (const int4*)w.tree.climb, (const int*)w.tree.leaf_parent, w.counter, w.sums,
                       w.status);
    if (e != cudaSuccess) return e;
    // the cell numbering and the reference layout, each kernel launched while
    // its predecessor drains (pdl_wait)
    const int sb = blocks_for(n, 1024);
    e = launch_pdl(k_c_ncells, nb, 256, 0, st, n, (const int*)w.tree.split,
                   (const int*)w.tree.parent, w.ncell);
    if (e == cudaSuccess)
        e = launch_pdl(k_c_scan_block, sb, 1024, 0, st, (const int*)w.ncell, w.cbase, w.bsum, n);
    if (e == cudaSuccess) e = launch_pdl(k_c_scan_top, 1, 1024, 0, st, w.bsum, sb, w.total);
    if (e == cudaSuccess) e = launch_pdl(k_c_scan_add, nb, 256, 0, st, w.cbase, (const int*)w.bsum, n);
    if (e == cudaSuccess)
        e = launch_pdl(k_c_materialize, nb, 256, 0, st, n, m, w.tree, (const uint64_t*)ka,
                       (const uint32_t*)va, (const int*)w.cbase, (const int*)w.total, w.sums, child,
                       count, start, x, y, mass, index, w.status);
    return e;
}

}  // namespace

extern "C" {

void bh_compat_set_constants(float theta, float eps2) {
    if (theta > 0.0f && eps2 > 0.0f) {
        g_set.theta = theta;
        g_set.eps2 = eps2;
    } else {
        record(BH_ERR_ARG);
    }
}

void bh_compat_set_stream(void* stream) { g_set.stream = (cudaStream_t)stream; }

int bh_compat_status(void) {
    cudaError_t e = cudaStreamSynchronize(g_set.stream);
    if (e != cudaSuccess) record(cuda_fail(e, "compat stream"));
    const int cur = current_device();
    std::lock_guard<std::mutex> lk(g_ws_mu);
    for (auto& w : g_ws)
        if (w->device == cur && w->base) record(fetch_status(w.get()));
    return t_status;
}

void bh_compat_clear_status(void) { t_status = BH_OK; }

void bh_compat_release(void) {
    std::lock_guard<std::mutex> lk(g_ws_mu);
    for (auto& w : g_ws)
        if (w->base) cudaFree(w->base);
    g_ws.clear();
    for (auto& l : g_layout) l = Layout{};
}

}  // extern "C"

namespace ssg {

void compat_SetDrawArray(float* ptr, float* x, float* y, int n) {
    if (n <= 0) return;
    record_cuda(launch_pdl(k_c_setdraw, blocks_for(n, 256), 256, 0, g_set.stream, ptr,
                           (const float*)x, (const float*)y, n),
                "SetDrawArray");
}

void compat_ResetArrays(int* mutex, float* x, float* y, float* mass, int* count, int* start, int* sorted,
                 int* child, int* index, float* left, float* right, float* bottom, float* top,
                 int n, int m) {
    if (n < 1 || m < n) {
        record(BH_ERR_ARG);
        return;
    }
    const int child16 = (reinterpret_cast<uintptr_t>(child) & 15) == 0 ? 1 : 0;
    record_cuda(launch_pdl(k_c_reset, blocks_for(m, 256), 256, 0, g_set.stream, mutex, x, y, mass,
                           count, start, sorted, child, index, left, right, bottom, top, n, m,
                           child16),
                "ResetArrays");
}

void compat_ComputeBoundingBox(int* mutex, float* x, float* y, float* left, float* right, float* bottom,
                        float* top, int n) {
    (void)mutex;
    if (n < 1) {
        record(BH_ERR_ARG);
        return;
    }
    Workspace* w = workspace(1, 1);
    if (!w) {
        record(BH_ERR_NOMEM);
        return;
    }
    int blocks = std::min(blocks_for(n, 256), 1024);
    record_cuda(launch_pdl(k_c_bbox, blocks, 256, 0, g_set.stream, (const float*)x, (const float*)y,
                           n, left, right, bottom, top, w->status),
                "ComputeBoundingBox");
}

void compat_BuildQuadTree(float* x, float* y, float* mass, int* count, int* start, int* child, int* index,
                   float* left, float* right, float* bottom, float* top, int n, int m) {
    if (n < 1 || m < n) {
        record(BH_ERR_ARG);
        return;
    }
    set_built(Built{});  // none until the tree below is enqueued
    if (n == 1) return;  // a lone body: no cells, *index stays n
    Workspace* w = workspace((size_t)n, (size_t)m);
    if (!w) {
        record(BH_ERR_NOMEM);
        return;
    }
    set_layout(child, m);
    const cudaError_t e = enqueue_build(*w, x, y, mass, count, start, child, index, left, right,
                                        bottom, top, n, m, g_set.stream);
    record_cuda(e, "BuildQuadTree");
    set_built(e == cudaSuccess ? Built{child, n, m, w, w->gen} : Built{});
}

void compat_ComputeCentreOfMass(float* x, float* y, float* mass, int* index, int n) {
    record_cuda(launch_pdl(k_c_com, 1024, 256, 0, g_set.stream, x, y, (const float*)mass,
                           (const int*)index, n),
                "ComputeCentreOfMass");
}

void compat_SortParticles(int* count, int* start, int* sorted, int* child, int* index, int n) {
    (void)index;
    if (n < 1) {
        record(BH_ERR_ARG);
        return;
    }
    {
        // the arrays of the last BuildQuadTree on this device, its workspace
        // not grown since: sorted[] and start[] from that build
        Built b;
        const int dev = current_device();
        if (dev >= 0 && dev < kMaxDevices) {
            std::lock_guard<std::mutex> lk(g_ws_mu);
            b = g_built[dev];
        }
        if (b.child == child && b.n == n && b.w && b.w->base && b.w->gen == b.gen) {
            const Workspace& w = *b.w;
            record_cuda(launch_pdl(k_c_sort_from_build, blocks_for(n, 256), 256, 0, g_set.stream, n,
                                   b.m, w.tree, (const uint32_t*)w.vals_alt, (const int*)w.cbase,
                                   (const int*)w.total, start, sorted),
                        "SortParticles");
            return;
        }
    }
    // queues for every cell of the layout, on the current device's workspace
    const int mlimit = layout_m(child, n);
    Workspace* w = workspace(1, (size_t)mlimit);
    if (!w) {
        record(BH_ERR_NOMEM);
        return;
    }
    // one grid over the device (cooperative: every block resident at once)
    static std::atomic<int> s_blocks_per_sm[kMaxDevices] = {};  // per device, read once
    const int dev = current_device();
    int bps = dev >= 0 && dev < kMaxDevices ? s_blocks_per_sm[dev].load() : 0;
    if (bps <= 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_c_sort_grid,
                                                                      kSortGridThreads, 0);
        if (e != cudaSuccess || bps < 1) bps = 0;
        if (dev >= 0 && dev < kMaxDevices) s_blocks_per_sm[dev] = bps;
    }
    if (bps < 1) {  // no cooperative grid: the single block
        k_c_sort<<<1, 1024, 0, g_set.stream>>>(count, start, sorted, child, n, mlimit, w->qa,
                                               w->qb, (int)w->mcap, w->status);
        record_cuda(cudaGetLastError(), "SortParticles");
        return;
    }
    const int* c_count = count;
    const int* c_child = child;
    int cap = (int)w->mcap;
    int child16 = (reinterpret_cast<uintptr_t>(child) & 15) == 0 ? 1 : 0;
    void* args[] = {(void*)&c_count, (void*)&start, (void*)&sorted, (void*)&c_child, (void*)&n,
                    (void*)&mlimit, (void*)&w->qa, (void*)&w->qb, (void*)&cap, (void*)&w->qcount,
                    (void*)&w->status, (void*)&child16};
    record_cuda(cudaLaunchCooperativeKernel((const void*)k_c_sort_grid, device_sms(),
                                            kSortGridThreads, args, 0, g_set.stream),
                "SortParticles");
}

// CalculateForces takes the vote walk on the last build's tree above this many
// bodies (its walk records cost one more kernel; measured on GB300, Plummer:
// 0.069 against 0.059 ms at 2^16, 0.081 against 0.092 ms at 2^17, 0.336
// against 0.439 ms at 2^20), else the walk over child[].
constexpr int kVoteForcesMinBodies = 3 << 15;

void compat_CalculateForces(float* x, float* y, float* vx, float* vy, float* ax, float* ay, float* mass,
                     int* sorted, int* child, float* left, float* right, int n, float g) {
    (void)vx;
    (void)vy;
    (void)g;  // unused in the reference too (kernels.cu:340)
    if (n < 1) {
        record(BH_ERR_ARG);
        return;
    }
    if (n > kVoteForcesMinBodies) {
        // the arrays of the last BuildQuadTree on this device, its workspace not
        // grown since: the vote walk on that build's compressed tree, bodies in
        // key order (the groups of 32 consecutive sorted[] bodies the reference
        // gives its warps, kernels.cu:342-362), the same interaction set
        Built b;
        const int dev = current_device();
        if (dev >= 0 && dev < kMaxDevices) {
            std::lock_guard<std::mutex> lk(g_ws_mu);
            b = g_built[dev];
        }
        if (b.child == child && b.n == n && b.w && b.w->base && b.w->gen == b.gen) {
            Workspace& w = *b.w;
            cudaStream_t st = g_set.stream;
            const Segs segs{1, w.seg_off, nullptr};
            const int nb = blocks_for(n, 256);
            cudaError_t e = cudaMemsetAsync(w.work, 0, sizeof(int), st);
            if (e == cudaSuccess)
                e = launch_pdl(k_records, nb, 256, 0, st, n, segs, 0, g_set.theta, 1.0f,
                               (const int*)w.box_ord, (const uint64_t*)w.keys_alt, w.tree, w.sums,
                               w.rec);
            // the vote rule's walk frontiers, one warp per 512 consecutive bodies
            constexpr int kFW = 8;
            const int nsup = num_supers(n);
            if (e == cudaSuccess)
                e = launch_pdl(k_frontier<kFW, true>, (nsup + kFW - 1) / kFW, kFW * 32, 0, st, segs,
                               nsup, (const float*)w.sx, (const float*)w.sy, (const float*)nullptr,
                               (const float4*)w.rec.A, (const int4*)w.rec.C, (const int4*)w.rec.D,
                               1, 32, 0.0f, w.flist, w.fcount, (const int*)nullptr,
                               (const int*)nullptr, (const int*)nullptr, (const int*)nullptr,
                               (int*)nullptr, (int*)nullptr, g_set.eps2);
            if (e == cudaSuccess) {
                const WalkIn in{w.sx, w.sy, nullptr, nullptr, w.sm, nullptr, nullptr,
                                reinterpret_cast<const int*>(w.vals_alt), nullptr, nullptr};
                WalkOut out{};
                out.ax = ax;
                out.ay = ay;
                const Groups gr{(n + 31) / 32, nullptr};
                const int blocks =
                    std::min(blocks_for(gr.ngroups, kVoteWarps), 16 * device_sms());
                e = launch_pdl(k_walk_vote, blocks, kVoteWarps * 32, 0, st, segs, gr, in,
                               (const float4*)w.rec.A, (const int4*)w.rec.C, g_set.eps2, 0.0f, 0.0f,
                               out, w.status, w.inter, w.work,
                               Frontier{w.flist, w.fcount, nullptr});
            }
            record_cuda(e, "CalculateForces");
            return;
        }
    }
    const int mlimit = layout_m(child, n);
    Workspace* w = workspace(1, 1);  // the current device's status word
    if (!w) {
        record(BH_ERR_NOMEM);
        return;
    }
    constexpr int W = 4, S = 1024;
    // a grid-stride loop over the warp groups: at most 16 blocks per SM
    int blocks = std::min(blocks_for((n + 31) / 32, W), 16 * device_sms());
    record_cuda(launch_pdl(k_c_forces_vote<W, S>, blocks, W * 32, 0, g_set.stream, (const float*)x,
                           (const float*)y, (const float*)mass, (const int*)sorted,
                           (const int*)child, (const float*)left, (const float*)right, n, mlimit,
                           g_set.theta, g_set.eps2, ax, ay, w->status),
                "CalculateForces");
}

void compat_IntegrateParticles(float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n,
                        float dt, float d) {
    if (n <= 0) return;
    record_cuda(launch_pdl(k_c_integrate, blocks_for(n, 256), 256, 0, g_set.stream, x, y, vx, vy,
                           (const float*)ax, (const float*)ay, n, dt, d * dt),
                "IntegrateParticles");
}

void compat_FillOutputArray(float* x, float* y, float* out, int n) {
    if (n <= 0) return;
    record_cuda(launch_pdl(k_c_setdraw, blocks_for(n, 256), 256, 0, g_set.stream, out,
                           (const float*)x, (const float*)y, n),
                "FillOutputArray");
}

}  // namespace ssg

// C-linkage entry points of include/Particle_cuda.cuh
extern "C" {
void SetDrawArray(float* ptr, float* x, float* y, int n) { ssg::compat_SetDrawArray(ptr, x, y, n); }
void ResetArrays(int* mutex, float* x, float* y, float* mass, int* count, int* start, int* sorted, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m) { ssg::compat_ResetArrays(mutex, x, y, mass, count, start, sorted, child, index, left, right, bottom, top, n, m); }
void ComputeBoundingBox(int* mutex, float* x, float* y, float* left, float* right, float* bottom, float* top, int n) { ssg::compat_ComputeBoundingBox(mutex, x, y, left, right, bottom, top, n); }
void BuildQuadTree(float* x, float* y, float* mass, int* count, int* start, int* child, int* index, float* left, float* right, float* bottom, float* top, int n, int m) { ssg::compat_BuildQuadTree(x, y, mass, count, start, child, index, left, right, bottom, top, n, m); }
void ComputeCentreOfMass(float* x, float* y, float* mass, int* index, int n) { ssg::compat_ComputeCentreOfMass(x, y, mass, index, n); }
void SortParticles(int* count, int* start, int* sorted, int* child, int* index, int n) { ssg::compat_SortParticles(count, start, sorted, child, index, n); }
void CalculateForces(float* x, float* y, float* vx, float* vy, float* ax, float* ay, float* mass, int* sorted, int* child, float* left, float* right, int n, float g) { ssg::compat_CalculateForces(x, y, vx, vy, ax, ay, mass, sorted, child, left, right, n, g); }
void IntegrateParticles(float* x, float* y, float* vx, float* vy, float* ax, float* ay, int n, float dt, float d) { ssg::compat_IntegrateParticles(x, y, vx, vy, ax, ay, n, dt, d); }
void FillOutputArray(float* x, float* y, float* out, int n) { ssg::compat_FillOutputArray(x, y, out, n); }
}  // extern "C"

// ---------------------------------------------------------------------------
// BuildQuadTreeNoAlloc: BuildQuadTree for callers that cannot allocate device
// memory.  Examples: a host that hands the GPU a fixed memory budget and owns
// every allocation itself, a real-time loop in which a cudaMalloc stall is not
// acceptable, or code whose allocator is a pool the library cannot reach.
// The existing wrapper grows a cached workspace with cudaMalloc.  This variant
// takes its scratch from one file-scope __device__ array instead, sized for at
// most kNoAllocMaxBodies bodies.  Every GPU that loads the library holds that
// array (about 8.5 MiB) until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoAllocMaxBodies = 1 << 16;

constexpr size_t na_al(size_t b) { return (b + 255) & ~size_t(255); }

// scratch bytes for n bodies, in the carve order of noalloc_layout()
constexpr size_t noalloc_bytes(size_t n) {
    return 3 * na_al(8 * n) + 3 * na_al(4 * n) + na_al(4)        // keys, values (3 each), overflow
           + na_al(4 * 256 * ((n + kSortTile - 1) / kSortTile))  // digit histograms
           + na_al(4 * 256) + na_al(16) + na_al(8)                // totals, box, system offsets
           + 8 * na_al(4 * n) + na_al(16 * n)                     // tree arrays, counter, climb
           + 2 * na_al(16 * n)                                    // node sums
           + 3 * na_al(4 * n)                                     // gathered x, y, m
           + 2 * na_al(4 * n)                                     // cells per node, cell base
           + na_al(4 * ((n + 1023) / 1024)) + na_al(4) + na_al(4);  // block sums, total, status
}

constexpr size_t kNoAllocBytes = noalloc_bytes(kNoAllocMaxBodies);

}  // namespace

// The scratch itself.  In host code this name is only a stand-in for the
// device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, resolved once per
// device (the first call on a device does this set-up).
unsigned char* noalloc_scratch(int dev, int* status) {
    if (dev < 0 || dev >= kMaxDevices) {
        *status = BH_ERR_NO_DEVICE;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            *status = cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            return nullptr;
        }
        g_noalloc_addr[dev] = static_cast<unsigned char*>(p);
    }
    return g_noalloc_addr[dev];
}

void noalloc_layout(unsigned char* base, size_t n, Workspace* w) {
    unsigned char* c = base;
    auto take = [&](size_t b) {
        void* p = c;
        c += na_al(b);
        return p;
    };
    const int tiles = (int)((n + kSortTile - 1) / kSortTile);
    const int nb = (int)((n + 1023) / 1024);
    w->keys = (uint64_t*)take(8 * n);
    w->keys_alt = (uint64_t*)take(8 * n);
    w->keys3 = (uint64_t*)take(8 * n);
    w->vals = (uint32_t*)take(4 * n);
    w->vals_alt = (uint32_t*)take(4 * n);
    w->vals3 = (uint32_t*)take(4 * n);
    w->overflow = (int*)take(4);
    w->hist = (uint32_t*)take(4 * 256 * (size_t)tiles);
    w->totals = (uint32_t*)take(4 * 256);
    w->box_ord = (int*)take(16);
    w->seg_off = (int*)take(8);
    w->tree.left = (int*)take(4 * n);
    w->tree.right = (int*)take(4 * n);
    w->tree.parent = (int*)take(4 * n);
    w->tree.leaf_parent = (int*)take(4 * n);
    w->tree.split = (int*)take(4 * n);
    w->tree.first = (int*)take(4 * n);
    w->tree.last = (int*)take(4 * n);
    w->counter = (int*)take(4 * n);
    w->tree.climb = (int4*)take(16 * n);
    w->sums.s0 = (float4*)take(16 * n);
    w->sums.s1 = (float4*)take(16 * n);
    w->sx = (float*)take(4 * n);
    w->sy = (float*)take(4 * n);
    w->sm = (float*)take(4 * n);
    w->ncell = (int*)take(4 * n);
    w->cbase = (int*)take(4 * n);
    w->bsum = (int*)take(4 * (size_t)nb);
    w->total = (int*)take(4);
    w->status = (int*)take(4);
    w->tiles = tiles;
}

// Status of one BuildQuadTreeNoAlloc call, also recorded for bh_compat_status().
int noalloc_result(int rc) {
    record(rc);
    return rc;
}

}  // namespace

extern "C" int BuildQuadTreeNoAlloc(float* x, float* y, float* mass, int* count, int* start,
                                    int* child, int* index, float* left, float* right,
                                    float* bottom, float* top, int n, int m) {
    if (n < 1 || m < n) return noalloc_result(BH_ERR_ARG);
    if (n > kNoAllocMaxBodies) {
        g_last_error = "BuildQuadTreeNoAlloc: n = " + std::to_string(n) +
                       " exceeds the static scratch limit of " +
                       std::to_string(kNoAllocMaxBodies) + " bodies";
        return noalloc_result(BH_ERR_CAPACITY);
    }
    if (n == 1) {  // a lone body: no cells, *index stays n
        set_layout(child, m);
        return BH_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_result(cuda_fail(e, "cudaGetDevice"));
    set_built(Built{});  // SortParticles walks this tree's cells: the scratch is reused
    int st_code = BH_OK;
    unsigned char* base = noalloc_scratch(dev, &st_code);
    if (!base) return noalloc_result(st_code);
    Workspace w;
    noalloc_layout(base, (size_t)n, &w);
    cudaStream_t st = g_set.stream;
    // the array keeps the previous call's contents: clear the status word here
    // (enqueue_build clears the arrival counters)
    e = cudaMemsetAsync(w.status, 0, sizeof(int), st);
    if (e != cudaSuccess) return noalloc_result(cuda_fail(e, "BuildQuadTreeNoAlloc memset"));
    e = enqueue_build(w, x, y, mass, count, start, child, index, left, right, bottom, top, n, m,
                      st);
    if (e != cudaSuccess) return noalloc_result(cuda_fail(e, "BuildQuadTreeNoAlloc launch"));
    // wait for this tree build and return its device status (the scratch is shared:
    // the next call may overwrite it as soon as this one returns)
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_result(cuda_fail(e, "BuildQuadTreeNoAlloc sync"));
    int bits = 0;
    e = cudaMemcpy(&bits, w.status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return noalloc_result(cuda_fail(e, "BuildQuadTreeNoAlloc status"));
    if (bits & ST_DUP) return noalloc_result(BH_ERR_DUPLICATE_KEYS);
    if (bits & ST_CAPACITY) return noalloc_result(BH_ERR_CAPACITY);
    if (bits & ST_NONFINITE) return noalloc_result(BH_ERR_NONFINITE);
    if (bits & ST_TREE) return noalloc_result(BH_ERR_TREE);
    set_layout(child, m);  // SortParticles and CalculateForces read up to node m - 1
    return BH_OK;
}
