// Device kernels of the GB300 (sm_103a) 2D Barnes-Hut step.
//
// Pipeline per step (one launch per phase over every system of the batch):
//   k_bbox     box of each system, origin included      kernels.cu:51-58, 62-114
//   k_keys     32-level quadrant keys by float bisection  kernels.cu:137-185
//   k_radix_*  LSD radix sort of (key, position)         replaces build+sort, kernels.cu:117-336
//   k_gather   bodies into key order                      (reference never reorders)
//   k_build    binary radix tree over the sorted keys     replaces kernels.cu:117-271
//   k_moments  bottom-up mass sums / quadrupoles           kernels.cu:180-183, 275-288
//   k_records  walk records of the branching nodes
//   k_walk_*   warp-cooperative walk fused with update    kernels.cu:340-435, 522-537
//
// Layout: bodies are SoA float arrays kept in key order between steps, so
// consecutive warps read consecutive memory.  Systems ("segments") are
// contiguous ranges [off[s], off[s+1]).  Internal tree node i (Karras
// numbering) covers a body range that starts or ends at position i; the node
// at a segment's first position is that segment's root and the node at its
// last position is unused.  A child reference >= 0 is a node, < 0 is ~body.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <climits>

namespace ssg {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kNoChild = INT_MIN;

// sticky device status bits, mapped to BH_* codes by the host
enum : int { ST_DUP = 1, ST_NONFINITE = 2, ST_STACK = 4, ST_CAPACITY = 8, ST_TREE = 16 };

// ------------------------------------------------------------------ helpers

// float <-> int with the same ordering, for lock-free atomicMin/Max
__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : (i ^ 0x7fffffff)); }

// Launch with programmatic stream serialisation: the kernel may begin while the
// previous kernel on the stream drains (it calls pdl_wait before reading).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, size_t smem,
                       cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// The same launch without the attribute (the body of a conditional graph node).
template <typename... KArgs, typename... Args>
cudaError_t launch_plain(void (*kernel)(KArgs...), int grid, int block, size_t smem,
                         cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while its predecessor drains; this waits until the
// predecessor's writes are visible.  A no-op for an ordinary launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct Segs {
    int nseg;               // number of systems
    const int* off;         // [nseg+1] body offsets
    const int* seg_of_pos;  // [n] system of each position (nullptr when nseg == 1)
};

__device__ __forceinline__ int seg_of(const Segs& s, int i) {
    return s.nseg == 1 ? 0 : __ldg(s.seg_of_pos + i);
}

struct Box {
    float l, r, b, t;
};

__device__ __forceinline__ Box load_box(const int* box_ord, int seg) {
    int4 o = *reinterpret_cast<const int4*>(box_ord + 4 * seg);
    return Box{ord2f(o.x), ord2f(o.y), ord2f(o.z), ord2f(o.w)};
}

// exclusive scan over a block of THREADS threads (one value each)
template <int THREADS>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total, uint32_t* s_tmp) {
    constexpr int W = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < W ? s_tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        if (lane < W) s_tmp[lane] = w;
    }
    __syncthreads();
    uint32_t prefix = warp > 0 ? s_tmp[warp - 1] : 0u;
    *total = s_tmp[W - 1];
    __syncthreads();
    return prefix + x - v;
}

// ------------------------------------------------------------------ (a) box

// One block per chunk of one system.  Each thread folds its bodies into a box
// that starts at the origin (the reference resets the box to 0, kernels.cu:54-57),
// then warp shuffles, shared memory, and one atomicMin/Max per value and block.
template <int THREADS>
static __global__ void __launch_bounds__(THREADS) k_bbox(const float* __restrict__ x,
                                                  const float* __restrict__ y,
                                                  const int* __restrict__ chunk_seg,
                                                  const int* __restrict__ chunk_begin,
                                                  const int* __restrict__ chunk_end,
                                                  int* __restrict__ box_ord, int* __restrict__ status) {
    pdl_wait();
    const int c = blockIdx.x;
    const int seg = chunk_seg[c], beg = chunk_begin[c], end = chunk_end[c];
    float l = 0.0f, r = 0.0f, b = 0.0f, t = 0.0f;
    bool bad = false;
    // 16-byte vector loads over the aligned middle of the chunk
    int a0 = (beg + 3) & ~3;
    if (a0 > end) a0 = end;
    int a1 = a0 + ((end - a0) & ~3);
    for (int i = beg + threadIdx.x; i < a0; i += THREADS) {
        float xv = x[i], yv = y[i];
        bad |= !isfinite(xv) || !isfinite(yv);
        l = fminf(l, xv); r = fmaxf(r, xv); b = fminf(b, yv); t = fmaxf(t, yv);
    }
    const float4* x4 = reinterpret_cast<const float4*>(x + a0);
    const float4* y4 = reinterpret_cast<const float4*>(y + a0);
    for (int i = threadIdx.x; i < (a1 - a0) / 4; i += THREADS) {
        float4 xv = __ldcs(x4 + i), yv = __ldcs(y4 + i);
        bad |= !isfinite(xv.x) || !isfinite(xv.y) || !isfinite(xv.z) || !isfinite(xv.w);
        bad |= !isfinite(yv.x) || !isfinite(yv.y) || !isfinite(yv.z) || !isfinite(yv.w);
        l = fminf(fminf(l, fminf(xv.x, xv.y)), fminf(xv.z, xv.w));
        r = fmaxf(fmaxf(r, fmaxf(xv.x, xv.y)), fmaxf(xv.z, xv.w));
        b = fminf(fminf(b, fminf(yv.x, yv.y)), fminf(yv.z, yv.w));
        t = fmaxf(fmaxf(t, fmaxf(yv.x, yv.y)), fmaxf(yv.z, yv.w));
    }
    for (int i = a1 + threadIdx.x; i < end; i += THREADS) {
        float xv = x[i], yv = y[i];
        bad |= !isfinite(xv) || !isfinite(yv);
        l = fminf(l, xv); r = fmaxf(r, xv); b = fminf(b, yv); t = fmaxf(t, yv);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        l = fminf(l, __shfl_xor_sync(kFull, l, o));
        r = fmaxf(r, __shfl_xor_sync(kFull, r, o));
        b = fminf(b, __shfl_xor_sync(kFull, b, o));
        t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
    }
    __shared__ float s[4][THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][warp] = l; s[1][warp] = r; s[2][warp] = b; s[3][warp] = t;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, ST_NONFINITE);
    if (warp == 0) {
        l = lane < THREADS / 32 ? s[0][lane] : 0.0f;
        r = lane < THREADS / 32 ? s[1][lane] : 0.0f;
        b = lane < THREADS / 32 ? s[2][lane] : 0.0f;
        t = lane < THREADS / 32 ? s[3][lane] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            l = fminf(l, __shfl_xor_sync(kFull, l, o));
            r = fmaxf(r, __shfl_xor_sync(kFull, r, o));
            b = fminf(b, __shfl_xor_sync(kFull, b, o));
            t = fmaxf(t, __shfl_xor_sync(kFull, t, o));
        }
        if (lane == 0) {
            int* bo = box_ord + 4 * seg;
            atomicMin(bo + 0, f2ord(l));
            atomicMax(bo + 1, f2ord(r));
            atomicMin(bo + 2, f2ord(b));
            atomicMax(bo + 3, f2ord(t));
        }
    }
}

// ------------------------------------------------------------------ bodies

struct BodyPtrs {
    float *x, *y, *vx, *vy, *m, *xlo, *ylo;  // xlo/ylo may be null
    int* id;
    float* amag;  // |a| of the previous step (accuracy modes; may be null)
    int* gcost;   // interaction entries of the body's walk group in the previous step
                  // (accuracy modes; may be null)
};

// Body i of src becomes body j of dst (the reorder into key order).
__device__ __forceinline__ void gather_body(int j, uint32_t i, const BodyPtrs& src,
                                            const BodyPtrs& dst) {
    dst.x[j] = src.x[i];
    dst.y[j] = src.y[i];
    dst.vx[j] = src.vx[i];
    dst.vy[j] = src.vy[i];
    dst.m[j] = src.m[i];
    dst.id[j] = src.id[i];
    if (src.xlo) {
        dst.xlo[j] = src.xlo[i];
        dst.ylo[j] = src.ylo[i];
    }
    if (src.amag) dst.amag[j] = src.amag[i];
    if (src.gcost) dst.gcost[j] = src.gcost[i];
}

// ------------------------------------------------------------------ (b1) keys

// Level by level: mid = (lo+hi)*0.5 in float, digit bit 0 = x < mid_x,
// bit 1 = y < mid_y, the body's half becomes the interval (kernels.cu:144-157,
// 165-177).  Explicit _rn intrinsics: no contraction may change a midpoint.
// The x and y intervals are bisected together in packed FP32x2 arithmetic
// (per component the same IEEE operations); the x and y bits are collected
// separately and interleaved at the end.
__device__ __forceinline__ uint64_t spread_even_bits(uint32_t v) {
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

__device__ __forceinline__ uint64_t quad_key(float px, float py, Box bx) {
    float2 lo = make_float2(bx.l, bx.b), hi = make_float2(bx.r, bx.t);
    const float2 half = make_float2(0.5f, 0.5f);
    uint32_t kx = 0, ky = 0;
#pragma unroll 8
    for (int level = 0; level < 32; ++level) {
        const float2 mid = __fmul2_rn(__fadd2_rn(lo, hi), half);
        const bool xl = px < mid.x, yl = py < mid.y;
        hi.x = xl ? mid.x : hi.x;
        lo.x = xl ? lo.x : mid.x;
        hi.y = yl ? mid.y : hi.y;
        lo.y = yl ? lo.y : mid.y;
        kx = (kx << 1) | (xl ? 1u : 0u);
        ky = (ky << 1) | (yl ? 1u : 0u);
    }
    return spread_even_bits(kx) | (spread_even_bits(ky) << 1);
}

static __global__ void k_keys(const float* __restrict__ x, const float* __restrict__ y, int n, Segs segs,
                       const int* __restrict__ box_ord, uint64_t* __restrict__ keys,
                       uint32_t* __restrict__ vals) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Box bx = load_box(box_ord, seg_of(segs, i));
    keys[i] = quad_key(x[i], y[i], bx);
    vals[i] = (uint32_t)i;
}

// k_keys for the engine's step: also clears the moments arrival counters of
// these positions, the per-step flags (flags[0..nflags)), the first `nstates`
// words of the walk's shared-group counters and slice states (nstates <= the
// grid's threads) and (block 0) the step's first `nzero` scheduling and
// statistics words.  With nzero > 0 (a
// step, not the energy pass) each system's walk cost of the last step
// (seg_cost, entries x bodies) becomes its mean walk-group cost (mean_cost)
// and is cleared.  box_copy (non-null when the box was carried from the last
// walk): block 0 copies the box read (box_ord) there, for the later phases.
static __global__ void k_keys_step(const float* __restrict__ x, const float* __restrict__ y, int n,
                                   Segs segs, const int* __restrict__ box_ord,
                                   uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                   int* __restrict__ counter, int* __restrict__ zero, int nzero,
                                   int* __restrict__ flags, int nflags,
                                   int* __restrict__ states, int nstates,
                                   unsigned long long* __restrict__ seg_cost,
                                   int* __restrict__ mean_cost, int* __restrict__ box_copy) {
    pdl_wait();
    {
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t < nstates) states[t] = 0;
    }
    if (blockIdx.x == 0) {
        if (threadIdx.x < nzero) zero[threadIdx.x] = 0;
        if (threadIdx.x < nflags) flags[threadIdx.x] = 0;
        if (box_copy)
            for (int w = threadIdx.x; w < 4 * segs.nseg; w += blockDim.x) box_copy[w] = box_ord[w];
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (nzero > 0 && t < segs.nseg) {
        const unsigned long long size = (unsigned long long)(segs.off[t + 1] - segs.off[t]);
        mean_cost[t] = (int)min(seg_cost[t] / size, (unsigned long long)INT_MAX);
        seg_cost[t] = 0ull;
    }
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Box bx = load_box(box_ord, seg_of(segs, i));
    keys[i] = quad_key(x[i], y[i], bx);
    vals[i] = (uint32_t)i;
    counter[i] = 0;
}

// ------------------------------------------------------------------ (b2) radix sort

// Digit of one element: 8 bits of the key, or of the element's system index
// (the final passes group the systems; stable LSD keeps key order inside).
__device__ __forceinline__ uint32_t radix_digit(uint64_t k, uint32_t v, int shift, int use_seg,
                                                const int* __restrict__ seg_of_pos) {
    return use_seg ? ((uint32_t)__ldg(seg_of_pos + v) >> shift) & 255u
                   : (uint32_t)(k >> shift) & 255u;
}

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
static_assert(kSortThreads == 256, "one thread per digit in the sort kernels");

// per-tile digit counts, written digit-major: hist[d * tiles + tile].  Each
// warp counts into its own shared sub-histogram with plain shared atomics
// (twice as fast as aggregating equal digits with warp votes first).
// The three pass kernels take `only_if`: when non-null they do nothing unless
// *only_if is set (the fallback full sort of k_sort_fixup's overflow).
// The three kernels of a pass are bodies over one tile (or one digit), so that
// the full sort's cooperative kernel (k_full_sort_grid) runs the same code.
// Each body starts with a block barrier: a block that loops over several tiles
// must not reset its shared arrays while a slower thread still reads them.
__device__ __forceinline__ void radix_hist_tile(int tile, const uint64_t* __restrict__ keys,
                                                const uint32_t* __restrict__ vals, int n, int shift,
                                                int use_seg, const int* __restrict__ seg_of_pos,
                                                uint32_t* __restrict__ hist, int tiles) {
    constexpr int W = kSortThreads / 32;
    __shared__ uint32_t s_h[W][256];
    __syncthreads();
    for (int i = threadIdx.x; i < W * 256; i += kSortThreads) (&s_h[0][0])[i] = 0u;
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const int base = tile * kSortTile;
    uint32_t dg[kSortItems];
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        int idx = base + it * kSortThreads + threadIdx.x;
        dg[it] = idx < n ? radix_digit(keys[idx], use_seg ? vals[idx] : 0u, shift, use_seg,
                                       seg_of_pos)
                         : 256u;
    }
#pragma unroll
    for (int it = 0; it < kSortItems; ++it)
        if (dg[it] < 256u) atomicAdd(&s_h[warp][dg[it]], 1u);
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < W; ++w) t += s_h[w][threadIdx.x];
    hist[threadIdx.x * tiles + tile] = t;
}

static __global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint64_t* __restrict__ keys,
                                                             const uint32_t* __restrict__ vals, int n,
                                                             int shift, int use_seg,
                                                             const int* __restrict__ seg_of_pos,
                                                             uint32_t* __restrict__ hist, int tiles,
                                                             const int* __restrict__ only_if) {
    pdl_wait();
    if (only_if && *only_if == 0) return;
    radix_hist_tile(blockIdx.x, keys, vals, n, shift, use_seg, seg_of_pos, hist, tiles);
}

// digit d: column d of hist into exclusive offsets; totals[d] = column sum
__device__ __forceinline__ void radix_scan_digit(int d, uint32_t* __restrict__ hist, int tiles,
                                                 uint32_t* __restrict__ totals) {
    __shared__ uint32_t s_tmp[kSortThreads / 32];
    __syncthreads();
    uint32_t* col = hist + (size_t)d * tiles;
    uint32_t running = 0;
    for (int base = 0; base < tiles; base += kSortThreads) {
        int i = base + threadIdx.x;
        uint32_t v = i < tiles ? col[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_excl_scan<kSortThreads>(v, &tot, s_tmp);
        if (i < tiles) col[i] = running + ex;
        running += tot;
    }
    if (threadIdx.x == 0) totals[d] = running;
}

static __global__ void __launch_bounds__(kSortThreads) k_radix_scan(uint32_t* __restrict__ hist, int tiles,
                                                             uint32_t* __restrict__ totals,
                                                             const int* __restrict__ only_if) {
    pdl_wait();
    if (only_if && *only_if == 0) return;
    radix_scan_digit(blockIdx.x, hist, tiles, totals);
}

// Lanes of the warp holding the same 8-bit digit as this lane (valid lanes
// only; an invalid lane gets a mask it does not use): one vote per digit bit.
__device__ __forceinline__ unsigned digit_peers(uint32_t d, bool valid) {
    unsigned peers = __ballot_sync(kFull, valid);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (d >> b) & 1u;
        const unsigned v = __ballot_sync(kFull, bit);
        peers &= bit ? v : ~v;
    }
    return peers;
}

// Stable scatter of one tile: warp w owns 256 consecutive elements, ranks are
// (earlier rounds of the warp) + (lower lanes with the same digit); warps are
// then offset by the counts of lower warps.  Elements are staged in shared
// memory in digit order and written out as contiguous runs.
__device__ __forceinline__ void radix_scatter_tile(
    int tile, const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
    uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, int n, int shift, int use_seg,
    const int* __restrict__ seg_of_pos, const uint32_t* __restrict__ hist,
    const uint32_t* __restrict__ totals, int tiles) {
    constexpr int W = kSortThreads / 32;
    constexpr int WCHUNK = 32 * kSortItems;
    __shared__ uint32_t s_wh[W][256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_lstart[256];
    __shared__ uint32_t s_tmp[W];
    __shared__ uint64_t s_k[kSortTile];
    __shared__ uint32_t s_v[kSortTile];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    __syncthreads();
    for (int i = tid; i < W * 256; i += kSortThreads) (&s_wh[0][0])[i] = 0u;
    {
        uint32_t tot;
        uint32_t ex = block_excl_scan<kSortThreads>(totals[tid], &tot, s_tmp);
        s_gbase[tid] = ex + hist[(size_t)tid * tiles + tile];
    }
    __syncthreads();
    const int base = tile * kSortTile;
    uint64_t k[kSortItems];
    uint32_t v[kSortItems];
    uint32_t rank[kSortItems];
    int dg[kSortItems];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {  // the tile's loads, then the ranking
        int idx = base + warp * WCHUNK + r * 32 + lane;
        bool valid = idx < n;
        k[r] = valid ? kin[idx] : 0ull;
        v[r] = valid ? vin[idx] : 0u;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        int idx = base + warp * WCHUNK + r * 32 + lane;
        bool valid = idx < n;
        uint32_t d = valid ? radix_digit(k[r], v[r], shift, use_seg, seg_of_pos) : 0u;
        dg[r] = valid ? (int)d : -1;
        unsigned peers = digit_peers(d, valid);
        rank[r] = valid ? s_wh[warp][d] + (uint32_t)__popc(peers & lt) : 0u;
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == lane) s_wh[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) {
            uint32_t c = s_wh[w][tid];
            s_wh[w][tid] = run;
            run += c;
        }
        uint32_t tot;
        s_lstart[tid] = block_excl_scan<kSortThreads>(run, &tot, s_tmp);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        if (dg[r] >= 0) {
            uint32_t pos = s_lstart[dg[r]] + s_wh[warp][dg[r]] + rank[r];
            s_k[pos] = k[r];
            s_v[pos] = v[r];
        }
    }
    __syncthreads();
    const int tile_n = min(kSortTile, n - base);
    for (int i = tid; i < tile_n; i += kSortThreads) {
        uint64_t kk = s_k[i];
        uint32_t vv = s_v[i];
        uint32_t d = radix_digit(kk, vv, shift, use_seg, seg_of_pos);
        uint32_t o = s_gbase[d] + ((uint32_t)i - s_lstart[d]);
        kout[o] = kk;
        vout[o] = vv;
    }
}

static __global__ void __launch_bounds__(kSortThreads) k_radix_scatter(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, int n, int shift, int use_seg, const int* __restrict__ seg_of_pos,
    const uint32_t* __restrict__ hist, const uint32_t* __restrict__ totals, int tiles,
    const int* __restrict__ only_if) {
    pdl_wait();
    if (only_if && *only_if == 0) return;
    radix_scatter_tile(blockIdx.x, kin, vin, kout, vout, n, shift, use_seg, seg_of_pos, hist, totals,
                       tiles);
}

// The sort's fast path: P stable 8-bit passes over the key's top 8P bits (the
// high word, bits `shift` = 64 - 8P .. 63), then k_sort_fixup.  Elements with
// equal high words then form runs in input order; each run is put in
// whole-key order with ties kept in input order, which gives the stable sort
// by the whole key.  Element i's place in its run is the number of run members
// before it in that order, so the fixup's work grows with the run lengths: P
// is 3 (runs of one 2^-12 box cell) for systems up to kShortSortMax bodies and
// 4 (2^-16 cells) above, where the bodies per cell grow.  A run longer than
// kFixupRun is not ordered: *overflow is set, and (set_cond, graph replay) the
// conditional node that holds the full sort is switched on; exactly one
// thread does either.
constexpr int kShortSortMax = 1 << 21;
constexpr int kFixupRun = 256;

//
// Block 0 also resets box_reset (box_words ints, when non-null) to the origin
// box: the key kernel, which may have read it, has completed.
static __global__ void k_sort_fixup(int n, int shift, const uint64_t* __restrict__ kin,
                                    const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                    uint32_t* __restrict__ vout, int* __restrict__ overflow,
                                    cudaGraphConditionalHandle cond, int set_cond,
                                    int* __restrict__ box_reset, int box_words) {
    pdl_wait();
    if (box_reset && blockIdx.x == 0)
        for (int w = threadIdx.x; w < box_words; w += blockDim.x) box_reset[w] = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t k = kin[i];
    const uint32_t hi = (uint32_t)(k >> shift);
    const bool left = i > 0 && (uint32_t)(kin[i - 1] >> shift) == hi;
    const bool right = i + 1 < n && (uint32_t)(kin[i + 1] >> shift) == hi;
    if (!left && !right) {
        kout[i] = k;
        vout[i] = vin[i];
        return;
    }
    // the run's start, then one pass from it to the run's end that also ranks
    int a = i;
    while (a > 0 && (uint32_t)(kin[a - 1] >> shift) == hi && i - a < kFixupRun) --a;
    int rank = 0, j = a;
    for (; j < n && j - a <= kFixupRun; ++j) {
        const uint64_t kj = kin[j];
        if ((uint32_t)(kj >> shift) != hi) break;
        rank += (kj < k || (kj == k && j < i)) ? 1 : 0;
    }
    if (j - a > kFixupRun) {
        if (atomicCAS(overflow, 0, 1) == 0 && set_cond) cudaGraphSetConditional(cond, 1u);
        return;
    }
    kout[a + rank] = k;
    vout[a + rank] = vin[i];
}

// The full sort (the fast path's fallback, when *only_if is set) as one
// cooperative kernel: the eight 8-bit passes k0 -> kB -> kA -> ... -> kA of the
// 24 pass kernels, every block looping over tiles and digits, a grid barrier
// between the phases.  Every block returns at once when the flag is clear: one
// launch where the stream-ordered fallback took 24 (about 1 us each on GB300
// when they return at once).
static __global__ void __launch_bounds__(kSortThreads) k_full_sort_grid(
    const uint64_t* __restrict__ k0, const uint32_t* __restrict__ v0, uint64_t* __restrict__ kA,
    uint32_t* __restrict__ vA, uint64_t* __restrict__ kB, uint32_t* __restrict__ vB, int n,
    uint32_t* __restrict__ hist, uint32_t* __restrict__ totals, int tiles,
    const int* __restrict__ only_if) {
    pdl_wait();
    if (*only_if == 0) return;
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    const uint64_t* ki = k0;
    const uint32_t* vi = v0;
    for (int ps = 0; ps < 8; ++ps) {
        uint64_t* ko = (ps & 1) ? kA : kB;
        uint32_t* vo = (ps & 1) ? vA : vB;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x)
            radix_hist_tile(t, ki, vi, n, 8 * ps, 0, nullptr, hist, tiles);
        grid.sync();
        for (int d = blockIdx.x; d < 256; d += gridDim.x) radix_scan_digit(d, hist, tiles, totals);
        grid.sync();
        for (int t = blockIdx.x; t < tiles; t += gridDim.x)
            radix_scatter_tile(t, ki, vi, ko, vo, n, 8 * ps, 0, nullptr, hist, totals, tiles);
        grid.sync();
        ki = ko;
        vi = vo;
    }
}

// Launch k_full_sort_grid over the resident grid of the current device; false
// when no cooperative grid can be formed (the caller launches the 24 kernels).
static bool launch_full_sort_grid(const uint64_t* k0, const uint32_t* v0, uint64_t* kA,
                                  uint32_t* vA, uint64_t* kB, uint32_t* vB, int n, uint32_t* hist,
                                  uint32_t* totals, int tiles, const int* only_if,
                                  cudaStream_t st, cudaError_t* err) {
    constexpr int kDevs = 64;
    static std::atomic<int> s_grid[kDevs] = {};  // resident blocks per device, read once
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs) return false;
    int grid = s_grid[dev].load();
    if (grid == 0) {
        int bps = 0, sms = 0, coop = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_full_sort_grid, kSortThreads, 0) !=
                cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess)
            bps = 0;
        grid = (coop && bps > 0 && sms > 0) ? bps * sms : -1;
        s_grid[dev] = grid;
    }
    if (grid < 1) return false;
    void* args[] = {(void*)&k0, (void*)&v0, (void*)&kA, (void*)&vA, (void*)&kB, (void*)&vB,
                    (void*)&n, (void*)&hist, (void*)&totals, (void*)&tiles, (void*)&only_if};
    *err = cudaLaunchCooperativeKernel((const void*)k_full_sort_grid, grid, kSortThreads, args, 0,
                                       st);
    return true;
}

// ------------------------------------------------------------------ (d) reorder

static __global__ void k_gather(int n, const uint32_t* __restrict__ perm, BodyPtrs src, BodyPtrs dst) {
    pdl_wait();
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    gather_body(j, perm[j], src, dst);
}

// ------------------------------------------------------------------ (b3) tree

// Leading equal bits of sorted keys i and j inside [lo, hi]; equal keys are
// told apart by position (bits 64..95) so the tree stays binary.
__device__ __forceinline__ int kdelta(const uint64_t* __restrict__ k, int i, int j, int lo, int hi) {
    if (j < lo || j > hi) return -1;
    uint64_t a = k[i], b = k[j];
    return a != b ? __clzll(a ^ b) : 64 + __clz(i ^ j);
}

// kdelta with key i already in a register (ki = k[i]).
__device__ __forceinline__ int kdelta_i(const uint64_t* __restrict__ k, uint64_t ki, int i, int j,
                                        int lo, int hi) {
    if (j < lo || j > hi) return -1;
    const uint64_t b = k[j];
    return ki != b ? __clzll(ki ^ b) : 64 + __clz(i ^ j);
}

struct TreePtrs {
    int *left, *right, *parent, *leaf_parent, *split, *first, *last;
    int4* climb;  // per internal node: left, right, parent, w = (split << 1) | inside one
                  // moments block
};

// k_moments runs one thread per leaf in blocks of kMomentsThreads; a node whose
// body range lies inside one block's leaves is combined with block-scope
// synchronisation (climb record .w = 1).
constexpr int kMomentsLog2 = 8;
constexpr int kMomentsThreads = 1 << kMomentsLog2;

// Karras (2012) radix-tree construction, one thread per internal node.
static __global__ void k_build(const uint64_t* __restrict__ k, int n, Segs segs, TreePtrs t,
                        int* __restrict__ status) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s = seg_of(segs, i);
    int lo = segs.off[s], hi = segs.off[s + 1] - 1;
    if (i < hi && k[i] == k[i + 1]) atomicOr(status, ST_DUP);
    if (i == hi) {  // last position of a system: not an internal node
        t.left[i] = kNoChild;
        t.right[i] = kNoChild;
        t.split[i] = -1;
        t.first[i] = i;
        t.last[i] = i;
        if (lo == hi) {
            t.leaf_parent[i] = -1;
            t.parent[i] = -1;
        }
        return;
    }
    if (i == lo) {
        t.parent[i] = -1;
        t.climb[i].z = -1;
    }
    const uint64_t ki = k[i];
    int dl = kdelta_i(k, ki, i, i - 1, lo, hi), dr = kdelta_i(k, ki, i, i + 1, lo, hi);
    int d = dr > dl ? 1 : -1;
    int dmin = min(dl, dr);
    int lmax = 2;
    while (kdelta_i(k, ki, i, i + lmax * d, lo, hi) > dmin) lmax <<= 1;
    int l = 0;
    for (int step = lmax >> 1; step >= 1; step >>= 1)
        if (kdelta_i(k, ki, i, i + (l + step) * d, lo, hi) > dmin) l += step;
    int j = i + l * d;
    int dnode = kdelta_i(k, ki, i, j, lo, hi);
    int sp = 0;
    for (int sh = 1;; ++sh) {
        const int step = ((l - 1) >> sh) + 1;  // ceil(l / 2^sh) for l >= 1, no division
        if (kdelta_i(k, ki, i, i + (sp + step) * d, lo, hi) > dnode) sp += step;
        if (step <= 1) break;
    }
    int g = i + sp * d + min(d, 0);
    int a = min(i, j), b = max(i, j);
    int lc, rc;
    if (a == g) {
        lc = ~g;
        t.leaf_parent[g] = i;
    } else {
        lc = g;
        t.parent[g] = i;
        t.climb[g].z = i;
    }
    if (b == g + 1) {
        rc = ~(g + 1);
        t.leaf_parent[g + 1] = i;
    } else {
        rc = g + 1;
        t.parent[g + 1] = i;
        t.climb[g + 1].z = i;
    }
    t.left[i] = lc;
    t.right[i] = rc;
    t.split[i] = dnode;
    t.first[i] = a;
    t.last[i] = b;
    // .z (parent) is written by the parent's thread
    *reinterpret_cast<int2*>(&t.climb[i].x) = make_int2(lc, rc);
    t.climb[i].w = (dnode << 1) | ((a >> kMomentsLog2) == (b >> kMomentsLog2) ? 1 : 0);
}

// ------------------------------------------------------------------ (c) moments

// Node sums, two 16-byte records per node so that a child is read with two
// loads (REFERENCE: one) and a node written with two stores.
struct NodeSums {
    float4* s0;  // M, sum m*x, sum m*y, centre-of-mass x
    float4* s1;  // centre-of-mass y, Sxx, Sxy, Syy (second moments about it; accuracy modes)
};

struct ChildVals {
    float m, mx, my, cx, cy, sxx, sxy, syy;
};

__device__ __forceinline__ ChildVals body_vals(int bi, const float* __restrict__ sx,
                                               const float* __restrict__ sy,
                                               const float* __restrict__ sm) {
    ChildVals v;
    v.m = sm[bi];
    v.cx = sx[bi];
    v.cy = sy[bi];
    v.mx = __fmul_rn(v.m, v.cx);  // kernels.cu:180: mass*x
    v.my = __fmul_rn(v.m, v.cy);
    v.sxx = v.sxy = v.syy = 0.0f;
    return v;
}

__device__ __forceinline__ ChildVals load_child(int c, const float* __restrict__ sx,
                                                const float* __restrict__ sy,
                                                const float* __restrict__ sm, const NodeSums& ns,
                                                bool quad) {
    if (c < 0) return body_vals(~c, sx, sy, sm);
    // written by another thread of this launch: read through L2
    ChildVals v;
    const float4 a = __ldcg(ns.s0 + c);
    v.m = a.x;
    v.mx = a.y;
    v.my = a.z;
    v.cx = a.w;
    if (quad) {
        const float4 b = __ldcg(ns.s1 + c);
        v.cy = b.x;
        v.sxx = b.y;
        v.sxy = b.z;
        v.syy = b.w;
    } else {
        v.cy = 0.0f;  // not an input of the REFERENCE combination
        v.sxx = v.sxy = v.syy = 0.0f;
    }
    return v;
}

// Node p from its left child a and right child b; returns p's values.
__device__ __forceinline__ ChildVals combine_node(int p, const ChildVals& a, const ChildVals& b,
                                                  int accuracy, const NodeSums& ns) {
    ChildVals r;
    r.m = __fadd_rn(a.m, b.m);
    r.mx = __fadd_rn(a.mx, b.mx);
    r.my = __fadd_rn(a.my, b.my);
    if (!accuracy) {
        r.cx = __fdiv_rn(r.mx, r.m);
        r.cy = __fdiv_rn(r.my, r.m);
        r.sxx = r.sxy = r.syy = 0.0f;
    } else {
        float w = r.m > 0.0f ? b.m / r.m : 0.5f;
        r.cx = fmaf(w, b.cx - a.cx, a.cx);
        r.cy = fmaf(w, b.cy - a.cy, a.cy);
        float ax = a.cx - r.cx, ay = a.cy - r.cy, bx = b.cx - r.cx, by = b.cy - r.cy;
        r.sxx = a.sxx + b.sxx + a.m * ax * ax + b.m * bx * bx;
        r.sxy = a.sxy + b.sxy + a.m * ax * ay + b.m * bx * by;
        r.syy = a.syy + b.syy + a.m * ay * ay + b.m * by * by;
    }
    ns.s0[p] = make_float4(r.m, r.mx, r.my, r.cx);
    ns.s1[p] = make_float4(r.cy, r.sxx, r.sxy, r.syy);
    return r;
}

// Bottom-up: each body climbs from its leaf; the second thread to reach a node
// combines both children (left + right, so the sums do not depend on which
// thread arrives last) and continues.  REFERENCE mode keeps the reference's
// definition com = (sum m*x) / (sum m) (kernels.cu:283-284); accuracy modes
// combine centres relative to each other and add second moments.  The child a
// thread climbs from stays in its registers; only the sibling is loaded.
//
// A block owns kMomentsThreads consecutive leaves.  A node whose body range
// lies inside them is reached only by threads of that block: its arrival
// counter lives in shared memory, taken with one block-scope acquire-release
// atomic that orders the child data.
// Only nodes that span two blocks' leaves use a global counter, taken with one
// acquire-release atomic: its release publishes the node this thread wrote,
// its acquire makes the sibling's sums visible to the loads that follow.  The
// parent's climb record is loaded while the counter is taken.
// Block-scope acquire-release add on a shared-memory counter: the one atomic
// orders this thread's earlier global writes before the later reads of the
// thread that arrives second, within one block.
__device__ __forceinline__ int atomic_add_acq_rel_cta_shared(int* p, int v) {
    int old;
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("atom.acq_rel.cta.shared::cta.add.s32 %0, [%1], %2;"
                 : "=r"(old)
                 : "r"(a), "r"(v)
                 : "memory");
    return old;
}

__device__ __forceinline__ int atomic_add_acq_rel_gpu(int* p, int v) {
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;"
                 : "=r"(old)
                 : "l"(p), "r"(v)
                 : "memory");
    return old;
}

constexpr int kMaxClimb = 256;

static __global__ void __launch_bounds__(kMomentsThreads) k_moments(int n, int accuracy, const float* __restrict__ sx,
                                                     const float* __restrict__ sy,
                                                     const float* __restrict__ sm,
                                                     const int4* __restrict__ climb,
                                                     const int* __restrict__ leaf_parent,
                                                     int* __restrict__ counter, NodeSums ns,
                                                     int* __restrict__ status) {
    pdl_wait();
    __shared__ int s_cnt[kMomentsThreads];
    const int c0 = blockIdx.x * kMomentsThreads;  // this block's leaves: [c0, c0 + kMomentsThreads)
    const int j = c0 + threadIdx.x;
    s_cnt[threadIdx.x] = 0;
    __syncthreads();
    if (j >= n) return;
    int p = leaf_parent[j];
    if (p < 0) return;
    int4 T = climb[p];  // left, right, parent, range inside one moments block
    int from = ~j;      // the child this thread climbs from
    ChildVals own = body_vals(j, sx, sy, sm);
    // a radix tree of 64-bit keys (ties broken by position) is at most 96 levels deep
    for (int level = 0;; ++level) {
        if (level == kMaxClimb) {
            atomicOr(status, ST_TREE);
            return;
        }
        int4 TN = make_int4(0, 0, -1, 0);
        if (T.z >= 0) TN = climb[T.z];
        if (T.w & 1) {
            if (atomic_add_acq_rel_cta_shared(s_cnt + (p - c0), 1) == 0) return;
        } else {
            if (atomic_add_acq_rel_gpu(counter + p, 1) == 0) return;
        }
        const bool from_left = T.x == from;
        const ChildVals sib = load_child(from_left ? T.y : T.x, sx, sy, sm, ns, accuracy);
        own = from_left ? combine_node(p, own, sib, accuracy, ns)
                        : combine_node(p, sib, own, accuracy, ns);
        if (T.z < 0) return;
        from = p;
        p = T.z;
        T = TN;
    }
}

// ------------------------------------------------------------------ walk records

// Branching quadtree nodes: a binary node splitting the low bit of a digit is
// folded into its parent when the parent splits the high bit of the same digit.
__device__ __forceinline__ bool merged_into(int c_split, int p_split) {
    return (c_split & 1) && p_split == c_split - 1;
}

// Records A and D of a node sit side by side in one 32-byte sector (a node
// test reads both): A of node i at A[kRecStride i], D at D[kRecStride i], with
// D = (int4*)A + 1.  One sector per tested node instead of two: the frontier
// kernel, whose traversal chains wait on these loads, 42 -> 36 us at 2^20.
constexpr int kRecStride = 2;
struct Records {
    float4* A;  // cx, cy, M, criterion (REFERENCE: dp of the node's level; accuracy: ropen^2)
    float4* B;  // accuracy: 3Sxx, 3Sxy, 3Syy, 1.5 (Sxx+Syy)
    int4* C;    // up to four children, kNoChild padded
    int4* D;    // first body, body count, bits of G*M*l^3 (accuracy), 0
};

// Every other bit of x (bits 0, 2, 4, ...) packed into the low 32 bits.
__device__ __forceinline__ uint64_t compact_even_bits(uint64_t x) {
    x &= 0x5555555555555555ull;
    x = (x | (x >> 1)) & 0x3333333333333333ull;
    x = (x | (x >> 2)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x >> 4)) & 0x00ff00ff00ff00ffull;
    x = (x | (x >> 8)) & 0x0000ffff0000ffffull;
    x = (x | (x >> 16)) & 0x00000000ffffffffull;
    return x;
}

// dp_L = w_L^2/theta with w_L the level-L cell width from the x extent only:
// radius = (right-left)*0.5 (kernels.cu:349), root children pushed with
// radius^2/theta (:376), times 0.25 per level (:395).  Cells at level <= 1 are
// never approximated (+inf).
__device__ __forceinline__ float ref_dp(Box bx, float theta, int level) {
    if (level < 2) return __int_as_float(0x7f800000);
    float radius = __fmul_rn(__fsub_rn(bx.r, bx.l), 0.5f);
    float dp1 = __fdiv_rn(__fmul_rn(radius, radius), theta);
    return ldexpf(dp1, -2 * (level - 1));
}


// Opening angle of the bootstrap pass (|a| estimate after bh_set_state, cells
// as monopoles).  At 1.25 its |a| is within about 15 % (RMS) and it costs about
// a third of the theta = 0.5 walk; the relative rule it feeds opens the same
// nodes as with exact |a| to within 1 %.  Plummer, colliding disks and disk
// at 2^20 on the oracle: 17-22 % fewer bootstrap interactions than at 1.0,
// main-pass interactions within 0.6 % and the same force error.  Near 1.5 the
// estimate breaks down (cells as large as the system accepted).
constexpr float kBootstrapTheta = 1.25f;

// Walk record of branching node i, from its sums and the tree (the body of
// k_records).
__device__ __forceinline__ void emit_record(int i, int sp, int4 T, int accuracy, float theta,
                                            float G, const int* __restrict__ box_ord, int seg,
                                            const uint64_t* __restrict__ skeys,
                                            const TreePtrs& t, float M, float cx, float cy,
                                            float4 quad, Records rec) {
    int ch[4] = {kNoChild, kNoChild, kNoChild, kNoChild};
    int nc = 0;
    const int lr[2] = {T.x, T.y};
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
        const int c = lr[s2];
        int4 Tc = make_int4(0, 0, 0, 0);
        if (c >= 0) Tc = t.climb[c];
        if (c >= 0 && merged_into(Tc.w >> 1, sp)) {
            ch[nc++] = Tc.x;
            ch[nc++] = Tc.y;
        } else {
            ch[nc++] = c;
        }
    }
    rec.C[i] = make_int4(ch[0], ch[1], ch[2], ch[3]);
    const int f = t.first[i], cnt = t.last[i] - f + 1;
    const int level = sp >> 1;
    const Box bx = load_box(box_ord, seg);
    if (!accuracy) {
        rec.A[kRecStride * i] = make_float4(cx, cy, M, ref_dp(bx, theta, level));
        rec.D[kRecStride * i] = make_int4(f, cnt, 0, 0);
        return;
    }
    const int L = level < 32 ? level : 32;
    const uint64_t pre = L > 0 ? skeys[f] >> (64 - 2 * L) : 0ull;
    const uint64_t mask = L > 0 ? (~0ull >> (64 - L)) : 0ull;
    const uint64_t ix = ~compact_even_bits(pre) & mask;
    const uint64_t iy = ~compact_even_bits(pre >> 1) & mask;
    const float scale = ldexpf(1.0f, -L);
    const float wx = bx.r - bx.l, wy = bx.t - bx.b;
    const float l = fmaxf(wx, wy) * scale;
    // cell centre in FP32: exact in ix, iy up to level 23, then within an ulp of
    // the box width, as precise as the centre of mass it is compared with
    const float ccx = fmaf(wx, ((float)ix + 0.5f) * scale, bx.l);
    const float ccy = fmaf(wy, ((float)iy + 0.5f) * scale, bx.b);
    const float ddx = cx - ccx, ddy = cy - ccy;
    const float delta = sqrtf(fmaf(ddx, ddx, ddy * ddy));
    const float r = l / theta + delta;
    rec.A[kRecStride * i] = make_float4(cx, cy, M, r * r);
    const float qerr = G * M * l * l * l;
    // the bootstrap pass only needs |a| to a few per cent: a wider opening angle
    const float rb = l / fmaxf(theta, kBootstrapTheta) + delta;
    rec.D[kRecStride * i] = make_int4(f, cnt, __float_as_int(qerr), __float_as_int(rb * rb));
    rec.B[i] = make_float4(3.0f * quad.x, 3.0f * quad.y, 3.0f * quad.z, 1.5f * (quad.x + quad.z));
}

// One thread per node: the walk record of every branching node (binary nodes
// folded into their parent emit nothing).  Topology comes from the climb
// records: one 16-byte load per node, its parent and its children.
static __global__ void k_records(int n, Segs segs, int accuracy, float theta, float G,
                                 const int* __restrict__ box_ord, const uint64_t* __restrict__ skeys,
                                 TreePtrs t, NodeSums ns, Records rec) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int sp = t.split[i];
    if (sp < 0) return;  // unused slot
    const int4 T = t.climb[i];
    if (T.z >= 0 && merged_into(sp, t.climb[T.z].w >> 1)) return;  // folded into its parent
    const float4 a = ns.s0[i], b = ns.s1[i];
    const float4 q = accuracy ? make_float4(b.y, b.z, b.w, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    emit_record(i, sp, T, accuracy, theta, G, box_ord, seg_of(segs, i), skeys, t, a.x, a.w, b.x, q,
                rec);
}

}  // namespace ssg
