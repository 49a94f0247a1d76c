// Force walks fused with the integration step (sm_103a, FP32 FMA + MUFU rsqrt;
// no tensor cores: the walk is not a dense contraction).
//
// Both walks give one warp a group of up to 32 consecutive bodies in key order
// (the reference's warp, kernels.cu:342-362) and keep the warp's traversal
// state in shared memory.
//
// k_walk_ref   REFERENCE mode.  Node-serial: every lane evaluates the same
//              node; a cell is approximated iff all lanes vote dp <= r
//              (kernels.cu:395-406), bodies always interact, opened cells are
//              pushed on the warp's stack.  The interaction set is the
//              reference's; only the summation order differs.
// k_walk_acc   PLAIN / MIXED modes.  Lanes test up to 32 stack nodes at once
//              against the group's bounding box (accept iff
//              dist(COM, box)^2 > (bmax/theta)^2); accepted cells and the
//              bodies of opened leaves go to shared-memory lists which are
//              flushed 32 entries at a time as dense quadrupole / body-body
//              interactions (every lane computes its body against every entry).
#pragma once

#include "bh_device.cuh"

namespace ssg {

struct WalkIn {
    const float *x, *y, *vx, *vy, *m, *xlo, *ylo;
    const int* id;
};
struct WalkOut {
    float *x, *y, *vx, *vy, *m, *xlo, *ylo;
    int* id;
    float *ax, *ay;
};

struct Groups {
    int ngroups;
    const int* gseg_off;  // [nseg+1] first group of each system (nullptr when nseg == 1)
};

__device__ __forceinline__ void group_range(const Segs& segs, const Groups& gr, int g, int* lo,
                                            int* hi, int* gstart) {
    int s = 0;
    if (segs.nseg > 1) {
        int a = 0, b = segs.nseg;  // find s with gseg_off[s] <= g < gseg_off[s+1]
        while (b - a > 1) {
            int mid = (a + b) >> 1;
            if (__ldg(gr.gseg_off + mid) <= g)
                a = mid;
            else
                b = mid;
        }
        s = a;
    }
    *lo = segs.off[s];
    *hi = segs.off[s + 1];
    int g0 = segs.nseg > 1 ? __ldg(gr.gseg_off + s) : 0;
    *gstart = *lo + 32 * (g - g0);
}

// ------------------------------------------------------------------ REFERENCE walk

__device__ __forceinline__ float ref_r(float cx, float cy, float px, float py, float eps2, float* dx,
                                       float* dy) {
    *dx = __fsub_rn(cx, px);  // kernels.cu:403-405, no contraction
    *dy = __fsub_rn(cy, py);
    return __fadd_rn(__fadd_rn(__fmul_rn(*dx, *dx), __fmul_rn(*dy, *dy)), eps2);
}

template <int WARPS, int STACK>
__global__ void __launch_bounds__(WARPS * 32) k_walk_ref(Segs segs, Groups gr, WalkIn in,
                                                         const float4* __restrict__ recA,
                                                         const int4* __restrict__ recC, float eps2,
                                                         float dt, float ddt, WalkOut out,
                                                         int* __restrict__ status,
                                                         unsigned long long* __restrict__ inter_total) {
    __shared__ int s_stack[WARPS][STACK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int* stack = s_stack[warp];
    unsigned long long my_inter = 0;
    for (int g = blockIdx.x * WARPS + warp; g < gr.ngroups; g += gridDim.x * WARPS) {
        int lo, hi, gstart;
        group_range(segs, gr, g, &lo, &hi, &gstart);
        const int j = gstart + lane;
        const bool valid = j < hi;
        const int cnt = min(32, hi - gstart);
        const float px = valid ? in.x[j] : 0.0f, py = valid ? in.y[j] : 0.0f;
        float ax = 0.0f, ay = 0.0f;
        long long inter = 0;
        bool overflow = false;
        if (hi - lo >= 2) {
            int top = 0;
            {
                float4 A = recA[lo];  // the system's root
                float dx, dy;
                float r = ref_r(A.x, A.y, px, py, eps2, &dx, &dy);
                if (__all_sync(kFull, !valid || A.w <= r)) {
                    float ri = rsqrtf(r);
                    float f = A.z * ri * ri * ri;
                    ax = fmaf(f, dx, ax);
                    ay = fmaf(f, dy, ay);
                    inter += cnt;
                } else {
                    if (lane == 0) stack[0] = lo;
                    top = 1;
                }
            }
            while (top > 0 && !overflow) {
                __syncwarp();
                const int node = stack[--top];
                const int4 C = recC[node];
                const int cs[4] = {C.x, C.y, C.z, C.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = cs[q];
                    if (c == kNoChild) continue;
                    float cx, cy, cm, crit;
                    if (c < 0) {
                        cx = in.x[~c];
                        cy = in.y[~c];
                        cm = in.m[~c];
                        crit = 0.0f;
                    } else {
                        float4 A = recA[c];
                        cx = A.x;
                        cy = A.y;
                        cm = A.z;
                        crit = A.w;
                    }
                    float dx, dy;
                    float r = ref_r(cx, cy, px, py, eps2, &dx, &dy);
                    bool accept = (c < 0) || __all_sync(kFull, !valid || crit <= r);
                    if (accept) {
                        float ri = rsqrtf(r);  // kernels.cu:407-411
                        float f = cm * ri * ri * ri;
                        ax = fmaf(f, dx, ax);
                        ay = fmaf(f, dy, ay);
                        inter += cnt;
                    } else if (top < STACK) {
                        __syncwarp();
                        if (lane == 0) stack[top] = c;
                        ++top;
                    } else {
                        overflow = true;
                    }
                }
            }
        }
        if (overflow && lane == 0) atomicOr(status, ST_STACK);
        my_inter += (unsigned long long)inter;
        if (valid) {
            // kernels.cu:529-533: v += dt*a; x += d*dt*v
            float vx = __fadd_rn(in.vx[j], __fmul_rn(dt, ax));
            float vy = __fadd_rn(in.vy[j], __fmul_rn(dt, ay));
            out.x[j] = __fadd_rn(px, __fmul_rn(ddt, vx));
            out.y[j] = __fadd_rn(py, __fmul_rn(ddt, vy));
            out.vx[j] = vx;
            out.vy[j] = vy;
            out.m[j] = in.m[j];
            out.id[j] = in.id[j];
            out.ax[j] = ax;
            out.ay[j] = ay;
        }
    }
    if (lane == 0 && my_inter) atomicAdd(inter_total, my_inter);
}

// ------------------------------------------------------------------ accuracy walk

__device__ __forceinline__ int warp_excl_scan(int v, int* total) {
    const int lane = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += t;
    }
    *total = __shfl_sync(kFull, x, 31);
    return x - v;
}

// a += m * d * u^-3/2 (softened body-body / monopole term)
__device__ __forceinline__ void p2p(float bx, float by, float bm, float px, float py, float eps2,
                                    float& ax, float& ay) {
    float dx = bx - px, dy = by - py;
    float u = fmaf(dx, dx, fmaf(dy, dy, eps2));
    float ri = u > 0.0f ? rsqrtf(u) : 0.0f;
    float f = bm * ri * ri * ri;
    ax = fmaf(f, dx, ax);
    ay = fmaf(f, dy, ay);
}

// Quadrupole term about the centre of mass c, d = c - p, u = |d|^2 + eps2,
// T = 3S (S = second moments about c), h = 1.5 tr S:
//   a += u^-3/2 [ (M + u^-1 (2.5 u^-1 d.T.d - h)) d - u^-1 T d ]
// which is -(grad of the softened potential expanded to second order).
__device__ __forceinline__ void p2m(float4 A, float4 B, float px, float py, float eps2, float& ax,
                                    float& ay) {
    float dx = A.x - px, dy = A.y - py;
    float u = fmaf(dx, dx, fmaf(dy, dy, eps2));
    float ri = rsqrtf(u);
    float r2 = ri * ri;
    float r3 = ri * r2;
    float tdx = fmaf(B.x, dx, B.y * dy);
    float tdy = fmaf(B.y, dx, B.z * dy);
    float dtd = fmaf(dx, tdx, dy * tdy);
    float t = fmaf(2.5f * dtd, r2, -B.w);
    float coef = fmaf(r2, t, A.z);
    float fx = fmaf(coef, dx, -r2 * tdx);
    float fy = fmaf(coef, dy, -r2 * tdy);
    ax = fmaf(r3, fx, ax);
    ay = fmaf(r3, fy, ay);
}

template <int WARPS, int STACK, int BUCKET>
struct AccSmem {
    static constexpr int kBodyCap = 32 + 32 * (BUCKET > 4 ? BUCKET : 4);
    int stack[WARPS][STACK];
    int clist[WARPS][64];
    int blist[WARPS][kBodyCap];
    float4 cA[WARPS][32];
    float4 cB[WARPS][32];
    float4 bP[WARPS][32];
};

template <int WARPS, int STACK, int BUCKET, bool MIXED>
__global__ void __launch_bounds__(WARPS * 32) k_walk_acc(Segs segs, Groups gr, WalkIn in,
                                                         const float4* __restrict__ recA,
                                                         const float4* __restrict__ recB,
                                                         const int4* __restrict__ recC,
                                                         const int2* __restrict__ recD, float eps2,
                                                         float G, float dt, float ddt, WalkOut out,
                                                         int* __restrict__ status,
                                                         unsigned long long* __restrict__ inter_total) {
    using Sm = AccSmem<WARPS, STACK, BUCKET>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Sm& sm = *reinterpret_cast<Sm*>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = lanemask_lt();
    int* stack = sm.stack[warp];
    int* clist = sm.clist[warp];
    int* blist = sm.blist[warp];
    float4* cA = sm.cA[warp];
    float4* cB = sm.cB[warp];
    float4* bP = sm.bP[warp];
    unsigned long long my_inter = 0;

    for (int g = blockIdx.x * WARPS + warp; g < gr.ngroups; g += gridDim.x * WARPS) {
        int lo, hi, gstart;
        group_range(segs, gr, g, &lo, &hi, &gstart);
        const int j = gstart + lane;
        const bool valid = j < hi;
        const int cnt = min(32, hi - gstart);
        const int jj = valid ? j : gstart;  // invalid lanes mirror lane 0's body
        const float px = in.x[jj], py = in.y[jj];
        float gx0 = px, gx1 = px, gy0 = py, gy1 = py;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            gx0 = fminf(gx0, __shfl_xor_sync(kFull, gx0, o));
            gx1 = fmaxf(gx1, __shfl_xor_sync(kFull, gx1, o));
            gy0 = fminf(gy0, __shfl_xor_sync(kFull, gy0, o));
            gy1 = fmaxf(gy1, __shfl_xor_sync(kFull, gy1, o));
        }
        float ax = 0.0f, ay = 0.0f;     // running sums
        float cax = 0.0f, cay = 0.0f;   // Kahan compensation (MIXED)
        long long entries = 0;
        bool overflow = false;
        int top = 0, ccnt = 0, bcnt = 0;
        if (hi - lo >= 2) {
            if (lane == 0) stack[0] = lo;
            top = 1;
        }
        // flush helpers ---------------------------------------------------
        auto add_batch = [&](float bx, float by) {
            if (MIXED) {
                float yx = bx - cax, tx = ax + yx;
                cax = (tx - ax) - yx;
                ax = tx;
                float yy = by - cay, ty = ay + yy;
                cay = (ty - ay) - yy;
                ay = ty;
            } else {
                ax += bx;
                ay += by;
            }
        };
        auto flush_cells = [&](int k) {  // the last k entries of clist
            __syncwarp();
            if (lane < k) {
                int node = clist[ccnt - k + lane];
                cA[lane] = recA[node];
                cB[lane] = recB[node];
            }
            __syncwarp();
            float bx = 0.0f, by = 0.0f;
            for (int e = 0; e < k; ++e) p2m(cA[e], cB[e], px, py, eps2, bx, by);
            add_batch(bx, by);
            ccnt -= k;
            entries += k;
        };
        auto flush_bodies = [&](int k) {
            __syncwarp();
            if (lane < k) {
                int b = blist[bcnt - k + lane];
                bP[lane] = make_float4(in.x[b], in.y[b], in.m[b], 0.0f);
            }
            __syncwarp();
            float bx = 0.0f, by = 0.0f;
            for (int e = 0; e < k; ++e) {
                float4 P = bP[e];
                p2p(P.x, P.y, P.z, px, py, eps2, bx, by);
            }
            add_batch(bx, by);
            bcnt -= k;
            entries += k;
        };
        // traversal -------------------------------------------------------
        while (top > 0) {
            int k = min(32, top);
            int room = (STACK - top) / 3;  // pop k, push <= 4k: keep top+3k <= STACK
            if (room < k) k = max(room, 0);
            if (k == 0) {
                overflow = true;
                break;
            }
            __syncwarp();
            const int node = lane < k ? stack[top - 1 - lane] : -1;
            top -= k;
            int cat = -1;  // 0 accept cell, 1 leaf bodies, 2 open
            float4 A;
            int2 D = make_int2(0, 0);
            if (node >= 0) {
                A = recA[node];
                D = recD[node];
                float ddx = fmaxf(fmaxf(gx0 - A.x, A.x - gx1), 0.0f);
                float ddy = fmaxf(fmaxf(gy0 - A.y, A.y - gy1), 0.0f);
                float d2 = fmaf(ddx, ddx, ddy * ddy);
                cat = d2 > A.w ? 0 : (D.y <= BUCKET ? 1 : 2);
            }
            // accepted cells
            unsigned mc = __ballot_sync(kFull, cat == 0);
            if (cat == 0) clist[ccnt + __popc(mc & lt)] = node;
            ccnt += __popc(mc);
            // opened nodes: children
            int4 C = make_int4(kNoChild, kNoChild, kNoChild, kNoChild);
            if (cat == 2) C = recC[node];
            const int cs[4] = {C.x, C.y, C.z, C.w};
            int nb = cat == 1 ? D.y : 0, nn = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                nb += (cs[q] != kNoChild && cs[q] < 0);
                nn += (cs[q] >= 0);
            }
            int btot, ntot;
            int boff = warp_excl_scan(nb, &btot);
            int noff = warp_excl_scan(nn, &ntot);
            int* bw = blist + bcnt + boff;
            __syncwarp();  // every lane has read its stack slot before children overwrite it
            if (cat == 1) {
                for (int e = 0; e < D.y; ++e) bw[e] = D.x + e;
            } else if (cat == 2) {
                int* nw = stack + top + noff;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (cs[q] == kNoChild) continue;
                    if (cs[q] < 0)
                        *bw++ = ~cs[q];
                    else
                        *nw++ = cs[q];
                }
            }
            bcnt += btot;
            top += ntot;
            __syncwarp();
            while (ccnt >= 32) flush_cells(32);
            while (bcnt >= 32) flush_bodies(32);
        }
        if (ccnt > 0) flush_cells(ccnt);
        if (bcnt > 0) flush_bodies(bcnt);
        if (overflow && lane == 0) atomicOr(status, ST_STACK);
        my_inter += (unsigned long long)(entries * cnt);
        if (valid) {
            float gax = G * (MIXED ? ax - cax : ax);
            float gay = G * (MIXED ? ay - cay : ay);
            float vx = fmaf(dt, gax, in.vx[j]);
            float vy = fmaf(dt, gay, in.vy[j]);
            if (MIXED) {
                // x_hi + x_lo += d*dt*v with an error-free sum (TwoSum), renormalised
                float inc = ddt * vx, hx = px, s = hx + inc, bb = s - hx;
                float e = (hx - (s - bb)) + (inc - bb);
                float lo2 = in.xlo[j] + e, h2 = s + lo2;
                out.x[j] = h2;
                out.xlo[j] = lo2 - (h2 - s);
                inc = ddt * vy;
                hx = py;
                s = hx + inc;
                bb = s - hx;
                e = (hx - (s - bb)) + (inc - bb);
                lo2 = in.ylo[j] + e;
                h2 = s + lo2;
                out.y[j] = h2;
                out.ylo[j] = lo2 - (h2 - s);
            } else {
                out.x[j] = fmaf(ddt, vx, px);
                out.y[j] = fmaf(ddt, vy, py);
            }
            out.vx[j] = vx;
            out.vy[j] = vy;
            out.m[j] = in.m[j];
            out.id[j] = in.id[j];
            out.ax[j] = gax;
            out.ay[j] = gay;
        }
    }
    if (lane == 0 && my_inter) atomicAdd(inter_total, my_inter);
}

}  // namespace ssg
